// Launch helpers shared by the projection translation units: geometry
// checks, launch-shape selection (z-block, lanes per bin, angle groups) and
// the templated kernel launches.
#pragma once

#include "gr_internal.cuh"
#include "projection_fast.cuh"

namespace gr {
namespace launch {

// A quarter-turn map must send the N x N grid onto itself: a signed
// permutation of (x, y) whose offsets keep two opposite corners inside.
inline bool valid_quarter_map(const int* m, int N) {
  auto unit = [](int v) { return v == 1 || v == -1; };
  const bool perm = (unit(m[0]) && m[1] == 0 && m[2] == 0 && unit(m[3])) ||
                    (m[0] == 0 && unit(m[1]) && unit(m[2]) && m[3] == 0);
  if (!perm) return false;
  const int64_t last = N - 1;
  const int64_t x0 = m[4], y0 = m[5];
  const int64_t x1 = m[4] + (int64_t)(m[0] + m[1]) * last;
  const int64_t y1 = m[5] + (int64_t)(m[2] + m[3]) * last;
  auto in = [&](int64_t v) { return v >= 0 && v <= last; };
  return in(x0) && in(y0) && in(x1) && in(y1);
}

inline int check_geometry(const gr_geometry* g) {
  if (g == nullptr || g->ofs == nullptr) return GR_ERR_ARG;
  if (g->kind != GR_RADON && g->kind != GR_FANBEAM) return GR_ERR_ARG;
  if (!valid_dtype(g->dtype)) return GR_ERR_ARG;
  if (g->kind == GR_FANBEAM && g->sdpd == nullptr) return GR_ERR_ARG;
  if (g->Nx <= 0 || g->Ny <= 0 || g->Ns <= 0 || g->Na <= 0) return GR_ERR_SHAPE;
  if (g->sym != 0) {
    // 4: fan-beam quarter-turn orbits; 2: parallel-beam half-circle orbits
    const bool kind_ok = (g->sym == 4 && g->kind == GR_FANBEAM) ||
                         (g->sym == 2 && g->kind == GR_RADON && g->Na % 2 == 0);
    if (!kind_ok || g->Nx != g->Ny) return GR_ERR_ARG;
    for (int m = 0; m < 3; ++m)
      if (!valid_quarter_map(g->sym_map[m], g->Nx)) return GR_ERR_ARG;
  }
  if (g->mirror != 0 && g->sym == 4) {
    // a reflection (determinant -1) of a quarter-turn symmetric fan geometry
    // (without the quarter-turn maps the mirror is not used)
    const int* mm = g->mirror_map;
    if (g->mirror_pair < 0 || g->mirror_pair >= g->Na || !valid_quarter_map(mm, g->Nx) ||
        mm[0] * mm[3] - mm[1] * mm[2] != -1)
      return GR_ERR_ARG;
  }
  if (g->Na > 65535) return GR_ERR_TOO_BIG;
  return GR_OK;
}

inline Dims dims_of(const gr_geometry* g, int Nz) {
  Dims d;
  d.Nx = g->Nx;
  d.Ny = g->Ny;
  d.Nz = Nz;
  d.Ns = g->Ns;
  d.Na = g->Na;
  return d;
}

template <typename T>
inline RadonGeo<T> radon_geo(const double* geo) {
  RadonGeo<T> r;
  r.delta_x = (float)geo[0];
  r.delta_xi = (float)geo[1];
  return r;
}

template <typename T>
inline FanGeo<T> fan_geo(const double* geo) {
  FanGeo<T> f;
  f.R = (T)geo[0];
  f.RE = (T)geo[1];
  f.delta_xi = (T)geo[2];
  f.midx = (T)geo[3];
  f.midy = (T)geo[4];
  f.mid_det = (T)geo[5];
  f.delta_x = (T)geo[10];
  return f;
}

inline int zblock(int Nz) { return Nz == 1 ? 1 : 4; }

// C-ordered stacks whose slice count is a multiple of 4 on a 16-byte aligned
// base keep every 4-slice group of a pixel in one aligned 16-byte word.
template <typename T>
inline bool aligned_groups_of_4(const T* base, int Nz) {
  return Nz % 4 == 0 && (reinterpret_cast<uintptr_t>(base) & 15u) == 0;
}

// Resident threads the device holds (SM count x 2048), cached per device.
inline int64_t device_capacity() {
  static int64_t cap[64] = {0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152 * 2048;
  if (cap[dev] == 0) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
      sms = 152;
    cap[dev] = (int64_t)sms * 2048;
  }
  return cap[dev];
}

inline bool valid_split(int v) { return v == 1 || v == 2 || v == 4 || v == 8; }

// Lanes per detector bin: enough that the launch holds about two waves of
// resident threads (small problems), 1 for large ones.
// float64 launches use 1 or 4 only (fewer instantiations; float64 is the
// parity path, not the throughput path).
inline int clamp_split(const gr_geometry* g, int sp) {
  return g->dtype == GR_F64 ? (sp >= 4 ? 4 : 1) : sp;
}

inline int fwd_split(const gr_geometry* g, int Nz) {
  if (valid_split(g->fwd_split)) return clamp_split(g, g->fwd_split);
  // float32 forward: 8 lanes per group of bins measured fastest on GB300 at
  // every size tried (256^2 .. 1200^2, single slices and 16-slice stacks).
  if (g->dtype == GR_F32) return 8;
  const int group = g->dtype == GR_F32 ? fast::kRayGroup : 1;
  const int64_t work = (int64_t)g->Ns * g->Na * ((Nz + zblock(Nz) - 1) / zblock(Nz)) / group;
  const int64_t want = 2 * device_capacity();
  for (int sp = 1; sp < 8; sp <<= 1)
    if (work * sp >= want) return clamp_split(g, sp);
  return clamp_split(g, 8);
}

inline bool use_quarter_bwd(const gr_geometry* g, int Nz);
inline bool use_radon_orbit_bwd(const gr_geometry* g, int Nz);

inline int bwd_split(const gr_geometry* g, int Nz) {
  if (valid_split(g->bwd_split)) return clamp_split(g, g->bwd_split);
  // orbit backprojection: 8 angle groups measured fastest or within 1% of it
  // from 128^2 to 2048^2 (360 to 1440 angles)
  if (use_quarter_bwd(g, Nz) || use_radon_orbit_bwd(g, Nz)) return 8;
  if (g->dtype == GR_F32) {
    // float32 tiles stage detector windows per block, so angles are split
    // over thread rows only when the image alone cannot fill 40% of the
    // GPU's thread slots (single slices: 2 pixels per thread without a split)
    const int64_t pix = (int64_t)g->Nx * g->Ny * ((Nz + zblock(Nz) - 1) / zblock(Nz));
    const int64_t want = device_capacity() * 2 / 5;
    if ((Nz == 1 ? pix / 2 : pix) >= want) return 1;
    for (int sp = 2; sp < 8; sp <<= 1)
      if (pix * sp >= want) return sp;
    return 8;
  }
  const int64_t work = (int64_t)g->Nx * g->Ny * ((Nz + zblock(Nz) - 1) / zblock(Nz));
  const int64_t want = 2 * device_capacity();
  for (int sp = 1; sp < 8; sp <<= 1)
    if (work * sp >= want) return clamp_split(g, sp);
  return clamp_split(g, 8);
}

inline int64_t pixel_angles(const gr_geometry* g) {
  return (int64_t)g->Nx * g->Ny * g->Na;
}

// Stacks take the orbit kernels (one slice per block) from this many
// pixel-angles per slice; smaller slices keep the 4-slice per-angle kernels,
// which share each pixel-angle's geometry over 4 slices instead (measured,
// Gpixel-angle/s forward / back: 512^2 x 360 orbit 922 / 1824, per-angle
// 1033 / 1807; 1024^2 x 720 orbit 1318 / 2087, per-angle 1031 / 1868).
constexpr int64_t kQuarterStackMin = 256ll << 20;

// float32 fan beam with a quarter-turn symmetric angle set: one block row per
// base angle, four angles per lane group, one slice per block.  Offsets within
// a slice are 32-bit, so a slice holds fewer than 2^31 pixels.
inline bool use_quarter(const gr_geometry* g, int Nz) {
  return g->sym == 4 && g->dtype == GR_F32 && g->kind == GR_FANBEAM && Nz >= 1 &&
         Nz <= 65535 && (Nz == 1 || pixel_angles(g) >= kQuarterStackMin) &&
         g->Na % 4 == 0 && g->Nx == g->Ny && (int64_t)g->Nx * g->Ny <= INT32_MAX;
}

// Backprojection over quarter-turn pixel orbits: the first map is a turn by
// a quarter about the image centre and the others are its powers, the side
// is even (the quadrant x, y < N/2 then holds one pixel of every orbit),
// and a slice of the sinogram has fewer than 2^31 values (32-bit offsets).
// The three maps are the powers of one quarter turn about the image centre.
__host__ __device__ inline bool maps_cyclic_of(const int (*sym_map)[6]) {
  const int* m1 = sym_map[0];
  if (m1[0] != 0 || m1[3] != 0 || m1[1] * m1[2] != -1) return false;
  // apply the first map after an affine map (axx, axy, ayx, ayy, cx, cy)
  auto after_m1 = [&](const int* f, int* out) {
    out[0] = m1[0] * f[0] + m1[1] * f[2];
    out[1] = m1[0] * f[1] + m1[1] * f[3];
    out[2] = m1[2] * f[0] + m1[3] * f[2];
    out[3] = m1[2] * f[1] + m1[3] * f[3];
    out[4] = m1[4] + m1[0] * f[4] + m1[1] * f[5];
    out[5] = m1[5] + m1[2] * f[4] + m1[3] * f[5];
  };
  int m2[6], m3[6], m4[6];
  after_m1(m1, m2);
  after_m1(m2, m3);
  after_m1(m3, m4);
  const int id[6] = {1, 0, 0, 1, 0, 0};
  for (int k = 0; k < 6; ++k)
    if (m2[k] != sym_map[1][k] || m3[k] != sym_map[2][k] || m4[k] != id[k]) return false;
  return true;
}

inline bool maps_cyclic(const gr_geometry* g) { return maps_cyclic_of(g->sym_map); }

inline bool use_quarter_bwd(const gr_geometry* g, int Nz) {
  if (!use_quarter(g, Nz) || g->Nx % 2 != 0) return false;
  if ((int64_t)g->Ns * g->Na > INT32_MAX) return false;
  return maps_cyclic(g);
}

// Registers of the fan-beam orbit backprojection (fan_bwd_orbit_rows).  With
// 8 angle groups and slices of at most 512^2 pixels it runs 5 blocks per SM
// at 48 registers instead of 4 at 64 (8-20 bytes of spill): 512^2 x 360
// backprojection 1618 -> 1676-1704 Gpixel-angle/s, CG-50 112.2 -> 115.0
// reconstructions/s.  The TV epilogues keep 4 blocks: at 48 registers their
// F-ordered form spills 40 bytes, and the 2048^2 x 64 TV iteration took
// 349.8 instead of 314.6 ms.  Larger slices keep 4 blocks as well (that
// iteration is the only measurement above 512^2).
template <class Epi>
struct tv_epilogue : std::false_type {};
template <typename T, int O>
struct tv_epilogue<BwdTVPrimal<T, O>> : std::true_type {};
template <typename T, int O>
struct tv_epilogue<BwdTVAdjoint<T, O>> : std::true_type {};
template <class Epi, int G>
constexpr int kDenseFanBwdBlocks = (G == 8 && !tv_epilogue<Epi>::value) ? 5 : 1;
constexpr int64_t kDenseFanBwdMaxPixels = 512 * 512;
template <class Epi, int G>
inline bool dense_fan_bwd(const gr_geometry* g) {
  return kDenseFanBwdBlocks<Epi, G> > 1 && (int64_t)g->Nx * g->Ny <= kDenseFanBwdMaxPixels;
}

// Scratch of the orbit kernels: the forward's orbit pixels (one float4 per
// pixel) and the backprojection's interleaved rows (one float4 per base
// angle and bin); one call uses one of them, so the larger one is needed.
// Below these sizes (pixel-angles per projection) the extra launch costs more
// than the copy saves (measured, fan beam with 360 angles, us per forward at
// the best split, copy with the mirror against direct gathers: 128^2 26.6 /
// 24.7, 192^2 31.9 / 31.4, 256^2 38.6 / 42.5, 384^2 54.9 / 77.0; the
// backprojection's copy loses at 128^2 and wins at 256^2).
constexpr int64_t kQuarterFwdCopyMin = 16ll << 20;
constexpr int64_t kQuarterBwdCopyMin = 12ll << 20;
// slices copied per launch pair at most (a stack runs in chunks of as many
// slices as the scratch holds)
constexpr int kQuarterCopySlices = 8;

// Bytes of one slice's copy (0: no copy for this geometry).
inline size_t quarter_fwd_bytes(const gr_geometry* g, int Nz) {
  if (!use_quarter(g, Nz) || pixel_angles(g) < kQuarterFwdCopyMin) return 0;
  return (size_t)g->Nx * (size_t)g->Ny * sizeof(float4);
}

inline size_t quarter_bwd_bytes(const gr_geometry* g, int Nz) {
  if (!use_quarter_bwd(g, Nz) || pixel_angles(g) < kQuarterBwdCopyMin) return 0;
  return (size_t)(g->Na / 4) * (size_t)(g->Ns + fast::kOrbitRowPad + fast::kOrbitRec) *
         sizeof(float4);
}

// Stacks take the parallel-beam orbit forward slice by slice from this many
// pixel-angles per slice, and never the orbit backprojection: the 4-slice
// per-angle kernels share each pixel-angle's geometry over 4 slices instead
// (measured with a one-slice scratch, Gpixel-angle/s forward / back:
// 256^2 x 180 x 16 orbit 615 / 698, per-angle 829 / 1593; 512^2 x 360 x 16
// orbit 1448 / 1749, per-angle 919 / 2020; 1024^2 x 720 x 4 orbit 2004 /
// 2021, per-angle 901 / 2055).
constexpr int64_t kRadonOrbitStackMin = 32ll << 20;

// Parallel beam, float32 with the half-circle orbit maps (sym = 2): the orbit
// kernels read copies of the image (the forward, any side) and of the
// sinogram (the backprojection, even sides), so each runs only when the
// caller's scratch holds its copy of a slice; otherwise the per-angle kernels
// run.
inline bool use_radon_orbit(const gr_geometry* g, int Nz) {
  return g->sym == 2 && g->dtype == GR_F32 && g->kind == GR_RADON && Nz >= 1 &&
         Nz <= 65535 && g->Na % 2 == 0 && g->Nx == g->Ny &&
         (int64_t)g->Nx * g->Ny <= INT32_MAX &&
         (int64_t)(g->Ns + fast::kOrbitRowPad) * (g->Na / 2) <= INT32_MAX;
}

// From this many pixel-angles the orbit forward reads the orbit copy (one
// 16-byte load per candidate) instead of gathering the four orbit members
// from the image, whose turned members walk across rows (measured, us per
// forward with / without the copy at fwd_split 8: 128^2 x 90 22.8 / 19.3,
// 256^2 x 180 28.6 / 30.0, 512^2 x 360 73.6 / 132.7, 2048^2 x 1440 2653 /
// 7106).
constexpr int64_t kRadonFwdCopyMin = 4ll << 20;

inline size_t radon_orbit_fwd_bytes(const gr_geometry* g, int Nz) {
  if (!use_radon_orbit(g, Nz) || pixel_angles(g) < kRadonFwdCopyMin ||
      (Nz > 1 && pixel_angles(g) < kRadonOrbitStackMin))
    return 0;
  return (size_t)g->Nx * (size_t)g->Ny * sizeof(float4);
}


// The orbit backprojection reads the row copy from this many pixel-angles
// and gathers from the sinogram below (measured, us per backprojection with
// / without the copy at 8 angle groups: 128^2 x 90 22.4 / 19.2, 256^2 x 180
// 23.6 / 24.0, 512^2 x 360 66.6 / 79.7, 1024^2 x 720 350 / 503; the
// per-angle kernel 21.8, 34.6, 100.6, 583).
constexpr int64_t kRadonBwdCopyMin = 4ll << 20;

inline size_t radon_orbit_bwd_bytes(const gr_geometry* g, int Nz) {
  if (!use_radon_orbit(g, Nz) || Nz != 1 || g->Nx % 2 != 0 || pixel_angles(g) < kRadonBwdCopyMin)
    return 0;
  return (size_t)(g->Na / 2) * (size_t)(g->Ns + fast::kOrbitRowPad) * sizeof(float4);
}

inline size_t orbit_work_bytes(const gr_geometry* g, int Nz) {
  if (g->kind == GR_RADON) {
    const size_t f = radon_orbit_fwd_bytes(g, Nz), b = radon_orbit_bwd_bytes(g, Nz);
    const int slices = Nz < kQuarterCopySlices ? Nz : kQuarterCopySlices;
    return (f > b ? f : b) * (size_t)(slices > 0 ? slices : 0);
  }
  const size_t f = quarter_fwd_bytes(g, Nz), b = quarter_bwd_bytes(g, Nz);
  const int slices = Nz < kQuarterCopySlices ? Nz : kQuarterCopySlices;
  return (f > b ? f : b) * (size_t)(slices > 0 ? slices : 0);
}

// Slices per launch pair that the caller's scratch holds (16-byte aligned)
// for copies of `per_slice` bytes; 0: no copy.
inline int work_slices(const gr_geometry* g, size_t per_slice, int Nz) {
  if (per_slice == 0 || g->work == nullptr || (reinterpret_cast<uintptr_t>(g->work) & 15u) != 0)
    return 0;
  const size_t n = g->work_bytes / per_slice;
  return n >= (size_t)Nz ? Nz : (int)n;
}


// The orbit forward: single slices (without the copy, gathering the orbit
// members: still ahead of the per-angle kernel, 512^2 x 360 133 vs 160 us),
// and stacks of large slices with their copies (gathering, 512^2 x 360 x 16
// ran 766 Gpixel-angle/s against the 4-slice per-angle kernel's 919).
inline bool use_radon_orbit_fwd(const gr_geometry* g, int Nz) {
  if (!use_radon_orbit(g, Nz)) return false;
  return Nz == 1 || work_slices(g, radon_orbit_fwd_bytes(g, Nz), Nz) > 0;
}

// The orbit backprojection: single slices of even side, from the row copy
// when the scratch holds it, else gathering from the sinogram.
inline bool use_radon_orbit_bwd(const gr_geometry* g, int Nz) {
  return use_radon_orbit(g, Nz) && Nz == 1 && g->Nx % 2 == 0;
}

// The fan-beam orbit forward with the mirror: quarter-turn orbits with cyclic
// maps, the mirror set, reading the orbit copy.
inline bool use_fan_mirror_fwd(const gr_geometry* g, int Nz) {
  return use_quarter(g, Nz) && g->mirror != 0 && maps_cyclic(g) &&
         work_slices(g, quarter_fwd_bytes(g, Nz), Nz) > 0;
}

inline dim3 fwd_grid(const gr_geometry* g, int Nz, int split) {
  const int ZB = zblock(Nz);
  const int group = g->dtype == GR_F32 ? fast::kRayGroup : 1;  // bins per lane group
  const int per_block = (32 / split) * (kFwdBlock / 32) * group;
  if (use_quarter(g, Nz)) {
    // one slice per block; 2 * split lanes per group, or 4 * split over the
    // bins s < ceil(Ns/2) with the mirror
    const bool mir = use_fan_mirror_fwd(g, Nz);
    const int apb = fast::kQuarterAnglesPerBlock;
    const int qb = (32 / ((mir ? 4 : 2) * split)) * (kFwdBlock / 32 / apb) * group;
    const int bins = mir ? (g->Ns + 1) / 2 : g->Ns;
    return dim3((bins + qb - 1) / qb, (g->Na / 4 + apb - 1) / apb, Nz);
  }
  if (use_radon_orbit_fwd(g, Nz)) {  // bins s < ceil(Ns/2), base angles k < Na/2
    const int apb = fast::kQuarterAnglesPerBlock;
    const int qb = (32 / (4 * split)) * (kFwdBlock / 32 / apb) * group;  // 4 * split lanes
    const int H = (int)((g->Ns + 1) / 2);
    return dim3((H + qb - 1) / qb, (g->Na / 2 + apb - 1) / apb, Nz);  // one launch per slice
  }
  if (g->dtype == GR_F32 && g->kind == GR_RADON && Nz == 1) {  // 2 * split lanes per group
    const int rb = (32 / (2 * split)) * (kFwdBlock / 32) * group;
    return dim3((g->Ns + rb - 1) / rb, g->Na, 1);
  }
  return dim3((g->Ns + per_block - 1) / per_block, g->Na, (Nz + ZB - 1) / ZB);
}

__host__ __device__ inline fast::QuarterMaps quarter_maps_of(const int (*sym_map)[6]) {
  fast::QuarterMaps q;
  q.mxx = q.mxy = q.myx = q.myy = q.mcx = q.mcy = 0;
  q.mirror_pair = -1;
  for (int m = 0; m < 3; ++m) {
    q.axx[m] = sym_map[m][0];
    q.axy[m] = sym_map[m][1];
    q.ayx[m] = sym_map[m][2];
    q.ayy[m] = sym_map[m][3];
    q.cx[m] = sym_map[m][4];
    q.cy[m] = sym_map[m][5];
  }
  q.cyclic = maps_cyclic_of(sym_map) ? 1 : 0;
  return q;
}

inline fast::QuarterMaps quarter_maps(const gr_geometry* g) {
  fast::QuarterMaps q = quarter_maps_of(g->sym_map);
  if (g->mirror != 0) {
    const int* mm = g->mirror_map;
    q.mxx = mm[0];
    q.mxy = mm[1];
    q.myx = mm[2];
    q.myy = mm[3];
    q.mcx = mm[4];
    q.mcy = mm[5];
    q.mirror_pair = g->mirror_pair;
  }
  return q;
}

inline dim3 bwd_grid(const gr_geometry* g, int Nz, int io, int split) {
  if (use_quarter_bwd(g, Nz) || use_radon_orbit_bwd(g, Nz)) {  // 32 x (8 / split) quadrant tiles
    const int half = g->Nx / 2, rows = kBwdTileSlow / split;
    return dim3((half + kBwdTileFast - 1) / kBwdTileFast, (half + rows - 1) / rows, Nz);
  }
  const int ZB = zblock(Nz);
  const int fast = io == ORDER_F ? g->Nx : g->Ny;
  const int slow = io == ORDER_F ? g->Ny : g->Nx;
  const int rows = kBwdTileSlow / split;  // slow extent of a pixel tile
  return dim3((fast + kBwdTileFast - 1) / kBwdTileFast, (slow + rows - 1) / rows, (Nz + ZB - 1) / ZB);
}

template <typename T, int SO, int IO, int ZB, int SPLIT, class Epi>
int launch_fwd_zb(const gr_geometry* g, const T* img, int Nz, Epi epi, double* partials,
                  const int* skip, cudaStream_t st) {
  Dims d = dims_of(g, Nz);
  d.vec4 = aligned_groups_of_4(img, Nz);
  const dim3 grid = fwd_grid(g, Nz, SPLIT);
  if constexpr (std::is_same<T, float>::value) {
    if (g->kind == GR_RADON) {
      if (use_radon_orbit_fwd(g, Nz)) {
        // half-circle orbits, one launch per slice (each launch's block
        // partials follow the previous slice's); four times the lanes per
        // group: a group's work is shared by four outputs, so the orbit
        // forward has a quarter of the groups (256^2 x 180: 16 lanes 41.6
        // us, 8 lanes 63.4 us, 32 lanes 29.8 us)
        const fast::QuarterMaps qm = quarter_maps(g);
        const float* ofs = static_cast<const float*>(g->ofs);
        const dim3 sgrid(grid.x, grid.y, 1);
        const int64_t per_slice_blocks = (int64_t)grid.x * grid.y;
        int64_t sx, sy, sz;
        img_strides<IO>(d, sx, sy, sz);
        const int chunk = work_slices(g, radon_orbit_fwd_bytes(g, Nz), Nz);
        if (chunk == 0) {
          // no copy: the four orbit members gathered from the image
          for (int64_t z = 0; z < Nz; ++z)
            launch_pdl(fast::radon_fwd_quarter<SO, IO, 4 * SPLIT, false, 1, Epi>, sgrid,
                       dim3(kFwdBlock), st, img + z * sz, nullptr, ofs, radon_geo<float>(g->geo),
                       d, qm, epi, partials ? partials + z * per_slice_blocks : nullptr, skip, z);
          return check_launch();
        }
        // slices in chunks: each pixel's four orbit pixels as one float4,
        // then the forward over the copies
        float4* img4 = static_cast<float4*>(g->work);
        const int64_t slice4 = (int64_t)g->Nx * g->Ny;
        for (int z0 = 0; z0 < Nz; z0 += chunk) {
          const int zc = Nz - z0 < chunk ? Nz - z0 : chunk;
          if constexpr (IO == ORDER_F) {
            constexpr int kTile = fast::kOrbitTile;
            const dim3 tgrid((g->Nx + kTile - 1) / kTile, (g->Ny + kTile - 1) / kTile, zc);
            launch_pdl(fast::orbit_pixels_tiled<IO>, tgrid, dim3(kTile, kTile), st, img, d, qm,
                       img4, (int64_t)z0, skip);
          } else {
            const dim3 pgrid((g->Nx + 255) / 256, g->Ny, zc);
            launch_pdl(fast::orbit_pixels<IO>, pgrid, dim3(256), st, img, d, qm, img4,
                       (int64_t)z0, skip);
          }
          // slices in pairs: a candidate's weights serve both slices' copies
          for (int c = 0; c < zc; c += 2) {
            const int64_t z = z0 + c;
            double* pz = partials ? partials + z * per_slice_blocks : nullptr;
            if (c + 1 < zc)
              launch_pdl(fast::radon_fwd_quarter<SO, IO, 4 * SPLIT, true, 2, Epi>, sgrid,
                         dim3(kFwdBlock), st, img + z * sz, (const float4*)(img4 + c * slice4),
                         ofs, radon_geo<float>(g->geo), d, qm, epi, pz, skip, z);
            else
              launch_pdl(fast::radon_fwd_quarter<SO, IO, 4 * SPLIT, true, 1, Epi>, sgrid,
                         dim3(kFwdBlock), st, img + z * sz, (const float4*)(img4 + c * slice4),
                         ofs, radon_geo<float>(g->geo), d, qm, epi, pz, skip, z);
          }
        }
        return check_launch();
      }
      if constexpr (ZB == 1) {
        // single slices run twice the lanes per bin group (fwd_grid): one
        // Radon slice is too small to fill the GPU with SPLIT lanes
        fast::radon_fwd_fast<SO, IO, 1, 2 * SPLIT, Epi><<<grid, kFwdBlock, 0, st>>>(
            img, static_cast<const float*>(g->ofs), radon_geo<float>(g->geo), d, epi, partials,
            skip);
      } else {
        fast::radon_fwd_fast<SO, IO, ZB, SPLIT, Epi><<<grid, kFwdBlock, 0, st>>>(
            img, static_cast<const float*>(g->ofs), radon_geo<float>(g->geo), d, epi, partials,
            skip);
      }
    } else if (use_quarter(g, Nz)) {
      // the orbit forward runs twice the lanes per bin group: its rows are
      // shared by four angles, so the wider split (and twice the blocks)
      // pays (measured at fwd_split 8: 512^2 x 360 99 -> 89 us, 1024^2 x 720
      // 1427 -> 1585 Gpixel-angle/s, never slower from 128^2 to 2048^2)
      constexpr int kQSplit = 2 * SPLIT;
      // one launch per slice on its base pointers (grid.z of fwd_grid counts
      // the slices; each launch's block partials follow the previous slice's)
      const float* ofs = static_cast<const float*>(g->ofs);
      const float* sdpd = static_cast<const float*>(g->sdpd);
      const fast::QuarterMaps qm = quarter_maps(g);
      const dim3 sgrid(grid.x, grid.y, 1);
      const int64_t per_slice_blocks = (int64_t)grid.x * grid.y;
      int64_t sx, sy, sz;
      img_strides<IO>(d, sx, sy, sz);
      const int chunk = work_slices(g, quarter_fwd_bytes(g, Nz), Nz);
      const bool mirror = use_fan_mirror_fwd(g, Nz);
      if (chunk > 0) {
        // slices in chunks: orbit-pixel copies, then the forward on them
        float4* img4 = static_cast<float4*>(g->work);
        const int64_t slice4 = (int64_t)g->Nx * g->Ny;
        for (int z0 = 0; z0 < Nz; z0 += chunk) {
          const int zc = Nz - z0 < chunk ? Nz - z0 : chunk;
          if constexpr (IO == ORDER_F) {
            constexpr int kTile = fast::kOrbitTile;
            const dim3 tgrid((g->Nx + kTile - 1) / kTile, (g->Ny + kTile - 1) / kTile, zc);
            launch_pdl(fast::orbit_pixels_tiled<IO>, tgrid, dim3(kTile, kTile), st, img, d, qm,
                       img4, (int64_t)z0, skip);
          } else {
            const dim3 pgrid((g->Nx + 255) / 256, g->Ny, zc);
            launch_pdl(fast::orbit_pixels<IO>, pgrid, dim3(256), st, img, d, qm, img4,
                       (int64_t)z0, skip);
          }
          for (int k = 0; k < zc; ++k) {
            const int64_t z = z0 + k;
            double* pz = partials ? partials + z * per_slice_blocks : nullptr;
            if (mirror)  // half the bins: twice the lanes per group
              launch_pdl(fast::fan_fwd_quarter<SO, IO, 2 * kQSplit, true, true, Epi>, sgrid,
                         dim3(kFwdBlock), st, img + z * sz, img4 + k * slice4, ofs, sdpd,
                         fan_geo<float>(g->geo), d, qm, epi, pz, skip, z);
            else
              launch_pdl(fast::fan_fwd_quarter<SO, IO, kQSplit, true, false, Epi>, sgrid,
                         dim3(kFwdBlock), st, img + z * sz, img4 + k * slice4, ofs, sdpd,
                         fan_geo<float>(g->geo), d, qm, epi, pz, skip, z);
          }
        }
      } else {
        for (int64_t z = 0; z < Nz; ++z)
          launch_pdl(fast::fan_fwd_quarter<SO, IO, kQSplit, false, false, Epi>, sgrid,
                     dim3(kFwdBlock), st,
              img + z * sz, nullptr, ofs, sdpd, fan_geo<float>(g->geo), d, qm, epi,
              partials ? partials + z * per_slice_blocks : nullptr, skip, z);
      }
    } else {
      fast::fan_fwd_fast<SO, IO, ZB, SPLIT, Epi><<<grid, kFwdBlock, 0, st>>>(
          img, static_cast<const float*>(g->ofs), static_cast<const float*>(g->sdpd),
          fan_geo<float>(g->geo), d, epi, partials, skip);
    }
  } else {
    if (g->kind == GR_RADON) {
      radon_fwd_kernel<T, SO, IO, ZB, SPLIT, Epi><<<grid, kFwdBlock, 0, st>>>(
          img, static_cast<const T*>(g->ofs), radon_geo<T>(g->geo), d, epi, partials, skip);
    } else {
      fan_fwd_kernel<T, SO, IO, ZB, SPLIT, Epi><<<grid, kFwdBlock, 0, st>>>(
          img, static_cast<const T*>(g->ofs), static_cast<const T*>(g->sdpd), fan_geo<T>(g->geo),
          d, epi, partials, skip);
    }
  }
  return check_launch();
}

template <typename T, int SO, int IO, int ZB, class Epi>
int launch_fwd_split(const gr_geometry* g, const T* img, int Nz, Epi epi, double* partials,
                     const int* skip, cudaStream_t st) {
  const int sp = fwd_split(g, Nz);
  if constexpr (std::is_same<T, double>::value) {
    if (sp == 1) return launch_fwd_zb<T, SO, IO, ZB, 1>(g, img, Nz, epi, partials, skip, st);
    return launch_fwd_zb<T, SO, IO, ZB, 4>(g, img, Nz, epi, partials, skip, st);
  } else {
    switch (sp) {
      case 1: return launch_fwd_zb<T, SO, IO, ZB, 1>(g, img, Nz, epi, partials, skip, st);
      case 2: return launch_fwd_zb<T, SO, IO, ZB, 2>(g, img, Nz, epi, partials, skip, st);
      case 4: return launch_fwd_zb<T, SO, IO, ZB, 4>(g, img, Nz, epi, partials, skip, st);
      default: return launch_fwd_zb<T, SO, IO, ZB, 8>(g, img, Nz, epi, partials, skip, st);
    }
  }
}

template <typename T, int SO, int IO, class Epi>
int launch_fwd(const gr_geometry* g, const void* img, int Nz, Epi epi, double* partials,
               const int* skip, void* stream) {
  int rc = check_geometry(g);
  if (rc) return rc;
  if (img == nullptr || Nz <= 0) return GR_ERR_ARG;
  if ((Nz + 3) / 4 > 65535) return GR_ERR_TOO_BIG;
  const T* im = static_cast<const T*>(img);
  if (Nz == 1) return launch_fwd_split<T, SO, IO, 1>(g, im, Nz, epi, partials, skip, as_stream(stream));
  return launch_fwd_split<T, SO, IO, 4>(g, im, Nz, epi, partials, skip, as_stream(stream));
}

template <typename T, int IO, int SO, int ZB, int SPLIT, class Epi>
int launch_bwd_zb(const gr_geometry* g, const T* sino, int Nz, Epi epi, double* partials,
                  const int* skip, cudaStream_t st) {
  Dims d = dims_of(g, Nz);
  d.vec4 = aligned_groups_of_4(sino, Nz);
  const dim3 grid = bwd_grid(g, Nz, IO, SPLIT);
  const dim3 block(kBwdTileFast, kBwdTileSlow);
  if constexpr (std::is_same<T, float>::value) {
    // single slices without an angle split: 2 pixels per thread, 128-thread
    // blocks (a 512^2 image then fits in one wave of resident blocks)
    constexpr int PY = (SPLIT == 1 && ZB == 1) ? 2 : 1;
    const dim3 fblock(kBwdTileFast, kBwdTileSlow / PY);
    if (use_quarter_bwd(g, Nz)) {
      const float* ofs = static_cast<const float*>(g->ofs);
      const float* sdpd = static_cast<const float*>(g->sdpd);
      const int chunk = work_slices(g, quarter_bwd_bytes(g, Nz), Nz);
      if (chunk > 0) {
        // slices in chunks: interleaved row copies, then the backprojection
        // on them; each chunk's block partials follow the previous chunk's
        float4* rows4 = static_cast<float4*>(g->work);
        const int64_t per_slice_blocks = (int64_t)grid.x * grid.y;
        for (int z0 = 0; z0 < Nz; z0 += chunk) {
          const int zc = Nz - z0 < chunk ? Nz - z0 : chunk;
          // one more block column writes the base angles' records
          const dim3 rgrid((g->Ns + fast::kOrbitRowPad + 255) / 256 + 1, g->Na / 4, zc);
          launch_pdl(fast::orbit_rows<SO>, rgrid, dim3(256), st, sino, sdpd, ofs,
                     fan_geo<float>(g->geo), d, rows4, (int64_t)z0, skip);
          auto* kernel = dense_fan_bwd<Epi, SPLIT>(g)
                             ? fast::fan_bwd_orbit_rows<IO, SPLIT, kDenseFanBwdBlocks<Epi, SPLIT>, Epi>
                             : fast::fan_bwd_orbit_rows<IO, SPLIT, 1, Epi>;
          launch_pdl(kernel, dim3(grid.x, grid.y, zc), block, st,
                     (const float4*)rows4, fan_geo<float>(g->geo), d, quarter_maps(g), epi,
                     partials ? partials + z0 * per_slice_blocks : nullptr, skip, (int64_t)z0);
        }
      } else {
        launch_pdl(fast::fan_bwd_orbit<IO, SO, SPLIT, Epi>, grid, block, st, sino, ofs, sdpd,
                   fan_geo<float>(g->geo), d, quarter_maps(g), epi, partials, skip, (int64_t)0);
      }
    } else if (use_radon_orbit_bwd(g, Nz)) {
      // half-circle orbits, slices in chunks: the mirror-interleaved row
      // copies, then the backprojection over the orbits (one slice per block)
      float4* rows4 = static_cast<float4*>(g->work);
      const int chunk = work_slices(g, radon_orbit_bwd_bytes(g, Nz), Nz);
      if (chunk == 0) {
        launch_pdl(fast::radon_bwd_orbit<IO, SO, SPLIT, Epi>, grid, block, st, sino,
                   static_cast<const float*>(g->ofs), d, quarter_maps(g), epi, partials, skip,
                   (int64_t)0);
        return check_launch();
      }
      const int64_t per_slice_blocks = (int64_t)grid.x * grid.y;
      for (int z0 = 0; z0 < Nz; z0 += chunk) {
        const int zc = Nz - z0 < chunk ? Nz - z0 : chunk;
        const dim3 rgrid((g->Ns + fast::kOrbitRowPad + 255) / 256, g->Na / 2, zc);
        launch_pdl(fast::radon_orbit_rows<SO>, rgrid, dim3(256), st, sino, d, rows4,
                   (int64_t)z0, skip);
        launch_pdl(fast::radon_bwd_orbit_rows<IO, SPLIT, Epi>, dim3(grid.x, grid.y, zc), block,
                   st, (const float4*)rows4, static_cast<const float*>(g->ofs), d,
                   quarter_maps(g), epi, partials ? partials + z0 * per_slice_blocks : nullptr,
                   skip, (int64_t)z0);
      }
    } else if (g->kind == GR_RADON) {
      fast::radon_bwd_fast<IO, SO, ZB, SPLIT, PY, Epi><<<grid, fblock, 0, st>>>(
          sino, static_cast<const float*>(g->ofs), d, epi, partials, skip);
    } else {
      fast::fan_bwd_fast<IO, SO, ZB, SPLIT, PY, Epi><<<grid, fblock, 0, st>>>(
          sino, static_cast<const float*>(g->ofs), static_cast<const float*>(g->sdpd),
          fan_geo<float>(g->geo), d, epi, partials, skip);
    }
  } else {
    if (g->kind == GR_RADON) {
      radon_bwd_kernel<T, IO, SO, ZB, SPLIT, Epi><<<grid, block, 0, st>>>(
          sino, static_cast<const T*>(g->ofs), d, epi, partials, skip);
    } else {
      fan_bwd_kernel<T, IO, SO, ZB, SPLIT, Epi><<<grid, block, 0, st>>>(
          sino, static_cast<const T*>(g->ofs), static_cast<const T*>(g->sdpd), fan_geo<T>(g->geo),
          d, epi, partials, skip);
    }
  }
  return check_launch();
}

template <typename T, int IO, int SO, int ZB, class Epi>
int launch_bwd_split(const gr_geometry* g, const T* sino, int Nz, Epi epi, double* partials,
                     const int* skip, cudaStream_t st) {
  const int sp = bwd_split(g, Nz);
  if constexpr (std::is_same<T, double>::value) {
    if (sp == 1) return launch_bwd_zb<T, IO, SO, ZB, 1>(g, sino, Nz, epi, partials, skip, st);
    return launch_bwd_zb<T, IO, SO, ZB, 4>(g, sino, Nz, epi, partials, skip, st);
  } else {
    switch (sp) {
      case 1: return launch_bwd_zb<T, IO, SO, ZB, 1>(g, sino, Nz, epi, partials, skip, st);
      case 2: return launch_bwd_zb<T, IO, SO, ZB, 2>(g, sino, Nz, epi, partials, skip, st);
      case 4: return launch_bwd_zb<T, IO, SO, ZB, 4>(g, sino, Nz, epi, partials, skip, st);
      default: return launch_bwd_zb<T, IO, SO, ZB, 8>(g, sino, Nz, epi, partials, skip, st);
    }
  }
}

template <typename T, int IO, int SO, class Epi>
int launch_bwd(const gr_geometry* g, const void* sino, int Nz, Epi epi, double* partials,
               const int* skip, void* stream) {
  int rc = check_geometry(g);
  if (rc) return rc;
  if (sino == nullptr || Nz <= 0) return GR_ERR_ARG;
  if ((Nz + 3) / 4 > 65535) return GR_ERR_TOO_BIG;
  const T* sn = static_cast<const T*>(sino);
  if (Nz == 1) return launch_bwd_split<T, IO, SO, 1>(g, sn, Nz, epi, partials, skip, as_stream(stream));
  return launch_bwd_split<T, IO, SO, 4>(g, sn, Nz, epi, partials, skip, as_stream(stream));
}

// Fills a gr_geometry from the reference-style argument list.
inline gr_geometry make_geo(int kind, int dtype, const void* ofs, const void* sdpd, const double* geo) {
  gr_geometry g;
  g.kind = kind;
  g.dtype = dtype;
  g.fwd_split = 0;
  g.bwd_split = 0;
  g.sym = 0;  // the reference-style entries keep every angle's own geometry
  for (int m = 0; m < 3; ++m)
    for (int k = 0; k < 6; ++k) g.sym_map[m][k] = 0;
  g.work = nullptr;
  g.work_bytes = 0;
  g.ofs = ofs;
  g.sdpd = sdpd;
  const int n = kind == GR_RADON ? 6 : 11;
  for (int i = 0; i < 11; ++i) g.geo[i] = i < n && geo ? geo[i] : 0.0;
  if (geo == nullptr) {
    g.Nx = g.Ny = g.Ns = g.Na = 0;
  } else if (kind == GR_RADON) {
    g.Nx = (int)geo[2];
    g.Ny = (int)geo[3];
    g.Ns = (int)geo[4];
    g.Na = (int)geo[5];
  } else {
    g.Nx = (int)geo[6];
    g.Ny = (int)geo[7];
    g.Ns = (int)geo[8];
    g.Na = (int)geo[9];
  }
  return g;
}

}  // namespace launch
}  // namespace gr
