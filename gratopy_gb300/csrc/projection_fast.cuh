// float32 throughput kernels for the four projections.
//
// Same operator as projection.cuh (gratopy radon.cl / fanbeam.cl), same
// deterministic gather structure and epilogues, restructured to issue fewer
// instructions per pixel-angle -- the kernels are issue-bound, not memory
// bound:
//  * backprojection: for every chunk of kWinAngles angles the block stages,
//    per angle, the window of kWin consecutive detector bins its pixel tile
//    projects onto (values outside the detector are zeros, fan values are
//    premultiplied by sdpd).  A pixel-angle then costs two 32-bit shared
//    loads, with no bounds tests; an angle whose window does not fit (extreme
//    magnification) falls back to direct global loads.
//  * forward: row bounds from one fused multiply-add each, a single
//    approximate reciprocal per candidate pixel (fan), 32-bit offsets and an
//    unrolled candidate loop.
// float64 keeps the reference-order kernels of projection.cuh.
#pragma once

#include <type_traits>

#include "projection.cuh"

namespace gr {
namespace fast {

constexpr int kWin = 128;  // staged detector bins per angle (at most)

// Angles staged per pass: 32 for single slices, 16 when 4 slices are staged.
template <int ZB>
struct WinAngles {
  static constexpr int value = ZB == 1 ? 32 : 16;
};

__device__ __forceinline__ float rcp_approx(float v) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(v));
  return r;
}

// ------------------------------------------------------------ backprojection
// Block: 32 lanes along the contiguous pixel axis x 8/PY thread rows; ASPLIT
// thread rows share a pixel row and take interleaved angles; each thread owns
// PY pixels spaced kRows apart along the slow axis.  The pixel tile is
// 32 x 8/ASPLIT whatever PY is.
template <int ASPLIT, int PY>
struct Tile {
  static constexpr int kThreadsY = kBwdTileSlow / PY;  // thread rows of the block
  static constexpr int kRows = kThreadsY / ASPLIT;     // pixel rows per thread layer
  static constexpr int kSlow = kRows * PY;             // slow extent of the tile
};

// Per-angle staged record: Radon (X, Y, off - ws, w) / fan (qx, qy, ddx, ddy,
// dx, dy, w / R, mid - ws); `ws` is the first staged bin and `wn` the number
// of staged bins; ws == INT_MIN marks an angle whose window does not fit
// (its record then keeps the absolute offset / detector midpoint).
struct RadonRec {
  float4 r;
  int ws, wn;
};
// Fan record: with P the pixel centre relative to the image midpoint,
// t = a.x P.x + a.y P.y + a.z and s = b.x P.x + b.y P.y + b.z (the source
// offset folded into a.z, b.z); a.w, b.w step t and s between the pixels one
// thread owns; c = (angle weight / R, detector midpoint - ws).
struct FanRec {
  float4 a, b;
  float2 c;
  int ws, wn;
};

template <int ZB>
struct Window {
  float v[WinAngles<ZB>::value][ZB][kWin];
};

// Stage the windows of angles [a0, a0 + na) for slices [z0, z0 + zn): one
// warp per angle, lanes along the detector bins (coalesced for F-ordered
// sinograms); bins outside the detector are stored as zeros.
template <int SO, int ZB, bool FAN, class Rec>
__device__ __forceinline__ void stage_windows(Window<ZB>& win, const Rec* rec, int na, int a0,
                                              const float* __restrict__ sino,
                                              const float* __restrict__ sdpd, const Dims& d,
                                              int64_t z0, int zn) {
  int64_t ss_, sa_, sz_;
  sino_strides<SO>(d, ss_, sa_, sz_);
  const int lane = threadIdx.x, warp = threadIdx.y;
  for (int j = warp; j < na; j += (int)blockDim.y) {
    const int w0 = rec[j].ws, wn = rec[j].wn;
    if (w0 == INT_MIN) continue;
    const float* prow = sino + (int64_t)(a0 + j) * sa_ + z0 * sz_;
    for (int k = lane; k < wn; k += 32) {
      const int bin = w0 + k;
      const bool in = bin >= 0 && bin < (int)d.Ns;
      const float sc = (FAN && in) ? ldg(sdpd + bin) : 1.0f;
      const float* p = prow + (int64_t)bin * ss_;
      if constexpr (SO == ORDER_C && ZB == 4) {
        if (d.vec4) {
          const float4 q = in ? __ldg(reinterpret_cast<const float4*>(p))
                              : make_float4(0.f, 0.f, 0.f, 0.f);
          win.v[j][0][k] = sc * q.x;
          win.v[j][1][k] = sc * q.y;
          win.v[j][2][k] = sc * q.z;
          win.v[j][3][k] = sc * q.w;
          continue;
        }
      }
#pragma unroll
      for (int zz = 0; zz < ZB; ++zz)
        win.v[j][zz][k] = (in && zz < zn) ? sc * ldg(p + zz * sz_) : 0.0f;
    }
  }
}

template <int IO, int SO, int ZB, int ASPLIT, int PY, class Epi>
__device__ __forceinline__ double radon_bwd_fast_tile(const float* __restrict__ sino, const float* __restrict__ ofs, Dims d, Epi epi,
               uint3 bid) {
  using TL = Tile<ASPLIT, PY>;
  constexpr int kWinAngles = WinAngles<ZB>::value;
  __shared__ RadonRec rec[kWinAngles];
  __shared__ Window<ZB> win;
  const int g = threadIdx.y % ASPLIT;
  const int64_t f0 = (int64_t)bid.x * kBwdTileFast;
  const int64_t s0 = (int64_t)bid.y * TL::kSlow;
  const int64_t fast = f0 + threadIdx.x;
  const int64_t slow0 = s0 + threadIdx.y / ASPLIT;
  const int64_t z0 = (int64_t)bid.z * ZB;
  const int zn = (int)min((int64_t)ZB, d.Nz - z0);
  // tile corners in (x, y)
  const float fx0 = (float)(IO == ORDER_F ? f0 : s0);
  const float fy0 = (float)(IO == ORDER_F ? s0 : f0);
  const float fx1 = fx0 + (float)((IO == ORDER_F ? kBwdTileFast : TL::kSlow) - 1);
  const float fy1 = fy0 + (float)((IO == ORDER_F ? TL::kSlow : kBwdTileFast) - 1);
  int64_t ss_, sa_, sz_;
  sino_strides<SO>(d, ss_, sa_, sz_);
  const int Ns = (int)d.Ns;
  float acc[PY][ZB];
#pragma unroll
  for (int p = 0; p < PY; ++p)
#pragma unroll
    for (int k = 0; k < ZB; ++k) acc[p][k] = 0.0f;
  const int tid = threadIdx.x + kBwdTileFast * threadIdx.y;
  float cxs[PY], cys[PY];
#pragma unroll
  for (int p = 0; p < PY; ++p) {
    const int64_t slow = slow0 + p * TL::kRows;
    cxs[p] = (float)(IO == ORDER_F ? fast : slow);
    cys[p] = (float)(IO == ORDER_F ? slow : fast);
  }
  for (int a0 = 0; a0 < d.Na; a0 += kWinAngles) {
    const int na = (int)min((int64_t)kWinAngles, d.Na - a0);
    __syncthreads();
    if (tid < na) {
      const float* o = ofs + 8 * (int64_t)(a0 + tid);
      const float X = o[0], Y = o[1], off = o[2];
      const float lo = off + fminf(fx0 * X, fx1 * X) + fminf(fy0 * Y, fy1 * Y);
      const float hi = off + fmaxf(fx0 * X, fx1 * X) + fmaxf(fy0 * Y, fy1 * Y);
      const bool finite = lo > -1e9f && hi < 1e9f;
      const int w0 = finite ? (int)floorf(lo) - 1 : 0;
      const int wn = finite ? (int)floorf(hi) + 3 - w0 : kWin + 1;
      const bool fits = finite && wn <= kWin;
      RadonRec r;
      r.r = make_float4(X, Y, fits ? off - (float)w0 : off, o[4]);
      r.ws = fits ? w0 : INT_MIN;
      r.wn = fits ? wn : 0;
      rec[tid] = r;
    }
    const int all_fit = __syncthreads_and(tid >= na || rec[tid].ws != INT_MIN);
    stage_windows<SO, ZB, false>(win, rec, na, a0, sino, nullptr, d, z0, zn);
    __syncthreads();
    if (all_fit && na == kWinAngles) {
      // common case: every window staged, no per-angle branch
#pragma unroll 4
      for (int jj = 0; jj < kWinAngles / ASPLIT; ++jj) {
        const int j = g + jj * ASPLIT;
        const float4 r = rec[j].r;
#pragma unroll
        for (int p = 0; p < PY; ++p) {
          const float s = fmaf(cxs[p], r.x, fmaf(cys[p], r.y, r.z));
          const float fl = floorf(s);
          const float fr = s - fl;
          const unsigned i = min((unsigned)(int)fl, (unsigned)(kWin - 2));
#pragma unroll
          for (int k = 0; k < ZB; ++k) {
            const float v0 = win.v[j][k][i], v1 = win.v[j][k][i + 1];
            acc[p][k] = fmaf(r.w, fmaf(fr, v1 - v0, v0), acc[p][k]);
          }
        }
      }
    } else {
    for (int j = g; j < na; j += ASPLIT) {
      const RadonRec r = rec[j];
#pragma unroll
      for (int p = 0; p < PY; ++p) {
        const float s = fmaf(cxs[p], r.r.x, fmaf(cys[p], r.r.y, r.r.z));
        const float fl = floorf(s);
        const float fr = s - fl;
        if (r.ws != INT_MIN) {
          const unsigned i = min((unsigned)(int)fl, (unsigned)(kWin - 2));
#pragma unroll
          for (int k = 0; k < ZB; ++k) {
            const float v0 = win.v[j][k][i], v1 = win.v[j][k][i + 1];
            acc[p][k] = fmaf(r.r.w, fmaf(fr, v1 - v0, v0), acc[p][k]);
          }
        } else {
          int sm = (int)fl, sp = sm + 1;
          float wm = 1.0f - fr, wp = fr;
          if (sm < 0 || sm >= Ns) { wm = 0.0f; sm = 0; }
          if (sp < 0 || sp >= Ns) { wp = 0.0f; sp = 0; }
          const float* pm = sino + (int64_t)(a0 + j) * sa_ + (int64_t)sm * ss_ + z0 * sz_;
          const float* pp = sino + (int64_t)(a0 + j) * sa_ + (int64_t)sp * ss_ + z0 * sz_;
#pragma unroll
          for (int k = 0; k < ZB; ++k)
            if (k < zn) acc[p][k] += r.r.w * (wm * ldg(pm + k * sz_) + wp * ldg(pp + k * sz_));
        }
      }
    }
    }
  }
  // fixed-order combination of the ASPLIT angle groups
  if constexpr (ASPLIT > 1) {
    __shared__ float cred[kBwdTileSlow][PY][ZB][kBwdTileFast];
    __syncthreads();
#pragma unroll
    for (int p = 0; p < PY; ++p)
#pragma unroll
      for (int k = 0; k < ZB; ++k) cred[threadIdx.y][p][k][threadIdx.x] = acc[p][k];
    __syncthreads();
    if (g == 0) {
#pragma unroll
      for (int p = 0; p < PY; ++p)
#pragma unroll
        for (int k = 0; k < ZB; ++k) {
          float t = cred[threadIdx.y][p][k][threadIdx.x];
#pragma unroll
          for (int q = 1; q < ASPLIT; ++q) t += cred[threadIdx.y + q][p][k][threadIdx.x];
          acc[p][k] = t;
        }
    }
  }
  double part = 0.0;
  if (g == 0) {
#pragma unroll
    for (int p = 0; p < PY; ++p) {
      const int64_t slow = slow0 + p * TL::kRows;
      const int64_t x = IO == ORDER_F ? fast : slow;
      const int64_t y = IO == ORDER_F ? slow : fast;
      if (x < d.Nx && y < d.Ny) {
#pragma unroll
        for (int k = 0; k < ZB; ++k)
          if (k < zn) part += epi(x, y, z0 + k, img_index<IO>(x, y, z0 + k, d), acc[p][k]);
      }
    }
  }
  return part;
}

template <int IO, int SO, int ZB, int ASPLIT, int PY, class Epi>
__global__ void __launch_bounds__(kBwdTileFast * kBwdTileSlow)
radon_bwd_fast(const float* __restrict__ sino, const float* __restrict__ ofs, Dims d, Epi epi,
               double* __restrict__ partials, const int* __restrict__ skip) {
  __shared__ double red[32];
  if (skip != nullptr && *skip) return;
  const double part = radon_bwd_fast_tile<IO, SO, ZB, ASPLIT, PY, Epi>(sino, ofs, d, epi, blockIdx);
  if (Epi::kReduce) {
    double t = block_sum(part, red);
    if (threadIdx.x + blockDim.x * threadIdx.y == 0)
      partials[bid_linear()] = t;
  }
}

template <int IO, int SO, int ZB, int ASPLIT, int PY, class Epi>
__device__ __forceinline__ double fan_bwd_fast_tile(const float* __restrict__ sino, const float* __restrict__ ofs,
             const float* __restrict__ sdpd, FanGeo<float> gg, Dims d, Epi epi,
             uint3 bid) {
  using TL = Tile<ASPLIT, PY>;
  constexpr int kWinAngles = WinAngles<ZB>::value;
  __shared__ FanRec rec[kWinAngles];
  __shared__ Window<ZB> win;
  const int g = threadIdx.y % ASPLIT;
  const int64_t f0 = (int64_t)bid.x * kBwdTileFast;
  const int64_t s0 = (int64_t)bid.y * TL::kSlow;
  const int64_t fast = f0 + threadIdx.x;
  const int64_t slow0 = s0 + threadIdx.y / ASPLIT;
  const int64_t z0 = (int64_t)bid.z * ZB;
  const int zn = (int)min((int64_t)ZB, d.Nz - z0);
  const float fx0 = (float)(IO == ORDER_F ? f0 : s0) - gg.midx;
  const float fy0 = (float)(IO == ORDER_F ? s0 : f0) - gg.midy;
  const float fx1 = fx0 + (float)((IO == ORDER_F ? kBwdTileFast : TL::kSlow) - 1);
  const float fy1 = fy0 + (float)((IO == ORDER_F ? TL::kSlow : kBwdTileFast) - 1);
  int64_t ss_, sa_, sz_;
  sino_strides<SO>(d, ss_, sa_, sz_);
  const int Ns = (int)d.Ns;
  const float R = gg.R;
  const float R_sqr_inv = 1.0f / (R * R);
  const float dxi_sqr_inv = 1.0f / (gg.delta_xi * gg.delta_xi);
  float acc[PY][ZB];
#pragma unroll
  for (int p = 0; p < PY; ++p)
#pragma unroll
    for (int k = 0; k < ZB; ++k) acc[p][k] = 0.0f;
  const int tid = threadIdx.x + kBwdTileFast * threadIdx.y;
  float pxs[PY], pys[PY];
#pragma unroll
  for (int p = 0; p < PY; ++p) {
    const int64_t slow = slow0 + p * TL::kRows;
    pxs[p] = (float)(IO == ORDER_F ? fast : slow) - gg.midx;
    pys[p] = (float)(IO == ORDER_F ? slow : fast) - gg.midy;
  }
  for (int a0 = 0; a0 < d.Na; a0 += kWinAngles) {
    const int na = (int)min((int64_t)kWinAngles, d.Na - a0);
    __syncthreads();
    if (tid < na) {
      const float* o = ofs + 8 * (int64_t)(a0 + tid);
      const float qx = o[2], qy = o[3];
      const float ddx = (o[4] - o[2]) * R_sqr_inv, ddy = (o[5] - o[3]) * R_sqr_inv;
      const float dx = o[0] * dxi_sqr_inv, dy = o[1] * dxi_sqr_inv;
      // projected detector coordinate of the four tile corners (a projective
      // map: its extremes over the rectangle are at the corners)
      float lo = 3.0e38f, hi = -3.0e38f;
      bool ok = true;
#pragma unroll
      for (int c = 0; c < 4; ++c) {
        const float px = ((c & 1) ? fx1 : fx0) - qx, py = ((c & 2) ? fy1 : fy0) - qy;
        const float t = ddx * px + ddy * py;
        ok = ok && t > 0.0f;
        const float xi = (dx * px + dy * py) / t + gg.mid_det;
        lo = fminf(lo, xi);
        hi = fmaxf(hi, xi);
      }
      const bool finite = ok && lo > -1e9f && hi < 1e9f;
      const int w0 = finite ? (int)floorf(lo) - 1 : 0;
      const int wn = finite ? (int)floorf(hi) + 3 - w0 : kWin + 1;
      const bool fits = finite && wn <= kWin;
      FanRec r;
      const float rows = (float)TL::kRows;
      r.a = make_float4(ddx, ddy, -fmaf(ddx, qx, ddy * qy), (IO == ORDER_F ? ddy : ddx) * rows);
      r.b = make_float4(dx, dy, -fmaf(dx, qx, dy * qy), (IO == ORDER_F ? dy : dx) * rows);
      r.c = make_float2(o[6] / R, fits ? gg.mid_det - (float)w0 : gg.mid_det);
      r.ws = fits ? w0 : INT_MIN;
      r.wn = fits ? wn : 0;
      rec[tid] = r;
    }
    const int all_fit = __syncthreads_and(tid >= na || rec[tid].ws != INT_MIN);
    stage_windows<SO, ZB, true>(win, rec, na, a0, sino, sdpd, d, z0, zn);
    __syncthreads();
    if (all_fit && na == kWinAngles) {
#pragma unroll 4
      for (int jj = 0; jj < kWinAngles / ASPLIT; ++jj) {
        const int j = g + jj * ASPLIT;
        const float4 ra = rec[j].a, rb = rec[j].b;
        const float2 rc = rec[j].c;
        float t = fmaf(ra.x, pxs[0], fmaf(ra.y, pys[0], ra.z));
        float ss = fmaf(rb.x, pxs[0], fmaf(rb.y, pys[0], rb.z));
#pragma unroll
        for (int p = 0; p < PY; ++p) {
          if (p > 0) {
            t += ra.w;
            ss += rb.w;
          }
          const float inv = rcp_approx(t);
          const float xi = fmaf(ss, inv, rc.y);
          const float scale = rc.x * inv;
          const float fl = floorf(xi);
          const float fr = xi - fl;
          // every staged window holds its tile's detector range with a
          // one-bin margin; the clamp only guards the shared-memory bounds
          const unsigned i = min((unsigned)(int)fl, (unsigned)(kWin - 2));
#pragma unroll
          for (int k = 0; k < ZB; ++k) {
            const float v0 = win.v[j][k][i], v1 = win.v[j][k][i + 1];
            acc[p][k] = fmaf(scale, fmaf(fr, v1 - v0, v0), acc[p][k]);
          }
        }
      }
    } else {
    for (int j = g; j < na; j += ASPLIT) {
      const FanRec r = rec[j];
      float t = fmaf(r.a.x, pxs[0], fmaf(r.a.y, pys[0], r.a.z));
      float ss = fmaf(r.b.x, pxs[0], fmaf(r.b.y, pys[0], r.b.z));
#pragma unroll
      for (int p = 0; p < PY; ++p) {
        if (p > 0) {
          t += r.a.w;
          ss += r.b.w;
        }
        const float inv = rcp_approx(t);
        const float xi = fmaf(ss, inv, r.c.y);
        const float scale = r.c.x * inv;
        const float fl = floorf(xi);
        const float fr = xi - fl;
        if (r.ws != INT_MIN) {
          const unsigned i = min((unsigned)(int)fl, (unsigned)(kWin - 2));
#pragma unroll
          for (int k = 0; k < ZB; ++k) {
            const float v0 = win.v[j][k][i], v1 = win.v[j][k][i + 1];
            acc[p][k] = fmaf(scale, fmaf(fr, v1 - v0, v0), acc[p][k]);
          }
        } else {
          int xim = (int)fl, xip = xim + 1;
          float Wm = 1.0f - fr, Wp = fr;
          if (xim < 0 || xim >= Ns) { Wm = 0.0f; xim = 0; } else { Wm *= ldg(sdpd + xim); }
          if (xip < 0 || xip >= Ns) { Wp = 0.0f; xip = 0; } else { Wp *= ldg(sdpd + xip); }
          const float* pm = sino + (int64_t)(a0 + j) * sa_ + (int64_t)xim * ss_ + z0 * sz_;
          const float* pp = sino + (int64_t)(a0 + j) * sa_ + (int64_t)xip * ss_ + z0 * sz_;
#pragma unroll
          for (int k = 0; k < ZB; ++k)
            if (k < zn) acc[p][k] += scale * (Wm * ldg(pm + k * sz_) + Wp * ldg(pp + k * sz_));
        }
      }
    }
    }
  }
  if constexpr (ASPLIT > 1) {
    __shared__ float cred[kBwdTileSlow][PY][ZB][kBwdTileFast];
    __syncthreads();
#pragma unroll
    for (int p = 0; p < PY; ++p)
#pragma unroll
      for (int k = 0; k < ZB; ++k) cred[threadIdx.y][p][k][threadIdx.x] = acc[p][k];
    __syncthreads();
    if (g == 0) {
#pragma unroll
      for (int p = 0; p < PY; ++p)
#pragma unroll
        for (int k = 0; k < ZB; ++k) {
          float t = cred[threadIdx.y][p][k][threadIdx.x];
#pragma unroll
          for (int q = 1; q < ASPLIT; ++q) t += cred[threadIdx.y + q][p][k][threadIdx.x];
          acc[p][k] = t;
        }
    }
  }
  double part = 0.0;
  if (g == 0) {
#pragma unroll
    for (int p = 0; p < PY; ++p) {
      const int64_t slow = slow0 + p * TL::kRows;
      const int64_t x = IO == ORDER_F ? fast : slow;
      const int64_t y = IO == ORDER_F ? slow : fast;
      if (x < d.Nx && y < d.Ny) {
#pragma unroll
        for (int k = 0; k < ZB; ++k)
          if (k < zn) part += epi(x, y, z0 + k, img_index<IO>(x, y, z0 + k, d), acc[p][k]);
      }
    }
  }
  return part;
}

template <int IO, int SO, int ZB, int ASPLIT, int PY, class Epi>
__global__ void __launch_bounds__(kBwdTileFast * kBwdTileSlow)
fan_bwd_fast(const float* __restrict__ sino, const float* __restrict__ ofs,
             const float* __restrict__ sdpd, FanGeo<float> gg, Dims d, Epi epi,
             double* __restrict__ partials, const int* __restrict__ skip) {
  __shared__ double red[32];
  if (skip != nullptr && *skip) return;
  const double part = fan_bwd_fast_tile<IO, SO, ZB, ASPLIT, PY, Epi>(sino, ofs, sdpd, gg, d, epi, blockIdx);
  if (Epi::kReduce) {
    double t = block_sum(part, red);
    if (threadIdx.x + blockDim.x * threadIdx.y == 0)
      partials[bid_linear()] = t;
  }
}

// -------------------------------------------------------------- forward
// A thread group of SPLIT lanes owns kRayGroup adjacent detector bins of one
// angle: the row bounds, the reciprocal (fan) and the image load of every
// candidate pixel are shared by the group's bins, and each bin keeps its own
// accumulator.  Candidate pixels are those between the rays through the bins
// s0 - 1 and s0 + kRayGroup; a bin's weight is clamped at zero outside its
// own pair of neighbouring rays, which selects exactly the pixels the
// reference's per-ray bounds select.  Rows whose candidate range misses the
// image are skipped by solving the two linear bound conditions for the rows.
constexpr int kRayGroup = 4;

// The ZB slices of one pixel, times `scale`: one float4 load when the image
// is C-ordered and 16-byte aligned in groups of 4 slices, else ZB loads.
template <int IO, int ZB>
__device__ __forceinline__ void load_slices(float (&v)[ZB], const float* p, int64_t sz, int zn,
                                            bool vec4, float scale) {
  if constexpr (IO == ORDER_C && ZB == 4) {
    if (vec4) {
      const float4 q = __ldg(reinterpret_cast<const float4*>(p));
      v[0] = q.x * scale;
      v[1] = q.y * scale;
      v[2] = q.z * scale;
      v[3] = q.w * scale;
      return;
    }
  }
#pragma unroll
  for (int k = 0; k < ZB; ++k) v[k] = k < zn ? ldg(p + k * sz) * scale : 0.0f;
}

template <int SPLIT>
struct GroupLayout {
  static constexpr int kGroupsPerWarp = 32 / SPLIT;
  static constexpr int kRaysPerBlock = kGroupsPerWarp * kRayGroup * (kFwdBlock / 32);
  int64_t s0;
  int lane_group;
  __device__ __forceinline__ explicit GroupLayout(uint3 bid) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    s0 = (int64_t)bid.x * kRaysPerBlock +
         ((int64_t)warp * kGroupsPerWarp + lane % kGroupsPerWarp) * kRayGroup;
    lane_group = lane / kGroupsPerWarp;
  }
};

// Rows y in [0, n) with lo(y) = a_lo + b_lo*y <= hi_lim and
// hi(y) = a_hi + b_hi*y >= 0 (a conservative superset: one row of margin).
__device__ __forceinline__ void row_range(float a_lo, float b_lo, float a_hi, float b_hi,
                                          float hi_lim, int n, int& y0, int& y1) {
  float lo = 0.0f, hi = (float)(n - 1);
  // a_lo + b_lo*y <= hi_lim
  if (fabsf(b_lo) > 1e-20f) {
    const float yb = (hi_lim - a_lo) / b_lo;
    if (b_lo > 0.0f) hi = fminf(hi, yb); else lo = fmaxf(lo, yb);
  } else if (a_lo > hi_lim + 1.0f) {
    hi = -1.0f;
  }
  // a_hi + b_hi*y >= 0
  if (fabsf(b_hi) > 1e-20f) {
    const float yb = -a_hi / b_hi;
    if (b_hi > 0.0f) lo = fmaxf(lo, yb); else hi = fminf(hi, yb);
  } else if (a_hi < -1.0f) {
    hi = -1.0f;
  }
  if (!(lo <= hi)) {  // also catches NaN bounds: then visit every row
    if (lo == lo && hi == hi) { y0 = 0; y1 = -1; return; }
    y0 = 0; y1 = n - 1; return;
  }
  y0 = max(0, (int)floorf(lo) - 1);
  y1 = min(n - 1, (int)ceilf(hi) + 1);
}

// Output oi of a lane group's R x C sums (acc[oi / C][oi % C]) picked by
// selects, so that the lanes of a group, each with its own oi, run one
// instruction stream (the epilogue's loads and stores of the group's outputs
// then go out together instead of one lane's one after another).
template <int R, int C>
__device__ __forceinline__ float pick_output(const float (&acc)[R][C], int oi) {
  float v = 0.0f;
#pragma unroll
  for (int r = 0; r < R; ++r)
#pragma unroll
    for (int c = 0; c < C; ++c) v = (oi == r * C + c) ? acc[r][c] : v;
  return v;
}

template <int SO, int IO, int ZB, int SPLIT, class Epi>
__device__ __forceinline__ double radon_fwd_fast_tile(const float* __restrict__ img, const float* __restrict__ ofs, RadonGeo<float> g,
               Dims d, Epi epi, uint3 bid) {
  const GroupLayout<SPLIT> L(bid);
  const int64_t s0 = L.s0;
  const int64_t a = bid.y;
  const int64_t z0 = (int64_t)bid.z * ZB;
  const bool active = s0 < d.Ns;
  const int zn = (int)min((int64_t)ZB, d.Nz - z0);
  float acc[kRayGroup][ZB];
#pragma unroll
  for (int r = 0; r < kRayGroup; ++r)
#pragma unroll
    for (int k = 0; k < ZB; ++k) acc[r][k] = 0.0f;
  if (active) {
    const float* o8 = ofs + 8 * a;
    float ox = o8[0], oy = o8[1];
    const float oz = o8[2], ow = o8[3];
    const bool flip = o8[5] != 0.0f;
    int Nxx = (int)d.Nx, Nyy = (int)d.Ny;
    int64_t sx, sy, sz;
    img_strides<IO>(d, sx, sy, sz);
    int64_t step_x = sx, step_y = sy;
    if (flip) {
      float t = ox; ox = oy; oy = t;
      Nxx = (int)d.Ny;
      Nyy = (int)d.Nx;
      step_x = sy;
      step_y = sx;
    }
    // position of pixel x in row y relative to bin s0: p = x*ox + dd,
    // dd = y*oy + oz - s0; candidates have p in (-1, kRayGroup)
    const float c_lo = ow < 0.0f ? (float)kRayGroup : -1.0f;
    const float c_hi = ow < 0.0f ? -1.0f : (float)kRayGroup;
    const float base = oz - (float)(int)s0;
    // rows where the candidate x-range meets [0, Nxx-1]
    const float lx = (float)(Nxx - 1) * ox;
    int y0, y1;
    row_range(base + fminf(0.0f, lx) - (float)kRayGroup, oy, base + fmaxf(0.0f, lx) + 1.0f, oy,
              0.0f, Nyy, y0, y1);
    const float* img0 = img + z0 * sz;
    const int ys = y0 + L.lane_group;
    float yf = (float)ys;
    for (int y = ys; y <= y1; y += SPLIT, yf += (float)SPLIT) {
      const float dd = fmaf(yf, oy, base);
      const int x_low = max((int)((c_lo - dd) * ow), 0);
      const int x_high = min((int)((c_hi - dd) * ow), Nxx - 1);
      const float* p = img0 + (int64_t)y * step_y + (int64_t)x_low * step_x;
      float pos = fmaf((float)x_low, ox, dd);
      if constexpr (ZB == 1) {
        // single slices: branch-free hat weights (a zero weight adds zero)
        // and the four bins' sums as two register pairs, updated by packed
        // float32 multiply-adds; two candidates per trip (measured: 256^2
        // Radon forward 43.7 -> 37 us with the unrolled loop)
        float2 s01 = make_float2(acc[0][0], acc[1][0]), s23 = make_float2(acc[2][0], acc[3][0]);
#pragma unroll 2
        for (int x = x_low; x <= x_high; ++x) {
          const float v = ldg(p);
          const float2 v2 = make_float2(v, v);
          const float2 w01 = make_float2(fmaxf(0.0f, 1.0f - fabsf(pos)),
                                         fmaxf(0.0f, 1.0f - fabsf(pos - 1.0f)));
          const float2 w23 = make_float2(fmaxf(0.0f, 1.0f - fabsf(pos - 2.0f)),
                                         fmaxf(0.0f, 1.0f - fabsf(pos - 3.0f)));
          s01 = __ffma2_rn(w01, v2, s01);
          s23 = __ffma2_rn(w23, v2, s23);
          pos += ox;
          p += step_x;
        }
        acc[0][0] = s01.x;
        acc[1][0] = s01.y;
        acc[2][0] = s23.x;
        acc[3][0] = s23.y;
      } else {
      for (int x = x_low; x <= x_high; ++x) {
        float v[ZB];
        load_slices<IO, ZB>(v, p, sz, zn, d.vec4, 1.0f);
#pragma unroll
        for (int r = 0; r < kRayGroup; ++r) {
          const float w = 1.0f - fabsf(pos - (float)r);
          if (w > 0.0f) {
#pragma unroll
            for (int k = 0; k < ZB; ++k) acc[r][k] = fmaf(w, v[k], acc[r][k]);
          }
        }
        pos += ox;
        p += step_x;
      }
      }
    }
  }
  if (SPLIT > 1) {
#pragma unroll
    for (int r = 0; r < kRayGroup; ++r) warp_reduce_rows<SPLIT>(acc[r]);
  }
  // every lane of the group now holds every sum: the lanes share the
  // group's outputs, one each per round
  constexpr int kN = kRayGroup * ZB;
  double part = 0.0;
  if (active) {
    const float scale = g.delta_x * g.delta_x / g.delta_xi;
#pragma unroll
    for (int base = 0; base < kN; base += SPLIT) {
      const int oi = base + L.lane_group;
      const float v = pick_output<kRayGroup, ZB>(acc, oi);
      const int64_t s = s0 + oi / ZB;
      const int k = oi % ZB;
      if (oi < kN && s < d.Ns && k < zn)
        part += epi(s, a, z0 + k, sino_index<SO>(s, a, z0 + k, d), v * scale);
    }
  }
  return part;
}

template <int SO, int IO, int ZB, int SPLIT, class Epi>
__global__ void __launch_bounds__(kFwdBlock)
radon_fwd_fast(const float* __restrict__ img, const float* __restrict__ ofs, RadonGeo<float> g,
               Dims d, Epi epi, double* __restrict__ partials, const int* __restrict__ skip) {
  __shared__ double red[32];
  if (skip != nullptr && *skip) return;
  const double part = radon_fwd_fast_tile<SO, IO, ZB, SPLIT, Epi>(img, ofs, g, d, epi, blockIdx);
  if (Epi::kReduce) {
    double t = block_sum(part, red);
    if (threadIdx.x + blockDim.x * threadIdx.y == 0)
      partials[bid_linear()] = t;
  }
}

template <int SO, int IO, int ZB, int SPLIT, class Epi>
__device__ __forceinline__ double fan_fwd_fast_tile(const float* __restrict__ img, const float* __restrict__ ofs,
             const float* __restrict__ sdpd, FanGeo<float> g, Dims d, Epi epi,
             uint3 bid) {
  const GroupLayout<SPLIT> L(bid);
  const int64_t s0 = L.s0;
  const int64_t a = bid.y;
  const int64_t z0 = (int64_t)bid.z * ZB;
  const bool active = s0 < d.Ns;
  const int zn = (int)min((int64_t)ZB, d.Nz - z0);
  float acc[kRayGroup][ZB];
#pragma unroll
  for (int r = 0; r < kRayGroup; ++r)
#pragma unroll
    for (int k = 0; k < ZB; ++k) acc[r][k] = 0.0f;
  const float R = g.R;
  if (active) {
    float midx = g.midx, midy = g.midy;
    const float* o = ofs + 8 * a;
    float dx = o[0], dy = o[1], qx = o[2], qy = o[3];
    const float d0x = o[4], d0y = o[5];
    const float sr = (float)(int)s0;
    // boundary rays of the group: through bins s0 - 1 and s0 + kRayGroup
    const float fp = -g.mid_det + sr + (float)kRayGroup;
    const float fm = -g.mid_det + sr - 1.0f;
    float dpx = d0x + dx * fp - qx, dpy = d0y + dy * fp - qy;
    float dmx = d0x + dx * fm - qx, dmy = d0y + dy * fm - qy;
    float ddx = (d0x - qx) / (R * R), ddy = (d0y - qy) / (R * R);
    const float xx2 = g.delta_xi * g.delta_xi;
    dx /= xx2;
    dy /= xx2;
    const float RE = g.RE * (1.0f / R);
    int Nyy = (int)d.Ny, Nxx = (int)d.Nx;
    int64_t sx, sy, sz;
    img_strides<IO>(d, sx, sy, sz);
    int64_t step_x = sx, step_y = sy;
    // Rows run along x unless a boundary ray is closer to the x axis than to
    // the y axis (fanbeam.cl:183-206).  The candidates of a row form the
    // interval between the two boundary rays only if the wedge between them
    // does not contain the row direction; the wedge of a group spans 5 bins,
    // so on coarse detectors it can hold a diagonal, and then the other
    // orientation is taken when the swapped one would contain its rows.
    const bool steep = fabsf(dpx) < fabsf(dpy) && fabsf(dmx) < fabsf(dmy);
    if (!steep && dpx * dmx > 0.0f) {
      float t;
      t = ddx; ddx = ddy; ddy = t;
      t = dx; dx = dy; dy = t;
      t = qx; qx = qy; qy = t;
      t = dpx; dpx = dpy; dpy = t;
      t = dmx; dmx = dmy; dmy = t;
      t = midx; midx = midy; midy = t;
      Nyy = (int)d.Nx;
      Nxx = (int)d.Ny;
      step_x = sy;
      step_y = sx;
    }
    dpx /= dpy;
    dmx /= dmy;
    if (qy * (dmx - dpx) < 0.0f) {
      float t = dpx; dpx = dmx; dmx = t;
    }
    const float s_mid0 = sr - g.mid_det;
    // row y: candidate x (absolute pixel index) in
    // [ceil(qxm + dmx*yrel), floor(qxm + dpx*yrel)], yrel = y - midy - qy
    const float qxm = qx + midx, yc = -midy - qy;
    const float hi_lim = (float)(Nxx - 1);
    const float t_c = RE - ddx * midx - ddy * midy;
    const float s_c = -dx * midx - dy * midy;
    int y0, y1;
    row_range(fmaf(dmx, yc, qxm), dmx, fmaf(dpx, yc, qxm), dpx, hi_lim, Nyy, y0, y1);
    const float* img0 = img + z0 * sz;
    const int ys = y0 + L.lane_group;
    float yf = (float)ys;
    for (int y = ys; y <= y1; y += SPLIT, yf += (float)SPLIT) {
      const float yrel = yf + yc;
      const int xhi = (int)floorf(fminf(hi_lim, fmaf(dpx, yrel, qxm)));
      const int xlo = (int)ceilf(fmaxf(0.0f, fmaf(dmx, yrel, qxm)));
      const float xlf = (float)xlo;
      float t = fmaf(ddx, xlf, fmaf(ddy, yf, t_c));
      float ss = fmaf(dx, xlf, fmaf(dy, yf, s_c));
      const float* p = img0 + (int64_t)y * step_y + (int64_t)xlo * step_x;
      for (int x = xlo; x <= xhi; ++x) {
        const float r = rcp_approx(t);
        const float u = fmaf(ss, r, -s_mid0);  // xi - (s0 - mid) in bins
        float v[ZB];
        load_slices<IO, ZB>(v, p, sz, zn, d.vec4, r);
#pragma unroll
        for (int q = 0; q < kRayGroup; ++q) {
          const float w = 1.0f - fabsf((float)q - u);
          if (w > 0.0f) {
#pragma unroll
            for (int k = 0; k < ZB; ++k) acc[q][k] = fmaf(w, v[k], acc[q][k]);
          }
        }
        p += step_x;
        t += ddx;
        ss += dx;
      }
    }
  }
  if (SPLIT > 1) {
#pragma unroll
    for (int r = 0; r < kRayGroup; ++r) warp_reduce_rows<SPLIT>(acc[r]);
  }
  // every lane of the group now holds every sum: the lanes share the
  // group's outputs, one each per round
  constexpr int kN = kRayGroup * ZB;
  double part = 0.0;
  if (active) {
#pragma unroll
    for (int base = 0; base < kN; base += SPLIT) {
      const int oi = base + L.lane_group;
      const float v = pick_output<kRayGroup, ZB>(acc, oi);
      const int64_t s = s0 + oi / ZB;
      const int k = oi % ZB;
      if (oi < kN && s < d.Ns && k < zn) {
        const float sc = sdpd[s] / g.delta_xi * g.delta_x / R;
        part += epi(s, a, z0 + k, sino_index<SO>(s, a, z0 + k, d), v * sc);
      }
    }
  }
  return part;
}

template <int SO, int IO, int ZB, int SPLIT, class Epi>
__global__ void __launch_bounds__(kFwdBlock)
fan_fwd_fast(const float* __restrict__ img, const float* __restrict__ ofs,
             const float* __restrict__ sdpd, FanGeo<float> g, Dims d, Epi epi,
             double* __restrict__ partials, const int* __restrict__ skip) {
  __shared__ double red[32];
  if (skip != nullptr && *skip) return;
  const double part = fan_fwd_fast_tile<SO, IO, ZB, SPLIT, Epi>(img, ofs, sdpd, g, d, epi, blockIdx);
  if (Epi::kReduce) {
    double t = block_sum(part, red);
    if (threadIdx.x + blockDim.x * threadIdx.y == 0)
      partials[bid_linear()] = t;
  }
}

// ------------------------------------------------- quarter-turn symmetry
// When the angles a + m*Na/4 (m = 1, 2, 3) see the pixel grid as angle a sees
// it after m quarter turns (square image centred on the rotation axis,
// equispaced full-circle angles; detected on the host), a lane group of the
// forward projection works on base angle a and, for every candidate pixel P
// of that angle, applies the interpolation weights of P (one reciprocal and
// four hat evaluations) to the four pixels S_m^-1 P: sino[s, a + m Na/4] is
// the projection of the turned image at angle a.  Index maps: pixel (x, y)
// of the base angle is pixel (cx + axx x + axy y, cy + ayx x + ayy y) for
// angle a + m Na/4.
// Lane layout of the orbit forward: a block's warps are split over
// kAnglesPerBlock adjacent base angles, each angle's warps covering the same
// bins, so the image strips the block streams overlap in L1 (adjacent base
// angles differ by 360/Na degrees).  Within a warp, 32 / SPLIT groups of
// SPLIT lanes each own kRayGroup adjacent bins.
constexpr int kQuarterAnglesPerBlock = 2;


template <int SPLIT>
struct QuarterLayout {
  static constexpr int kGroupsPerWarp = 32 / SPLIT;
  static constexpr int kWarpsPerAngle = (kFwdBlock / 32) / kQuarterAnglesPerBlock;
  static constexpr int kBinsPerBlock = kGroupsPerWarp * kRayGroup * kWarpsPerAngle;
  int64_t s0, a;
  int lane_group;
  __device__ __forceinline__ explicit QuarterLayout(uint3 bid) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    a = (int64_t)bid.y * kQuarterAnglesPerBlock + warp / kWarpsPerAngle;
    s0 = (int64_t)bid.x * kBinsPerBlock +
         ((int64_t)(warp % kWarpsPerAngle) * kGroupsPerWarp + lane % kGroupsPerWarp) * kRayGroup;
    lane_group = lane / kGroupsPerWarp;
  }
};

struct QuarterMaps {
  int axx[3], axy[3], ayx[3], ayy[3], cx[3], cy[3];
  // nonzero when map m is the m-th power of one quarter turn: then the
  // relation holds from every angle of an orbit, not only from the base
  // angles in [0, Na/4)
  int cyclic;
  // fan-beam mirror (mirror_pair >= 0): angle (mirror_pair - b) mod Na sees
  // pixel M P as angle b sees P with the detector reversed; M is the lookup
  // (mxx, mxy, myx, myy, mcx, mcy) in the format of the maps above
  int mxx, mxy, myx, myy, mcx, mcy;
  int mirror_pair;
};

// img (and img4) point at slice z; offsets within a slice are 32-bit except
// for C-ordered images, whose slices interleave.
//
// MIRROR (with the orbit copy and cyclic maps): the geometry also has the
// mirror M of qm (angle c0 - b sees M P as angle b sees P, the detector
// reversed).  A reflection turns a quarter turn into its inverse, M L_m =
// L_{-m} M, so the mirrored members img(M L_m P) are the orbit copy's entry
// at M P in the order (0, 3, 2, 1): one more 16-byte load per candidate
// gives the weights of bins s0 .. s0 + 3 four more outputs, at the mirrored
// bins Ns - 1 - s of the angles c0 - (a + m Q).  The groups then walk only
// the bins s < ceil(Ns/2) (the middle bin of an odd detector written once).
template <int SO, int IO, int SPLIT, bool PIX4, bool MIRROR, class Epi>
__device__ __forceinline__ double fan_fwd_quarter_tile(const float* __restrict__ img,
                                                       const float4* __restrict__ img4,
                                                       const float* __restrict__ ofs,
                                                       const float* __restrict__ sdpd,
                                                       FanGeo<float> g, Dims d, QuarterMaps qm,
                                                       Epi epi, uint3 bid, int64_t z) {
  constexpr int kOrbit = 4;
  static_assert(!MIRROR || PIX4, "the mirrored members come from the orbit copy");
  using Off = typename std::conditional<IO == ORDER_C && !PIX4, int64_t, int>::type;
  const QuarterLayout<SPLIT> L(bid);
  const int64_t s0 = L.s0;
  const int64_t a = L.a;                // base angle in [0, Na/4)
  const int64_t quarter = d.Na / kOrbit;
  const int64_t Hs = MIRROR ? (d.Ns + 1) / 2 : d.Ns;  // bins the groups walk
  const bool active = s0 < Hs && a < quarter;
  // bin q's sums for the orbit angles (0, 1) and (2, 3): one register pair
  // each, updated by packed float32 multiply-adds (two lanes per instruction);
  // with MIRROR the same for the entry at M P (mirror components 0 .. 3)
  float2 acc01[kRayGroup], acc23[kRayGroup];
  float2 macc01[MIRROR ? kRayGroup : 1], macc23[MIRROR ? kRayGroup : 1];
#pragma unroll
  for (int q = 0; q < kRayGroup; ++q) acc01[q] = acc23[q] = make_float2(0.0f, 0.0f);
#pragma unroll
  for (int q = 0; q < (MIRROR ? kRayGroup : 1); ++q) macc01[q] = macc23[q] = make_float2(0.0f, 0.0f);
  const float R = g.R;
  int shift = 0;  // accumulator m belongs to row a + ((m + shift) mod 4) Na/4
  if (active) {
    float midx = g.midx, midy = g.midy;
    const float sr = (float)(int)s0;
    const float fp = -g.mid_det + sr + (float)kRayGroup;
    const float fm = -g.mid_det + sr - 1.0f;
    // rays through the group's outer bins -1 and kRayGroup at angle `ang`
    auto boundary_rays = [&](int64_t ang, float& px, float& py, float& mx, float& my) {
      const float* q = ofs + 8 * ang;
      px = q[4] + q[0] * fp - q[2];
      py = q[5] + q[1] * fp - q[3];
      mx = q[4] + q[0] * fm - q[2];
      my = q[5] + q[1] * fm - q[3];
    };
    int64_t ab = a;  // the orbit angle whose geometry this group walks
    {
      float px, py, mx, my;
      boundary_rays(a, px, py, mx, my);
      // With cyclic maps every member of the orbit can serve as the base.
      // Walk a + Na/4 (rays turned by a quarter) when a's rays through this
      // group are steep: the group's lanes then take adjacent image columns
      // and walk down them, so one load instruction of a group reads
      // adjacent pixels (measured at 512^2 x 360: 1181 Gpixel-angle/s with
      // every group in this orientation, 1045 with every group walking
      // rows, 1152 with the orientation of the base angle a alone).
      if (qm.cyclic && fabsf(px) < fabsf(py) && fabsf(mx) < fabsf(my)) {
        ab = a + quarter;
        shift = 1;
      }
    }
    const float* o = ofs + 8 * ab;
    float dx = o[0], dy = o[1], qx = o[2], qy = o[3];
    const float d0x = o[4], d0y = o[5];
    float dpx, dpy, dmx, dmy;
    boundary_rays(ab, dpx, dpy, dmx, dmy);
    float ddx = (d0x - qx) / (R * R), ddy = (d0y - qy) / (R * R);
    const float xx2 = g.delta_xi * g.delta_xi;
    dx /= xx2;
    dy /= xx2;
    const float RE = g.RE * (1.0f / R);
    int Nyy = (int)d.Ny, Nxx = (int)d.Nx;
    int64_t sx, sy, sz;
    img_strides<IO>(d, sx, sy, sz);
    if constexpr (PIX4) {  // the orbit copy is x-fastest whatever the image order
      sx = 1;
      sy = d.Nx;
    }
    // element steps of the turned pixels along the array's x and y axes
    Off mstep_x[kOrbit - 1], mstep_y[kOrbit - 1], mbase[kOrbit - 1];
#pragma unroll
    for (int m = 0; m < kOrbit - 1; ++m) {
      mstep_x[m] = (Off)(qm.axx[m] * sx + qm.ayx[m] * sy);
      mstep_y[m] = (Off)(qm.axy[m] * sx + qm.ayy[m] * sy);
      mbase[m] = (Off)(qm.cx[m] * sx + qm.cy[m] * sy);
    }
    // and of the mirrored pixel M P in the orbit copy
    Off Mstep_x = (Off)(qm.mxx * sx + qm.myx * sy), Mstep_y = (Off)(qm.mxy * sx + qm.myy * sy);
    const Off Mbase = (Off)(qm.mcx * sx + qm.mcy * sy);
    int64_t step_x = sx, step_y = sy;
    const bool steep = fabsf(dpx) < fabsf(dpy) && fabsf(dmx) < fabsf(dmy);
    const bool swap = !steep && dpx * dmx > 0.0f;
    if (swap) {
      float t;
      t = ddx; ddx = ddy; ddy = t;
      t = dx; dx = dy; dy = t;
      t = qx; qx = qy; qy = t;
      t = dpx; dpx = dpy; dpy = t;
      t = dmx; dmx = dmy; dmy = t;
      t = midx; midx = midy; midy = t;
      Nyy = (int)d.Nx;
      Nxx = (int)d.Ny;
      step_x = sy;
      step_y = sx;
#pragma unroll
      for (int m = 0; m < kOrbit - 1; ++m) {
        const Off t2 = mstep_x[m];
        mstep_x[m] = mstep_y[m];
        mstep_y[m] = t2;
      }
      const Off t3 = Mstep_x;
      Mstep_x = Mstep_y;
      Mstep_y = t3;
    }
    dpx /= dpy;
    dmx /= dmy;
    if (qy * (dmx - dpx) < 0.0f) {
      float t = dpx; dpx = dmx; dmx = t;
    }
    const float s_mid0 = sr - g.mid_det;
    const float qxm = qx + midx, yc = -midy - qy;
    const float hi_lim = (float)(Nxx - 1);
    const float t_c = RE - ddx * midx - ddy * midy;
    const float s_c = -dx * midx - dy * midy;
    int y0, y1;
    row_range(fmaf(dmx, yc, qxm), dmx, fmaf(dpx, yc, qxm), dpx, hi_lim, Nyy, y0, y1);
    const int ys = y0 + L.lane_group;
    float yf = (float)ys;
    for (int y = ys; y <= y1; y += SPLIT, yf += (float)SPLIT) {
      const float yrel = yf + yc;
      const int xhi = (int)floorf(fminf(hi_lim, fmaf(dpx, yrel, qxm)));
      const int xlo = (int)ceilf(fmaxf(0.0f, fmaf(dmx, yrel, qxm)));
      const float xlf = (float)xlo;
      float t = fmaf(ddx, xlf, fmaf(ddy, yf, t_c));
      float ss = fmaf(dx, xlf, fmaf(dy, yf, s_c));
      const Off stp = (Off)step_x;
      Off o0 = (Off)(y * step_y + xlo * step_x);
      Off oM = MIRROR ? (Off)(Mbase + y * Mstep_y + xlo * Mstep_x) : 0;
      Off om[kOrbit - 1];
      if constexpr (!PIX4) {
#pragma unroll
        for (int m = 0; m < kOrbit - 1; ++m) om[m] = mbase[m] + y * mstep_y[m] + xlo * mstep_x[m];
      }
      if constexpr (PIX4) {
        // two candidates per trip, both loads in flight (one per trip
        // measured 1115 instead of 1181 Gpixel-angle/s at 512^2 x 360); the
        // second of an odd count is masked (its reciprocal set to zero adds
        // zeros).  t and ss advance by the same additions as one candidate
        // per trip.
        if constexpr (MIRROR) {
          // one candidate per trip: its two loads (P and M P) in flight and
          // 80 registers unbounded instead of 94 (two per trip: 512^2 x 360
          // equal, 1024^2 x 720 387.5 against 382.2 us, 2048^2 x 1440 2618
          // against 2592 us); the same sums bit for bit.  The kernel's
          // launch bounds now hold the 32-lane form to 72.
          for (int x = xlo; x <= xhi; ++x) {
            const float4 pa = __ldg(img4 + o0);
            const float4 qa = __ldg(img4 + oM);
            const float ra = rcp_approx(t);
            const float ua = fmaf(ss, ra, -s_mid0);
            const float2 ra2 = make_float2(ra, ra);
            const float2 a01 = __fmul2_rn(make_float2(pa.x, pa.y), ra2);
            const float2 a23 = __fmul2_rn(make_float2(pa.z, pa.w), ra2);
            const float2 ma01 = __fmul2_rn(make_float2(qa.x, qa.y), ra2);
            const float2 ma23 = __fmul2_rn(make_float2(qa.z, qa.w), ra2);
#pragma unroll
            for (int q = 0; q < kRayGroup; ++q) {
              const float wa = hat_weight(ua - (float)q);
              const float2 wa2 = make_float2(wa, wa);
              acc01[q] = __ffma2_rn(wa2, a01, acc01[q]);
              acc23[q] = __ffma2_rn(wa2, a23, acc23[q]);
              macc01[q] = __ffma2_rn(wa2, ma01, macc01[q]);
              macc23[q] = __ffma2_rn(wa2, ma23, macc23[q]);
            }
            o0 += stp;
            oM += Mstep_x;
            t += ddx;
            ss += dx;
          }
        } else
        for (int x = xlo; x <= xhi; x += 2) {
          const bool two = x < xhi;
          const float tb = t + ddx, sb = ss + dx;
          const float4 pa = __ldg(img4 + o0);
          const float4 pb = __ldg(img4 + (two ? o0 + stp : o0));
          const float ra = rcp_approx(t);
          const float rb = two ? rcp_approx(tb) : 0.0f;
          const float ua = fmaf(ss, ra, -s_mid0), ub = fmaf(sb, rb, -s_mid0);
          const float2 ra2 = make_float2(ra, ra), rb2 = make_float2(rb, rb);
          const float2 a01 = __fmul2_rn(make_float2(pa.x, pa.y), ra2);
          const float2 a23 = __fmul2_rn(make_float2(pa.z, pa.w), ra2);
          const float2 b01 = __fmul2_rn(make_float2(pb.x, pb.y), rb2);
          const float2 b23 = __fmul2_rn(make_float2(pb.z, pb.w), rb2);
          float2 ma01, ma23, mb01, mb23;
          if constexpr (MIRROR) {
            const float4 qa = __ldg(img4 + oM);
            const float4 qb = __ldg(img4 + (two ? oM + Mstep_x : oM));
            ma01 = __fmul2_rn(make_float2(qa.x, qa.y), ra2);
            ma23 = __fmul2_rn(make_float2(qa.z, qa.w), ra2);
            mb01 = __fmul2_rn(make_float2(qb.x, qb.y), rb2);
            mb23 = __fmul2_rn(make_float2(qb.z, qb.w), rb2);
            oM += 2 * Mstep_x;
          }
#pragma unroll
          for (int q = 0; q < kRayGroup; ++q) {
            const float wa = hat_weight(ua - (float)q);
            const float wb = hat_weight(ub - (float)q);
            const float2 wa2 = make_float2(wa, wa), wb2 = make_float2(wb, wb);
            acc01[q] = __ffma2_rn(wb2, b01, __ffma2_rn(wa2, a01, acc01[q]));
            acc23[q] = __ffma2_rn(wb2, b23, __ffma2_rn(wa2, a23, acc23[q]));
            if constexpr (MIRROR) {
              macc01[q] = __ffma2_rn(wb2, mb01, __ffma2_rn(wa2, ma01, macc01[q]));
              macc23[q] = __ffma2_rn(wb2, mb23, __ffma2_rn(wa2, ma23, macc23[q]));
            }
          }
          o0 += 2 * stp;
          t = tb + ddx;
          ss = sb + dx;
        }
      } else {
      for (int x = xlo; x <= xhi; ++x) {
        const float r = rcp_approx(t);
        const float u = fmaf(ss, r, -s_mid0);
        const float2 r2 = make_float2(r, r);
        const float2 v01 = __fmul2_rn(make_float2(ldg(img + o0), ldg(img + om[0])), r2);
        const float2 v23 = __fmul2_rn(make_float2(ldg(img + om[1]), ldg(img + om[2])), r2);
        // hat weights, zero outside a bin's pair of neighbouring rays: the
        // multiply-add of a zero weight leaves the sum unchanged, so no branch
#pragma unroll
        for (int q = 0; q < kRayGroup; ++q) {
          const float w = hat_weight(u - (float)q);
          const float2 w2 = make_float2(w, w);
          acc01[q] = __ffma2_rn(w2, v01, acc01[q]);
          acc23[q] = __ffma2_rn(w2, v23, acc23[q]);
        }
        o0 += stp;
#pragma unroll
        for (int m = 0; m < kOrbit - 1; ++m) om[m] += mstep_x[m];
        t += ddx;
        ss += dx;
      }
      }
    }
  }
  constexpr int kOut = MIRROR ? 2 * kOrbit : kOrbit;
  float acc[kOut][kRayGroup];
#pragma unroll
  for (int q = 0; q < kRayGroup; ++q) {
    acc[0][q] = acc01[q].x;
    acc[1][q] = acc01[q].y;
    acc[2][q] = acc23[q].x;
    acc[3][q] = acc23[q].y;
    if constexpr (MIRROR) {
      acc[4][q] = macc01[q].x;
      acc[5][q] = macc01[q].y;
      acc[6][q] = macc23[q].x;
      acc[7][q] = macc23[q].y;
    }
  }
  if (SPLIT > 1) {
#pragma unroll
    for (int m = 0; m < kOut; ++m) warp_reduce_rows<SPLIT>(acc[m]);
  }
  // every lane of the group now holds every sum: the lanes share the
  // group's outputs, one each per round
  constexpr int kN = kOut * kRayGroup;
  static_assert(kN % SPLIT == 0 || SPLIT > kN, "whole rounds of outputs");
  double part = 0.0;
  if (active) {
    const int64_t mirror_max = d.Ns - 1 - Hs;  // mirrored outputs for s <= this
#pragma unroll
    for (int base = 0; base < kN; base += SPLIT) {
      const int oi = base + L.lane_group;
      const float v = pick_output<kOut, kRayGroup>(acc, oi);
      const int m = oi / kRayGroup;
      const int64_t s = s0 + oi % kRayGroup;
      // component k = m - 4 of the entry at M P is member -k mod 4: the
      // output (Ns - 1 - s, c0 - (a + ((-k + shift) mod 4) Q))
      const bool mir = MIRROR && m >= kOrbit;
      const int mm = mir ? (kOrbit - (m - kOrbit)) & (kOrbit - 1) : m;
      const int64_t am = a + ((mm + shift) & (kOrbit - 1)) * quarter;
      int64_t bin = s, ang = am;
      if (mir) {
        bin = d.Ns - 1 - s;
        ang = qm.mirror_pair - am;
        if (ang < 0) ang += d.Na;
      }
      if (oi < kN && s < Hs && (!mir || s <= mirror_max)) {
        const float sc = sdpd[bin] / g.delta_xi * g.delta_x / R;
        part += epi(bin, ang, z, sino_index<SO>(bin, ang, z, d), v * sc);
      }
    }
  }
  return part;
}

// The four pixels a candidate of the orbit-sharing forward projection loads,
// as one float4 per pixel: img4[x + Nx y] = (img(P), img(M_1 P), img(M_2 P),
// img(M_3 P)) for P = (x, y) and the quarter-turn index maps M_m; slice
// z0 + blockIdx.z goes to copy blockIdx.z.
template <int IO>
__global__ void __launch_bounds__(256)
orbit_pixels(const float* __restrict__ img, Dims d, QuarterMaps qm, float4* __restrict__ img4,
             int64_t z0, const int* __restrict__ skip) {
  pdl_wait();
  pdl_trigger();
  if (skip != nullptr && *skip) return;
  const int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t y = blockIdx.y;
  const int64_t z = z0 + blockIdx.z;
  if (x >= d.Nx) return;
  float v[4];
  v[0] = ldg(img + img_index<IO>(x, y, z, d));
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    const int64_t mx = qm.cx[m] + qm.axx[m] * x + qm.axy[m] * y;
    const int64_t my = qm.cy[m] + qm.ayx[m] * x + qm.ayy[m] * y;
    v[m + 1] = ldg(img + img_index<IO>(mx, my, z, d));
  }
  img4[((int64_t)blockIdx.z * d.Ny + y) * d.Nx + x] = make_float4(v[0], v[1], v[2], v[3]);
}

// orbit_pixels for x-fastest (F-ordered) images: a block of 32 x 32 threads
// copies a 32 x 32 tile of P; the tile's three turned images are 32 x 32
// squares elsewhere in the slice, read row by row (coalesced) into shared
// memory and picked from there, so no global read walks down a column.
constexpr int kOrbitTile = 32;

template <int IO>
__global__ void __launch_bounds__(kOrbitTile * kOrbitTile)
orbit_pixels_tiled(const float* __restrict__ img, Dims d, QuarterMaps qm,
                   float4* __restrict__ img4, int64_t z0, const int* __restrict__ skip) {
  static_assert(IO == ORDER_F, "x-fastest images only");
  __shared__ float tile[3][kOrbitTile][kOrbitTile + 1];
  pdl_wait();
  pdl_trigger();
  if (skip != nullptr && *skip) return;
  // offsets within a slice in 32 bits (the orbit kernels' slices hold fewer
  // than 2^31 pixels): a quarter of the 64-bit form's index arithmetic
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int X0 = (int)blockIdx.x * kOrbitTile, Y0 = (int)blockIdx.y * kOrbitTile;
  const int Nx = (int)d.Nx, Ny = (int)d.Ny;
  const float* slice = img + (z0 + blockIdx.z) * (int64_t)Nx * Ny;
  int rx0[3], ry0[3];
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    // the turned tile: the images of two opposite corners bound it
    const int ax = qm.cx[m] + qm.axx[m] * X0 + qm.axy[m] * Y0;
    const int ay = qm.cy[m] + qm.ayx[m] * X0 + qm.ayy[m] * Y0;
    const int bx = ax + (qm.axx[m] + qm.axy[m]) * (kOrbitTile - 1);
    const int by = ay + (qm.ayx[m] + qm.ayy[m]) * (kOrbitTile - 1);
    rx0[m] = ax < bx ? ax : bx;
    ry0[m] = ay < by ? ay : by;
    const int x = rx0[m] + tx, y = ry0[m] + ty;
    if (x >= 0 && x < Nx && y >= 0 && y < Ny) tile[m][ty][tx] = ldg(slice + x + Nx * y);
  }
  const int x = X0 + tx, y = Y0 + ty;
  const bool in = x < Nx && y < Ny;
  const float v0 = in ? ldg(slice + x + Nx * y) : 0.0f;
  __syncthreads();
  if (!in) return;
  float v[3];
#pragma unroll
  for (int m = 0; m < 3; ++m) {
    const int mx = qm.cx[m] + qm.axx[m] * x + qm.axy[m] * y;
    const int my = qm.cy[m] + qm.ayx[m] * x + qm.ayy[m] * y;
    v[m] = tile[m][my - ry0[m]][mx - rx0[m]];
  }
  img4[(int64_t)blockIdx.z * Nx * Ny + (y * Nx + x)] = make_float4(v0, v[0], v[1], v[2]);
}

// The four sinogram rows of every quarter-turn orbit of angles, premultiplied
// by sdpd, as one float4 per (base angle, bin), with one zero entry before
// the detector and two after it: row a holds at 1 + s the float4
// sdpd[s] (sino[s, a], sino[s, a + Q], sino[s, a + 2Q], sino[s, a + 3Q]),
// Q = Na / 4, so a backprojection that clamps its interpolation position to
// [-1, Ns] reads zeros off the detector without testing the bins.  (Entries
// holding both taps of a position, 32 bytes read by one load, measured
// slower: twice the footprint, L1 hit rate 63% -> 22%.)  Lanes run along the
// bins (coalesced for F-ordered sinograms); slice z0 + blockIdx.z goes to
// copy blockIdx.z.
constexpr int kOrbitRowPad = 3;  // entries per row: Ns + kOrbitRowPad
constexpr int kOrbitRec = 4;     // float4 per base angle in the record table

// Per-base-angle record of the orbit backprojection, as broadcast pairs for
// the packed arithmetic: (ddx, ddx, ddy, ddy), (tz, tz, dx, dx),
// (dy, dy, sz, sz), (w0, w1, w2, w3) with t = ddx X + ddy Y + tz and
// s = dx X + dy Y + sz for pixel centres (X, Y) relative to the image
// midpoint (source offset folded into tz and sz), and w_j the angle weight
// of row a + j Q divided by R.
__device__ __forceinline__ void orbit_record(float4* __restrict__ rec, const float* __restrict__ ofs,
                                             const FanGeo<float>& gg, int64_t a, int64_t Q) {
  const float R = gg.R;
  const float R_sqr_inv = 1.0f / (R * R);
  const float dxi_sqr_inv = 1.0f / (gg.delta_xi * gg.delta_xi);
  const float* o = ofs + 8 * a;
  const float qx = ldg(o + 2), qy = ldg(o + 3);
  const float ddx = (ldg(o + 4) - qx) * R_sqr_inv, ddy = (ldg(o + 5) - qy) * R_sqr_inv;
  const float dx = ldg(o) * dxi_sqr_inv, dy = ldg(o + 1) * dxi_sqr_inv;
  const float tz = -fmaf(ddx, qx, ddy * qy), sz = -fmaf(dx, qx, dy * qy);
  rec[0] = make_float4(ddx, ddx, ddy, ddy);
  rec[1] = make_float4(tz, tz, dx, dx);
  rec[2] = make_float4(dy, dy, sz, sz);
  rec[3] = make_float4(ldg(ofs + 8 * a + 6) / R, ldg(ofs + 8 * (a + Q) + 6) / R,
                       ldg(ofs + 8 * (a + 2 * Q) + 6) / R, ldg(ofs + 8 * (a + 3 * Q) + 6) / R);
}

// Each slice's copy: Q rows of Ns + kOrbitRowPad float4, then the Q base
// angles' records (kOrbitRec float4 each), written by the last column of
// blocks.
template <int SO>
__global__ void __launch_bounds__(256)
orbit_rows(const float* __restrict__ sino, const float* __restrict__ sdpd,
           const float* __restrict__ ofs, FanGeo<float> gg, Dims d, float4* __restrict__ rows4,
           int64_t z0, const int* __restrict__ skip) {
  pdl_wait();
  pdl_trigger();
  if (skip != nullptr && *skip) return;
  const int64_t a = blockIdx.y;
  const int64_t nrow = d.Ns + kOrbitRowPad;
  const int64_t Q = d.Na / 4;
  float4* copy = rows4 + (int64_t)blockIdx.z * Q * (nrow + kOrbitRec);
  if (blockIdx.x == gridDim.x - 1) {
    if (threadIdx.x == 0) orbit_record(copy + Q * nrow + kOrbitRec * a, ofs, gg, a, Q);
    return;
  }
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;  // padded position
  if (e >= nrow) return;
  const int64_t s = e - 1;
  float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
  if (s >= 0 && s < d.Ns) {
    int64_t ss_, sa_, sz_;
    sino_strides<SO>(d, ss_, sa_, sz_);
    const float* p = sino + s * ss_ + a * sa_ + (z0 + blockIdx.z) * sz_;
    const float w = ldg(sdpd + s);
    v = make_float4(w * ldg(p), w * ldg(p + Q * sa_), w * ldg(p + 2 * Q * sa_),
                    w * ldg(p + 3 * Q * sa_));
  }
  copy[a * nrow + e] = v;
}

// The epilogue of an orbit backprojection, whose thread owns the four pixels
// of an orbit: with G > 1 angle groups the groups' sums meet in shared
// memory and group j finishes members j, j + G, ... (each member's sum added
// in the fixed group order), so up to four members' epilogues -- and their
// loads -- run on different threads at once instead of one after another on
// the first group's thread.  pixel(k, x, y) gives member k's pixel.
template <int IO, int G, class Epi, class Pix>
__device__ __forceinline__ double orbit_epilogue(const float (&sum)[4], bool own, Pix pixel,
                                                 const Epi& epi, int64_t z, const Dims& d) {
  constexpr int kOrbit = 4;
  constexpr int kRowsT = kBwdTileSlow / G;
  const int lane = threadIdx.x, trow = threadIdx.y;
  double part = 0.0;
  if constexpr (G > 1) {
    const int grp = trow / kRowsT, trow_t = trow % kRowsT;
    __shared__ float cred[kBwdTileSlow][kOrbit][kBwdTileFast];
#pragma unroll
    for (int k = 0; k < kOrbit; ++k) cred[trow][k][lane] = sum[k];
    __syncthreads();
#pragma unroll
    for (int k0 = 0; k0 < kOrbit; k0 += G) {
      const int k = k0 + grp;
      if (own && k < kOrbit) {
        float t = cred[trow_t][k][lane];
#pragma unroll
        for (int q = 1; q < G; ++q) t += cred[trow_t + q * kRowsT][k][lane];
        int x, y;
        pixel(k, x, y);
        part += epi(x, y, z, img_index<IO>(x, y, z, d), t);
      }
    }
  } else {
    if (own) {
#pragma unroll
      for (int k = 0; k < kOrbit; ++k) {
        int x, y;
        pixel(k, x, y);
        part += epi(x, y, z, img_index<IO>(x, y, z, d), sum[k]);
      }
    }
  }
  return part;
}

// Member k of four pixels held in arrays, by selects (no local memory).
__device__ __forceinline__ void pick_pixel(const int (&ox)[4], const int (&oy)[4], int k, int& x,
                                           int& y) {
  x = ox[0];
  y = oy[0];
#pragma unroll
  for (int m = 1; m < 4; ++m) {
    x = k == m ? ox[m] : x;
    y = k == m ? oy[m] : y;
  }
}

// Backprojection over quarter-turn pixel orbits.  With the maps powers of
// one quarter turn A (A_m = A^m about the image centre, N even) the pixels
// P_k = A^k P_0 satisfy u(a + j Na/4, P_k) = u(a, P_{k-j mod 4}) for the
// detector coordinate and the distance weight alike.  A thread owns the
// orbit of one pixel P_0 of the quadrant x, y < N/2: for a base angle a in
// [0, Na/4) it evaluates the geometry of its four pixels once and applies
// each to the four sinogram rows a + j Na/4, i.e. one reciprocal, one floor
// and two sdpd loads serve four pixel-angles.  The sinogram values are read
// directly (the rows of the four angles are L1/L2 resident; no staging, no
// barrier in the angle loop).  The G thread groups of a block take
// interleaved base angles and are added in a fixed order at the end.  This
// form runs without scratch; fan_bwd_orbit_rows below reads the row copy.
// The tile of block `bid` (32 x 8 threads) on slice z; returns the thread's
// share of the block's reduction.
template <int IO, int SO, int G, class Epi>
__device__ __forceinline__ double fan_bwd_orbit_tile(const float* __restrict__ sino,
                                                     const float* __restrict__ ofs,
                                                     const float* __restrict__ sdpd,
                                                     FanGeo<float> gg, Dims d, QuarterMaps qm,
                                                     Epi epi, uint3 bid, int64_t z) {
  constexpr int kOrbit = 4;
  constexpr int kRowsT = kBwdTileSlow / G;  // quadrant rows of the block tile
  const int lane = threadIdx.x, trow = threadIdx.y;
  const int grp = trow / kRowsT, trow_t = trow % kRowsT;
  const int half = (int)(d.Nx / 2);
  const int Q = (int)(d.Na / kOrbit);
  const int px0 = (int)bid.x * kBwdTileFast + lane;
  const int py0 = (int)bid.y * kRowsT + trow_t;
  const bool own = px0 < half && py0 < half;
  int ox[kOrbit], oy[kOrbit];
  ox[0] = px0;
  oy[0] = py0;
#pragma unroll
  for (int m = 0; m < kOrbit - 1; ++m) {
    ox[m + 1] = qm.cx[m] + qm.axx[m] * px0 + qm.axy[m] * py0;
    oy[m + 1] = qm.cy[m] + qm.ayx[m] * px0 + qm.ayy[m] * py0;
  }
  float pxs[kOrbit], pys[kOrbit];
#pragma unroll
  for (int i = 0; i < kOrbit; ++i) {
    pxs[i] = (float)ox[i] - gg.midx;
    pys[i] = (float)oy[i] - gg.midy;
  }
  const float R = gg.R;
  const float R_sqr_inv = 1.0f / (R * R);
  const float dxi_sqr_inv = 1.0f / (gg.delta_xi * gg.delta_xi);
  const float mid_det = gg.mid_det;
  int64_t ss_, sa_, sz_;
  sino_strides<SO>(d, ss_, sa_, sz_);
  // slice z of the sinogram (and its row copy); offsets within an F-ordered
  // slice are 32-bit, C-ordered slices interleave
  using Off = typename std::conditional<SO == ORDER_C, int64_t, int>::type;
  const Off ss = (Off)ss_, sa = (Off)sa_;
  sino += z * sz_;
  const int Ns = (int)d.Ns;
  float acc[kOrbit];
#pragma unroll
  for (int k = 0; k < kOrbit; ++k) acc[k] = 0.0f;
  // angle weight / R of the rows a + j Q, rounded as the reference does (a
  // reciprocal multiply would move every weight by up to an ulp in the same
  // direction, which CG amplifies): lane 4k + j divides for the k-th of the
  // next 8 base angles of this group, the values reach the other lanes by
  // shuffle (a warp shares its thread row, hence its group)
  float wdiv = 0.0f;
  int chunk = 0;
  for (int a = grp; a < Q; a += G, ++chunk) {
    if ((chunk & 7) == 0) {
      const int ak = a + (lane >> 2) * G;
      wdiv = ak < Q ? ldg(ofs + 8 * (ak + (lane & 3) * Q) + 6) / R : 0.0f;
    }
    const float* o = ofs + 8 * a;
    const float qx = ldg(o + 2), qy = ldg(o + 3);
    const float ddx = (ldg(o + 4) - qx) * R_sqr_inv, ddy = (ldg(o + 5) - qy) * R_sqr_inv;
    const float dx = ldg(o) * dxi_sqr_inv, dy = ldg(o + 1) * dxi_sqr_inv;
    const float tz = -fmaf(ddx, qx, ddy * qy), sz = -fmaf(dx, qx, dy * qy);
    float wj[kOrbit];
    const float* row[kOrbit];
#pragma unroll
    for (int j = 0; j < kOrbit; ++j) {
      wj[j] = __shfl_sync(0xffffffffu, wdiv, ((chunk & 7) << 2) + j);
      row[j] = sino + (a + j * Q) * sa;
    }
#pragma unroll
    for (int i = 0; i < kOrbit; ++i) {
      const float t = fmaf(ddx, pxs[i], fmaf(ddy, pys[i], tz));
      const float s = fmaf(dx, pxs[i], fmaf(dy, pys[i], sz));
      const float inv = rcp_approx(t);
      const float xi = fmaf(s, inv, mid_det);
      const float fl = floorf(xi);
      const float fr = xi - fl;
      const int xm = (int)fl;
      // bins outside the detector contribute nothing; their reads go to bin 0
      const bool okm = (unsigned)xm < (unsigned)Ns;
      const bool okp = (unsigned)(xm + 1) < (unsigned)Ns;
      const int im = okm ? xm : 0, ip = okp ? xm + 1 : 0;
      const float Wm = okm ? (1.0f - fr) * inv * ldg(sdpd + im) : 0.0f;
      const float Wp = okp ? fr * inv * ldg(sdpd + ip) : 0.0f;
#pragma unroll
      for (int j = 0; j < kOrbit; ++j) {
        const float v = fmaf(Wp, ldg(row[j] + ip * ss), Wm * ldg(row[j] + im * ss));
        acc[(i + j) % kOrbit] = fmaf(wj[j], v, acc[(i + j) % kOrbit]);
      }
    }
  }
  // fixed-order combination of the G angle groups, and the epilogue
  return orbit_epilogue<IO, G>(
      acc, own, [&](int k, int& x, int& y) { pick_pixel(ox, oy, k, x, y); }, epi, z, d);
}

template <int IO, int SO, int G, class Epi>
__global__ void __launch_bounds__(kBwdTileFast * kBwdTileSlow)
fan_bwd_orbit(const float* __restrict__ sino, const float* __restrict__ ofs,
              const float* __restrict__ sdpd, FanGeo<float> gg, Dims d, QuarterMaps qm, Epi epi,
              double* __restrict__ partials, const int* __restrict__ skip, int64_t z0) {
  __shared__ double red[32];
  pdl_wait();
  pdl_trigger();
  if (skip != nullptr && *skip) return;
  const double part = fan_bwd_orbit_tile<IO, SO, G, Epi>(sino, ofs, sdpd, gg, d, qm, epi,
                                                         blockIdx, z0 + blockIdx.z);
  if (Epi::kReduce) {
    const double t = block_sum(part, red);
    if (threadIdx.x + blockDim.x * threadIdx.y == 0) partials[bid_linear()] = t;
  }
}

// Backprojection over quarter-turn pixel orbits from the padded row copy
// (orbit_rows): same orbit decomposition as fan_bwd_orbit, restructured to
// issue fewer instructions per pixel-angle.
//  * Each base angle's geometry comes from the copy's record table (four
//    16-byte loads that every lane of a warp shares: the G thread groups
//    take interleaved base angles, one angle per warp at a time; computed
//    once per block into shared memory instead, the records' prologue and
//    barriers measured slower).
//  * Interpolation positions are clamped to [-1, Ns] (padded [0, Ns + 1]),
//    where the copy holds zeros, instead of testing both bins.
//  * Pairs of values go through Blackwell's packed float32 arithmetic
//    (__ffma2_rn and friends: two lanes of one 64-bit register pair per
//    instruction): t and s of two orbit pixels at once, and the four rows'
//    interpolation and weighting as two pairs.  Pixel i's geometry applied to
//    row j adds to pixel (i + j) mod 4: even i add to the pairs (0, 1) and
//    (2, 3), odd i to the pairs (1, 2) and (3, 0), and the two pair sets are
//    added at the end.
// Every value is rounded as in fan_bwd_orbit: t = ddx x + (ddy y + tz),
// s likewise, xi = s / t + midpoint, weights (1 - fr) / t and fr / t, the
// angle weight / R by division.  (Owning the eight-pixel orbits of the
// geometry's mirror as well -- the mirrored rows in a second plane of the
// copy, the quadrant's pixels x <= y -- measured slower: 512^2 x 360 77.2
// against 68.2 us, 2048^2 x 1440 3001 against 2620 us; the same L1 bytes per
// pixel-angle from half the threads, each with twice the footprint.)
//
// MINB: the minimum resident blocks per SM the registers are fitted to (1:
// the compiler's choice, 64 registers; 5: 48 registers, which the launch
// picks where it measured faster).
template <int IO, int G, int MINB, class Epi>
__global__ void __launch_bounds__(kBwdTileFast * kBwdTileSlow, MINB)
fan_bwd_orbit_rows(const float4* __restrict__ rows4, FanGeo<float> gg, Dims d, QuarterMaps qm,
                   Epi epi, double* __restrict__ partials, const int* __restrict__ skip,
                   int64_t z0) {
  constexpr int kOrbit = 4;
  constexpr int kRowsT = kBwdTileSlow / G;  // quadrant rows of the block tile
  __shared__ double red[32];
  pdl_wait();
  pdl_trigger();
  if (skip != nullptr && *skip) return;
  const int lane = threadIdx.x, trow = threadIdx.y;
  const int grp = trow / kRowsT, trow_t = trow % kRowsT;
  const int half = (int)(d.Nx / 2);
  const int Q = (int)(d.Na / kOrbit);
  const int nrow = (int)d.Ns + kOrbitRowPad;
  const int px0 = (int)blockIdx.x * kBwdTileFast + lane;
  const int py0 = (int)blockIdx.y * kRowsT + trow_t;
  const bool own = px0 < half && py0 < half;
  // the orbit's pixels (recomputed for the epilogue rather than kept live)
  auto orbit = [&](int (&ox)[kOrbit], int (&oy)[kOrbit]) {
    ox[0] = px0;
    oy[0] = py0;
#pragma unroll
    for (int m = 0; m < kOrbit - 1; ++m) {
      ox[m + 1] = qm.cx[m] + qm.axx[m] * px0 + qm.axy[m] * py0;
      oy[m + 1] = qm.cy[m] + qm.ayx[m] * px0 + qm.ayy[m] * py0;
    }
  };
  float2 pxa, pxb, pya, pyb;  // pixel centres relative to the image midpoint
  {
    int ox[kOrbit], oy[kOrbit];
    orbit(ox, oy);
    pxa = make_float2((float)ox[0] - gg.midx, (float)ox[1] - gg.midx);
    pxb = make_float2((float)ox[2] - gg.midx, (float)ox[3] - gg.midx);
    pya = make_float2((float)oy[0] - gg.midy, (float)oy[1] - gg.midy);
    pyb = make_float2((float)oy[2] - gg.midy, (float)oy[3] - gg.midy);
  }
  // position in the padded row: detector position + 1
  const float2 mid2 = make_float2(gg.mid_det + 1.0f, gg.mid_det + 1.0f);
  const float hi = (float)d.Ns + 1.0f;
  const int64_t z = z0 + blockIdx.z;
  rows4 += (int64_t)blockIdx.z * Q * (nrow + kOrbitRec);
  const float4* recs = rows4 + (int64_t)Q * nrow;
  // sums of pixels (0, 1), (2, 3) [even geometry] and (1, 2), (3, 0) [odd]
  float2 e01 = make_float2(0.f, 0.f), e23 = e01, o12 = e01, o30 = e01;
  for (int a = grp; a < Q; a += G) {
    const float4* rc = recs + kOrbitRec * a;
    const float4 r0 = __ldg(rc), r1 = __ldg(rc + 1), r2 = __ldg(rc + 2), r3 = __ldg(rc + 3);
    const float2 ddx = make_float2(r0.x, r0.y), ddy = make_float2(r0.z, r0.w);
    const float2 tz = make_float2(r1.x, r1.y), dx = make_float2(r1.z, r1.w);
    const float2 dy = make_float2(r2.x, r2.y), sz = make_float2(r2.z, r2.w);
    const float2 wlo = make_float2(r3.x, r3.y), whi = make_float2(r3.z, r3.w);
    const float4* row = rows4 + a * nrow;
    float2 t[2], s[2];
    t[0] = __ffma2_rn(ddx, pxa, __ffma2_rn(ddy, pya, tz));
    t[1] = __ffma2_rn(ddx, pxb, __ffma2_rn(ddy, pyb, tz));
    s[0] = __ffma2_rn(dx, pxa, __ffma2_rn(dy, pya, sz));
    s[1] = __ffma2_rn(dx, pxb, __ffma2_rn(dy, pyb, sz));
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const float2 inv = make_float2(rcp_approx(t[h].x), rcp_approx(t[h].y));
      const float2 xi = __ffma2_rn(s[h], inv, mid2);
      const float xc[2] = {fminf(fmaxf(xi.x, 0.0f), hi), fminf(fmaxf(xi.y, 0.0f), hi)};
      const float iv[2] = {inv.x, inv.y};
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int i = 2 * h + e;
        const float fl = floorf(xc[e]);
        const float fr = xc[e] - fl;
        const int xm = (int)fl;
        const float wm = (1.0f - fr) * iv[e], wp = fr * iv[e];
        const float2 Wm = make_float2(wm, wm), Wp = make_float2(wp, wp);
        const float4 vm = __ldg(row + xm);
        const float4 vp = __ldg(row + xm + 1);
        const float2 vlo = __ffma2_rn(Wp, make_float2(vp.x, vp.y),
                                      __fmul2_rn(Wm, make_float2(vm.x, vm.y)));
        const float2 vhi = __ffma2_rn(Wp, make_float2(vp.z, vp.w),
                                      __fmul2_rn(Wm, make_float2(vm.z, vm.w)));
        // rows (0, 1) go to pixels (i, i + 1), rows (2, 3) to (i + 2, i + 3)
        if (i == 0) {
          e01 = __ffma2_rn(wlo, vlo, e01);
          e23 = __ffma2_rn(whi, vhi, e23);
        } else if (i == 1) {
          o12 = __ffma2_rn(wlo, vlo, o12);
          o30 = __ffma2_rn(whi, vhi, o30);
        } else if (i == 2) {
          e23 = __ffma2_rn(wlo, vlo, e23);
          e01 = __ffma2_rn(whi, vhi, e01);
        } else {
          o30 = __ffma2_rn(wlo, vlo, o30);
          o12 = __ffma2_rn(whi, vhi, o12);
        }
      }
    }
  }
  float sum[kOrbit] = {e01.x + o30.y, e01.y + o12.x, e23.x + o12.y, e23.y + o30.x};
  // fixed-order combination of the G angle groups, and the epilogue
  const double part = orbit_epilogue<IO, G>(
      sum, own,
      [&](int k, int& x, int& y) {
        int ox[kOrbit], oy[kOrbit];
        orbit(ox, oy);
        pick_pixel(ox, oy, k, x, y);
      },
      epi, z, d);
  if (Epi::kReduce) {
    const double t = block_sum(part, red);
    if (threadIdx.x + blockDim.x * threadIdx.y == 0) partials[bid_linear()] = t;
  }
}

// ------------------------------------------ parallel beam: half-circle orbits
// For Na angles equispaced over [0, pi) (Na even), a square image centred on
// the rotation axis and a detector centred on the central ray, angle
// k + Na/2 sees the grid as angle k sees it after a quarter turn S, and
// angle k sees the grid turned by a half with its detector reversed
// (p(-s, phi) = p(s, phi + pi)).  With Q = Na/2 and s' = Ns - 1 - s the four
// outputs of the cycle
//   c = 0: (s, k)   c = 1: (s, k + Q)   c = 2: (s', k)   c = 3: (s', k + Q)
// are the weights of angle k applied to img(P), img(S^-1 P), img(-P) and
// img(-S^-1 P): the orbit copy of orbit_pixels with the maps
// (S^-1, -I, -S^-1).  Detected on the host (gratopy_gb300/symmetry.py).

__device__ __forceinline__ int radon_orbit_half(int64_t Ns) { return (int)((Ns + 1) / 2); }

// Forward over the orbits: a lane group owns kRayGroup adjacent bins s < H =
// ceil(Ns/2) of base angle k < Q and writes the 16 outputs of their cycles
// (the mirrored bins s' only where s' >= H, so the middle bin of an odd
// detector is written once).  A group walks the cycle member (k or k + Q,
// rays turned by a quarter) whose detector coordinate changes faster along
// the image's y axis: its lanes then take adjacent image columns and walk
// down them, so a load instruction reads adjacent pixels of the orbit copy.
// Two candidates per trip, packed pair sums, branch-free hat weights, as in
// fan_fwd_quarter.  PIX4: the four members of a pixel's orbit come from the
// orbit copy (one 16-byte load); otherwise from the slice `img` itself
// through the maps (four loads).  ZS = 2 (with the copy): slices z and z + 1
// at once, the second slice's copy following the first's; a candidate's
// four hat weights then serve both slices' members, one candidate per trip.
template <int SO, int IO, int SPLIT, bool PIX4, int ZS, class Epi>
__device__ __forceinline__ double radon_fwd_quarter_tile(const float* __restrict__ img,
                                                         const float4* __restrict__ img4,
                                                         const float* __restrict__ ofs,
                                                         RadonGeo<float> g, Dims d,
                                                         QuarterMaps qm, Epi epi, uint3 bid,
                                                         int64_t z) {
  constexpr int kOrbit = 4;
  static_assert(ZS == 1 || (ZS == 2 && PIX4), "two slices from the orbit copies");
  const QuarterLayout<SPLIT> L(bid);
  const int64_t s0 = L.s0;
  const int64_t k = L.a;
  const int64_t Q = d.Na / 2;
  const int H = radon_orbit_half(d.Ns);
  const bool active = s0 < H && k < Q;
  float2 acc01[kRayGroup], acc23[kRayGroup];
  float2 zacc01[ZS == 2 ? kRayGroup : 1], zacc23[ZS == 2 ? kRayGroup : 1];  // slice z + 1
#pragma unroll
  for (int q = 0; q < kRayGroup; ++q) acc01[q] = acc23[q] = make_float2(0.0f, 0.0f);
#pragma unroll
  for (int q = 0; q < (ZS == 2 ? kRayGroup : 1); ++q) zacc01[q] = zacc23[q] = make_float2(0.f, 0.f);
  int shift = 0;
  if (active) {
    int64_t ab = k;
    if (fabsf(ofs[8 * k + 1]) < fabsf(ofs[8 * k])) {  // walk the member turned by a quarter
      ab = k + Q;
      shift = 1;
    }
    const float X = ofs[8 * ab], Y = ofs[8 * ab + 1];
    const float base = ofs[8 * ab + 2] - (float)(int)s0;  // xi - s0 = X x + Y y + base
    const int N = (int)d.Nx;
    const float yinv = 1.0f / Y;
    // candidate y of column x: pos = xi - s0 in (-1, kRayGroup), i.e. y between
    // lo(x) = alo + bx x and hi(x) = ahi + bx x
    const float c_lo = yinv > 0.0f ? -1.0f : (float)kRayGroup;
    const float c_hi = yinv > 0.0f ? (float)kRayGroup : -1.0f;
    const float bx = -X * yinv;
    const float alo = (c_lo - base) * yinv, ahi = (c_hi - base) * yinv;
    int x0, x1;
    row_range(alo, bx, ahi, bx, (float)(N - 1), N, x0, x1);
    // element steps along x and y of the pixel and of its three orbit
    // members (the orbit copy is x-fastest; a slice has < 2^31 pixels)
    int sx, sy, mstep_x[3] = {0, 0, 0}, mstep_y[3] = {0, 0, 0}, mbase[3] = {0, 0, 0};
    if constexpr (PIX4) {
      sx = 1;
      sy = N;
    } else {
      int64_t sx_, sy_, sz_;
      img_strides<IO>(d, sx_, sy_, sz_);
      sx = (int)sx_;
      sy = (int)sy_;
#pragma unroll
      for (int m = 0; m < 3; ++m) {
        mstep_x[m] = qm.axx[m] * sx + qm.ayx[m] * sy;
        mstep_y[m] = qm.axy[m] * sx + qm.ayy[m] * sy;
        mbase[m] = qm.cx[m] * sx + qm.cy[m] * sy;
      }
    }
    for (int x = x0 + L.lane_group; x <= x1; x += SPLIT) {
      const float xf = (float)x;
      const int ylo = max(0, (int)ceilf(fmaf(bx, xf, alo)));
      const int yhi = min(N - 1, (int)floorf(fmaf(bx, xf, ahi)));
      float pos = fmaf(Y, (float)ylo, fmaf(X, xf, base));
      int o0 = ylo * sy + x * sx;
      if constexpr (ZS == 2) {
        // both slices' members, one candidate per trip
        const int64_t slice4 = (int64_t)N * N;
        for (int y = ylo; y <= yhi; ++y) {
          const float4 pa4 = __ldg(img4 + o0);
          const float4 qa4 = __ldg(img4 + slice4 + o0);
#pragma unroll
          for (int q = 0; q < kRayGroup; ++q) {
            const float wa = fmaxf(0.0f, 1.0f - fabsf(pos - (float)q));
            const float2 wa2 = make_float2(wa, wa);
            acc01[q] = __ffma2_rn(wa2, make_float2(pa4.x, pa4.y), acc01[q]);
            acc23[q] = __ffma2_rn(wa2, make_float2(pa4.z, pa4.w), acc23[q]);
            zacc01[q] = __ffma2_rn(wa2, make_float2(qa4.x, qa4.y), zacc01[q]);
            zacc23[q] = __ffma2_rn(wa2, make_float2(qa4.z, qa4.w), zacc23[q]);
          }
          o0 += sy;
          pos += Y;
        }
        continue;
      }
      int om[3];
#pragma unroll
      for (int m = 0; m < 3; ++m) om[m] = mbase[m] + x * mstep_x[m] + ylo * mstep_y[m];
      for (int y = ylo; y <= yhi; y += 2) {
        const bool two = y < yhi;
        const float pb = pos + Y;
        float4 pa4, pb4;
        if constexpr (PIX4) {
          pa4 = __ldg(img4 + o0);
          pb4 = __ldg(img4 + (two ? o0 + sy : o0));
        } else {
          pa4 = make_float4(ldg(img + o0), ldg(img + om[0]), ldg(img + om[1]), ldg(img + om[2]));
          pb4 = two ? make_float4(ldg(img + o0 + sy), ldg(img + om[0] + mstep_y[0]),
                                  ldg(img + om[1] + mstep_y[1]), ldg(img + om[2] + mstep_y[2]))
                    : pa4;
#pragma unroll
          for (int m = 0; m < 3; ++m) om[m] += 2 * mstep_y[m];
        }
        const float mb = two ? 1.0f : 0.0f;  // a masked second candidate adds zeros
        const float2 a01 = make_float2(pa4.x, pa4.y), a23 = make_float2(pa4.z, pa4.w);
        const float2 mb2 = make_float2(mb, mb);
        const float2 b01 = __fmul2_rn(make_float2(pb4.x, pb4.y), mb2);
        const float2 b23 = __fmul2_rn(make_float2(pb4.z, pb4.w), mb2);
#pragma unroll
        for (int q = 0; q < kRayGroup; ++q) {
          const float wa = fmaxf(0.0f, 1.0f - fabsf(pos - (float)q));
          const float wb = fmaxf(0.0f, 1.0f - fabsf(pb - (float)q));
          const float2 wa2 = make_float2(wa, wa), wb2 = make_float2(wb, wb);
          acc01[q] = __ffma2_rn(wb2, b01, __ffma2_rn(wa2, a01, acc01[q]));
          acc23[q] = __ffma2_rn(wb2, b23, __ffma2_rn(wa2, a23, acc23[q]));
        }
        o0 += 2 * sy;
        pos = pb + Y;
      }
    }
  }
  constexpr int kOut = kOrbit * ZS;  // members of slice z, then of slice z + 1
  float acc[kOut][kRayGroup];
#pragma unroll
  for (int q = 0; q < kRayGroup; ++q) {
    acc[0][q] = acc01[q].x;
    acc[1][q] = acc01[q].y;
    acc[2][q] = acc23[q].x;
    acc[3][q] = acc23[q].y;
    if constexpr (ZS == 2) {
      acc[4][q] = zacc01[q].x;
      acc[5][q] = zacc01[q].y;
      acc[6][q] = zacc23[q].x;
      acc[7][q] = zacc23[q].y;
    }
  }
  if (SPLIT > 1) {
#pragma unroll
    for (int m = 0; m < kOut; ++m) warp_reduce_rows<SPLIT>(acc[m]);
  }
  // every lane of the group now holds every sum.  Epilogues that read memory
  // (solver steps) share the group's outputs over its lanes, one each per
  // round, so their loads go out together; the plain store stays with the
  // group's first lane (spread, 256^2 x 180 measured 2 us slower a step)
  constexpr int kN = kOut * kRayGroup;
  constexpr bool kSpread = !std::is_same<Epi, FwdStore<float>>::value;
  constexpr int kLanes = kSpread ? SPLIT : 1;
  static_assert(kN % SPLIT == 0 || SPLIT > kN, "whole rounds of outputs");
  double part = 0.0;
  if (active && (kSpread || L.lane_group == 0)) {
    const float scale = g.delta_x * g.delta_x / g.delta_xi;
    const int64_t mirror_max = d.Ns - 1 - H;  // mirrored outputs for s <= this
#pragma unroll
    for (int base = 0; base < kN; base += kLanes) {
      const int oi = base + (kSpread ? L.lane_group : 0);
      const float v = pick_output<kOut, kRayGroup>(acc, oi);
      const int64_t s = s0 + oi % kRayGroup;
      const int m = oi / kRayGroup;
      const int64_t zz = z + m / kOrbit;
      const int c = (m + shift) & (kOrbit - 1);
      const int64_t bin = (c & 2) ? d.Ns - 1 - s : s;
      const int64_t ang = k + ((c & 1) ? Q : 0);
      if (oi < kN && s < H && !((c & 2) && s > mirror_max))
        part += epi(bin, ang, zz, sino_index<SO>(bin, ang, zz, d), v * scale);
    }
  }
  return part;
}

// One launch per slice (ZS = 2: per pair of slices): img points at slice z,
// img4 at its orbit copy (PIX4).  A pair's block partial covers both slices
// and lands in slice z's slot; slice z + 1's slot gets 0, so the partials of
// a stack keep one slot per block and slice.
template <int SO, int IO, int SPLIT, bool PIX4, int ZS, class Epi>
__global__ void __launch_bounds__(kFwdBlock)
radon_fwd_quarter(const float* __restrict__ img, const float4* __restrict__ img4,
                  const float* __restrict__ ofs, RadonGeo<float> g, Dims d, QuarterMaps qm,
                  Epi epi, double* __restrict__ partials, const int* __restrict__ skip,
                  int64_t z) {
  __shared__ double red[32];
  pdl_wait();
  pdl_trigger();
  if (skip != nullptr && *skip) return;
  const double part = radon_fwd_quarter_tile<SO, IO, SPLIT, PIX4, ZS, Epi>(
      img, img4, ofs, g, d, qm, epi, blockIdx, z);
  if (Epi::kReduce) {
    const double t = block_sum(part, red);
    if (threadIdx.x + blockDim.x * threadIdx.y == 0) {
      partials[bid_linear()] = t;
      if (ZS == 2) partials[bid_linear() + (int64_t)gridDim.x * gridDim.y] = 0.0;
    }
  }
}

// Row copy of the parallel-beam orbits: for base angle k < Q, entry 1 + j
// holds (row_k[j], row_{k+Q}[j], row_k[Ns-1-j], row_{k+Q}[Ns-1-j]), j = -1
// .. Ns + 1 (zeros off the detector).  Interpolating an entry pair at a
// position u gives the two rows at u and, in the last two lanes, the two
// rows at the mirrored position Ns - 1 - u, with the same weights.  Slice
// z0 + blockIdx.z goes to copy blockIdx.z.
template <int SO>
__global__ void __launch_bounds__(256)
radon_orbit_rows(const float* __restrict__ sino, Dims d, float4* __restrict__ rows4, int64_t z0,
                 const int* __restrict__ skip) {
  pdl_wait();
  pdl_trigger();
  if (skip != nullptr && *skip) return;
  const int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t k = blockIdx.y;
  const int64_t nrow = d.Ns + kOrbitRowPad;
  if (e >= nrow) return;
  const int64_t Q = d.Na / 2;
  int64_t ss_, sa_, sz_;
  sino_strides<SO>(d, ss_, sa_, sz_);
  const float* slice = sino + (z0 + blockIdx.z) * sz_;
  const int64_t j = e - 1, jm = d.Ns - 1 - j;
  auto at = [&](int64_t s, int64_t a) {
    return (s >= 0 && s < d.Ns) ? ldg(slice + s * ss_ + a * sa_) : 0.0f;
  };
  rows4[((int64_t)blockIdx.z * Q + k) * nrow + e] =
      make_float4(at(j, k), at(j, k + Q), at(jm, k), at(jm, k + Q));
}

// Backprojection over the parallel-beam orbits from radon_orbit_rows: a
// thread owns the orbit P0, P1 = S P0, P2 = -P0, P3 = -S P0 of one pixel of
// the quadrant x, y < N/2 (N even); for base angle k it evaluates the
// detector positions u0 of P0 and u1 of P1 (those of P2 and P3 are their
// mirrors) and, with one entry pair per position, adds 8 pixel-angles:
//   u0: (P0, k) (P3, k+Q) (P2, k) (P1, k+Q)   u1: (P1, k) (P0, k+Q) (P3, k) (P2, k+Q)
// (xi(k + Q, P) = xi(k, S P) and xi(k, -P) = Ns - 1 - xi(k, P)).  The row
// values are interpolated as v0 + fr (v1 - v0) and weighted by the angle's
// weight, as radon.cl:183-241 does; G thread groups take interleaved base
// angles and are added in a fixed order.  ROWS: the entries come from the
// row copy `rows4` of slice z; otherwise they are gathered from slice z of
// `sino` (zeros off the detector), the same values, so both forms give the
// same sums bit for bit.  The tile of block `bid` (32 x 8 threads).
template <int IO, int SO, int G, bool ROWS, class Epi>
__device__ __forceinline__ double radon_bwd_orbit_tile(const float4* __restrict__ rows4,
                                                       const float* __restrict__ sino,
                                                       const float* __restrict__ ofs, Dims d,
                                                       QuarterMaps qm, Epi epi, uint3 bid,
                                                       int64_t z) {
  constexpr int kOrbit = 4;
  constexpr int kRowsT = kBwdTileSlow / G;
  const int lane = threadIdx.x, trow = threadIdx.y;
  const int grp = trow / kRowsT, trow_t = trow % kRowsT;
  const int N = (int)d.Nx, half = N / 2;
  const int Q = (int)(d.Na / 2);
  const int nrow = (int)d.Ns + kOrbitRowPad;
  const int px0 = (int)bid.x * kBwdTileFast + lane;
  const int py0 = (int)bid.y * kRowsT + trow_t;
  const bool own = px0 < half && py0 < half;
  // S is the transpose of the first lookup map S^-1
  auto orbit = [&](int (&ox)[kOrbit], int (&oy)[kOrbit]) {
    const int c2 = N - 1;  // twice the centre
    const int dx = 2 * px0 - c2, dy = 2 * py0 - c2;  // twice P0 - centre
    const int sx = qm.axx[0] * dx + qm.ayx[0] * dy, sy = qm.axy[0] * dx + qm.ayy[0] * dy;
    ox[0] = px0;
    oy[0] = py0;
    ox[1] = (c2 + sx) / 2;
    oy[1] = (c2 + sy) / 2;
    ox[2] = c2 - px0;
    oy[2] = c2 - py0;
    ox[3] = c2 - ox[1];
    oy[3] = c2 - oy[1];
  };
  float2 pxr, pyr;  // P0 and P1 relative to the image centre
  {
    int ox[kOrbit], oy[kOrbit];
    orbit(ox, oy);
    const float c = 0.5f * (float)(N - 1);
    pxr = make_float2((float)ox[0] - c, (float)ox[1] - c);
    pyr = make_float2((float)oy[0] - c, (float)oy[1] - c);
  }
  const float mid1 = 0.5f * (float)(d.Ns - 1) + 1.0f;  // padded entry of the centre
  const float2 mid2 = make_float2(mid1, mid1);
  const float hi = (float)d.Ns + 1.0f;
  const float2 neg = make_float2(-1.0f, -1.0f);
  int64_t ss_ = 0, sa_ = 0, sz_ = 0;
  if constexpr (!ROWS) {
    sino_strides<SO>(d, ss_, sa_, sz_);
    sino += z * sz_;
  }
  // entry e of base angle k: (row_k[j], row_{k+Q}[j], row_k[Ns-1-j],
  // row_{k+Q}[Ns-1-j]) with j = e - 1, zeros off the detector
  auto entry = [&](const float4* row, int k, int e) -> float4 {
    if constexpr (ROWS) {
      return __ldg(row + e);
    } else {
      const int j = e - 1, jm = (int)d.Ns - 1 - j;
      const bool in = (unsigned)j < (unsigned)d.Ns;
      const int jj = in ? j : 0, jmm = in ? jm : 0;  // off the detector: bin 0, read and dropped
      const float* rk = sino + (int64_t)k * sa_;
      const float* rq = sino + (int64_t)(k + Q) * sa_;
      const float4 v = make_float4(ldg(rk + jj * ss_), ldg(rq + jj * ss_), ldg(rk + jmm * ss_),
                                   ldg(rq + jmm * ss_));
      return in ? v : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
  };
  // (P0, P3) (P2, P1) (P1, P0) (P3, P2)
  float2 A = make_float2(0.f, 0.f), B = A, C = A, D = A;
#pragma unroll 2
  for (int k = grp; k < Q; k += G) {
    const float X = ldg(ofs + 8 * k), Y = ldg(ofs + 8 * k + 1);
    const float2 W = make_float2(ldg(ofs + 8 * k + 4), ldg(ofs + 8 * (k + Q) + 4));
    const float2 u = __ffma2_rn(make_float2(X, X), pxr, __ffma2_rn(make_float2(Y, Y), pyr, mid2));
    const float uc[2] = {fminf(fmaxf(u.x, 0.0f), hi), fminf(fmaxf(u.y, 0.0f), hi)};
    const float4* row = ROWS ? rows4 + k * nrow : nullptr;
    float2 lo[2], hi2[2];
#pragma unroll
    for (int e = 0; e < 2; ++e) {
      const float fl = floorf(uc[e]);
      const float fr = uc[e] - fl;
      const int n = (int)fl;
      const float4 e0 = entry(row, k, n), e1 = entry(row, k, n + 1);
      const float2 f2 = make_float2(fr, fr);
      const float2 l0 = make_float2(e0.x, e0.y), h0 = make_float2(e0.z, e0.w);
      lo[e] = __ffma2_rn(f2, __ffma2_rn(l0, neg, make_float2(e1.x, e1.y)), l0);
      hi2[e] = __ffma2_rn(f2, __ffma2_rn(h0, neg, make_float2(e1.z, e1.w)), h0);
    }
    A = __ffma2_rn(W, lo[0], A);
    B = __ffma2_rn(W, hi2[0], B);
    C = __ffma2_rn(W, lo[1], C);
    D = __ffma2_rn(W, hi2[1], D);
  }
  const float sum[kOrbit] = {A.x + C.y, B.y + C.x, B.x + D.y, A.y + D.x};
  // fixed-order combination of the G angle groups, and the epilogue
  return orbit_epilogue<IO, G>(
      sum, own,
      [&](int k, int& x, int& y) {
        int ox[kOrbit], oy[kOrbit];
        orbit(ox, oy);
        pick_pixel(ox, oy, k, x, y);
      },
      epi, z, d);
}

// From the row copy: slice z0 + blockIdx.z, its copy is copy blockIdx.z.
template <int IO, int G, class Epi>
__global__ void __launch_bounds__(kBwdTileFast * kBwdTileSlow)
radon_bwd_orbit_rows(const float4* __restrict__ rows4, const float* __restrict__ ofs, Dims d,
                     QuarterMaps qm, Epi epi, double* __restrict__ partials,
                     const int* __restrict__ skip, int64_t z0) {
  __shared__ double red[32];
  pdl_wait();
  pdl_trigger();
  if (skip != nullptr && *skip) return;
  const int64_t nrow = d.Ns + kOrbitRowPad;
  const double part = radon_bwd_orbit_tile<IO, ORDER_F, G, true, Epi>(
      rows4 + (int64_t)blockIdx.z * (d.Na / 2) * nrow, nullptr, ofs, d, qm, epi, blockIdx,
      z0 + blockIdx.z);
  if (Epi::kReduce) {
    const double t = block_sum(part, red);
    if (threadIdx.x + blockDim.x * threadIdx.y == 0) partials[bid_linear()] = t;
  }
}

// Gathering from the sinogram (no scratch): slice z0 + blockIdx.z.
template <int IO, int SO, int G, class Epi>
__global__ void __launch_bounds__(kBwdTileFast * kBwdTileSlow)
radon_bwd_orbit(const float* __restrict__ sino, const float* __restrict__ ofs, Dims d,
                QuarterMaps qm, Epi epi, double* __restrict__ partials,
                const int* __restrict__ skip, int64_t z0) {
  __shared__ double red[32];
  pdl_wait();
  pdl_trigger();
  if (skip != nullptr && *skip) return;
  const double part = radon_bwd_orbit_tile<IO, SO, G, false, Epi>(nullptr, sino, ofs, d, qm, epi,
                                                                  blockIdx, z0 + blockIdx.z);
  if (Epi::kReduce) {
    const double t = block_sum(part, red);
    if (threadIdx.x + blockDim.x * threadIdx.y == 0) partials[bid_linear()] = t;
  }
}

// The mirrored kernel with 32 lanes per bin group (the form the projections
// launch) is held to 72 registers, 7 blocks per SM instead of 6 at its
// natural 80 (one 4-byte spill): 512^2 x 360 forward 1471-1473 -> 1516-1534
// Gpixel-angle/s, and the 2048^2 x 64 TV iteration 323.1 -> 314.5 ms.  At 64
// registers (8 blocks) it spills 80 bytes.  (Two candidates per trip took 94
// registers, and capped at 80 for 6 blocks per SM spilled and ran 512^2 x
// 360 in 99.4 instead of 77.0 us.)
template <int SO, int IO, int SPLIT, bool PIX4, bool MIRROR, class Epi>
__global__ void __launch_bounds__(kFwdBlock, MIRROR && SPLIT >= 32 ? 7 : 1)
fan_fwd_quarter(const float* __restrict__ img, const float4* __restrict__ img4,
                const float* __restrict__ ofs,
                const float* __restrict__ sdpd, FanGeo<float> g, Dims d, QuarterMaps qm, Epi epi,
                double* __restrict__ partials, const int* __restrict__ skip, int64_t z) {
  // one launch per slice: img and img4 point at slice z (a base offset
  // computed here instead of taken from the parameters measured 8% slower)
  __shared__ double red[32];
  pdl_wait();
  pdl_trigger();
  if (skip != nullptr && *skip) return;
  const double part = fan_fwd_quarter_tile<SO, IO, SPLIT, PIX4, MIRROR, Epi>(
      img, img4, ofs, sdpd, g, d, qm, epi, blockIdx, z);
  if (Epi::kReduce) {
    double t = block_sum(part, red);
    if (threadIdx.x + blockDim.x * threadIdx.y == 0)
      partials[bid_linear()] = t;
  }
}

}  // namespace fast
}  // namespace gr
