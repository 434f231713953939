// Pixel-driven Radon and fan-beam projection kernels (templates).
//
// Each kernel is a deterministic gather: one thread owns one output element
// (a detector bin for the forward projection, a pixel for the backprojection)
// for ZB consecutive z-slices, accumulates its sum in registers in the same
// order as gratopy's OpenCL kernels, and hands the result to an epilogue
// functor that stores it or fuses the next solver step into the store.
// No atomics anywhere, so every output is bit-reproducible.
//
// Reference kernels (gratopy): radon.cl:66-161 (radon), radon.cl:183-241
// (radon_ad), fanbeam.cl:72-256 (fanbeam), fanbeam.cl:290-391 (fanbeam_ad).
#pragma once

#include <type_traits>

#include "gr_common.cuh"

namespace gr {

// Angles staged in shared memory per chunk.
constexpr int kAngleChunk = 128;
constexpr int kBwdTileFast = 32;   // threads along the contiguous pixel axis
constexpr int kBwdTileSlow = 8;    // threads along the other pixel axis
constexpr int kFwdBlock = 128;     // detector bins per forward block

// Scalar geometry of one projection problem (values of gratopy's
// Geometryinformation vector, already rounded to the kernel precision).
template <typename T>
struct RadonGeo {
  float delta_x, delta_xi;  // read as float even in double kernels (radon.cl:82-83)
};

template <typename T>
struct FanGeo {
  T R, RE, delta_xi, midx, midy, mid_det, delta_x;
};

// ------------------------------------------------------------------ epilogues
// Forward epilogues see (s, a, z, linear sinogram index, value) and return a
// double contribution to the block partial sum (0 when not reducing).

template <typename T>
struct FwdStore {
  static constexpr bool kReduce = false;
  T* out;
  __device__ __forceinline__ double operator()(int64_t, int64_t, int64_t, int64_t i, T v) const {
    out[i] = v;
    return 0.0;
  }
};

// Landweber: out = A u - f  (gratopy.py:2437-2438)
template <typename T>
struct FwdResidual {
  static constexpr bool kReduce = false;
  T* out;
  const T* f;
  __device__ __forceinline__ double operator()(int64_t, int64_t, int64_t, int64_t i, T v) const {
    out[i] = v - f[i];
    return 0.0;
  }
};

// TV dual data step: lambda = (lambda + sigma (A u - f)) * mu''
// (total_variation.cl:95-106, with Ku never written to memory).
template <typename T>
struct FwdLambda {
  static constexpr bool kReduce = false;
  T* lambda;
  const T* f;
  float sigma, mu2;
  __device__ __forceinline__ double operator()(int64_t, int64_t, int64_t, int64_t i, T v) const {
    lambda[i] = (lambda[i] + sigma * (v - f[i])) * mu2;
    return 0.0;
  }
};

// CG: q = A p and the block partial of <W q, q> (angle weights W).
template <typename T>
struct FwdStoreWeightedSq {
  static constexpr bool kReduce = true;
  T* out;
  const T* w;  // angle weights, length Na
  __device__ __forceinline__ double operator()(int64_t, int64_t a, int64_t, int64_t i, T v) const {
    out[i] = v;
    T wv = v * w[a];  // weight_sinogram rounds the product in the array dtype
    return (double)wv * (double)v;
  }
};

// Backprojection epilogues see (x, y, z, linear image index, value).

template <typename T>
struct BwdStore {
  static constexpr bool kReduce = false;
  T* out;
  __device__ __forceinline__ double operator()(int64_t, int64_t, int64_t, int64_t i, T v) const {
    out[i] = v;
    return 0.0;
  }
};

// Landweber: u += a * (A^T r)  (equ_mul_add, utilities.cl:69-73)
template <typename T>
struct BwdAxpy {
  static constexpr bool kReduce = false;
  T* u;
  T a;
  __device__ __forceinline__ double operator()(int64_t, int64_t, int64_t, int64_t i, T v) const {
    u[i] += a * v;
    return 0.0;
  }
};

// Store and add the value to the block partial sum (normest's plain sum).
template <typename T>
struct BwdStoreSum {
  static constexpr bool kReduce = true;
  T* out;
  __device__ __forceinline__ double operator()(int64_t, int64_t, int64_t, int64_t i, T v) const {
    out[i] = v;
    return (double)v;
  }
};

// CG: snew = A^T d, x += alpha p, partial of <snew, snew>.
template <typename T>
struct BwdCG {
  static constexpr bool kReduce = true;
  T* snew;
  T* x;
  const T* p;
  const double* alpha;  // device scalar, already rounded to T
  __device__ __forceinline__ double operator()(int64_t, int64_t, int64_t, int64_t i, T v) const {
    snew[i] = v;
    const T al = (T)(*alpha);
    x[i] += al * p[i];
    return (double)v * (double)v;
  }
};

// TV primal step fused into the backprojection (total_variation.cl:108-148
// followed by gratopy.py:2708-2717):
//   u_new = max(0, u + tau (div v - norming * K^T lambda)),  ubar = 2 u_new - u
// v holds 4 reals per pixel in the image's index order.
template <typename T, int O>
struct BwdTVPrimal {
  static constexpr bool kReduce = false;
  T* u;
  T* ubar;
  const T* v;
  Dims d;
  float tau, norming, z_distance;
  __device__ __forceinline__ double operator()(int64_t x, int64_t y, int64_t z, int64_t i,
                                               T kl) const {
    int64_t sx, sy, sz;
    img_strides<O>(d, sx, sy, sz);
    const T* vp = v + 4 * i;
    T v0 = vp[0], v1 = vp[1], v2 = vp[2];
    if (x == d.Nx - 1) v0 = (T)0.;
    if (x > 0) v0 -= vp[-4 * sx + 0];
    if (y == d.Ny - 1) v1 = (T)0.;
    if (y > 0) v1 -= vp[-4 * sy + 1];
    if (z == d.Nz - 1) v2 = (T)0.;
    if (z > 0) v2 -= vp[-4 * sz + 2];
    if (z_distance > 0) v2 /= z_distance; else v2 = (T)0.;
    const T uo = u[i];
    const T un = gmax((T)0., uo + tau * (v0 + v1 + v2 - norming * kl));
    u[i] = un;
    ubar[i] = 2.0f * un - uo;
    return 0.0;
  }
};

// Transposes and the unrolled-TV adjoint.
// out = base + c * w[a] * (A u)   (base may be null): B^T h = (ds/dx / dx) W A h
// is this with base = null, c = ds/dx / dx; the TV adjoint uses a base.
template <typename T>
struct FwdAngleAxpy {
  static constexpr bool kReduce = false;
  T* out;
  const T* base;
  const T* w;
  T c;
  __device__ __forceinline__ double operator()(int64_t, int64_t a, int64_t, int64_t i, T v) const {
    const T b = base ? base[i] : (T)0.;
    out[i] = b + c * w[a] * v;
    return 0.0;
  }
};

// Adjoint of the TV extragradient/dual coupling on the image:
// out = c1 * (A^T lambda_bar) - sigma * div(gw), div as in total_variation.cl:119-143.
template <typename T, int O>
struct BwdTVAdjoint {
  static constexpr bool kReduce = false;
  T* out;
  const T* gw;
  Dims d;
  T c1;
  float sigma, z_distance;
  __device__ __forceinline__ double operator()(int64_t x, int64_t y, int64_t z, int64_t i,
                                               T v) const {
    int64_t sx, sy, sz;
    img_strides<O>(d, sx, sy, sz);
    const T* vp = gw + 4 * i;
    T v0 = vp[0], v1 = vp[1], v2 = vp[2];
    if (x == d.Nx - 1) v0 = (T)0.;
    if (x > 0) v0 -= vp[-4 * sx + 0];
    if (y == d.Ny - 1) v1 = (T)0.;
    if (y > 0) v1 -= vp[-4 * sy + 1];
    if (z == d.Nz - 1) v2 = (T)0.;
    if (z > 0) v2 -= vp[-4 * sz + 2];
    if (z_distance > 0) v2 /= z_distance; else v2 = (T)0.;
    out[i] = c1 * v - sigma * (v0 + v1 + v2);
    return 0.0;
  }
};

// ------------------------------------------------------------------ helpers

// Per-angle record of the Radon backprojection staged in shared memory.
template <typename T>
struct alignas(sizeof(T) * 4) RadonAngle {
  T X, Y, off, w;
};

// Warp layout of the forward kernels: a warp holds 32/SPLIT consecutive
// detector bins of one angle; the SPLIT lanes of a bin walk interleaved image
// rows and are summed with warp shuffles (fixed xor order: deterministic).
template <int SPLIT>
struct FwdLayout {
  static constexpr int kRaysPerWarp = 32 / SPLIT;
  static constexpr int kRaysPerBlock = kRaysPerWarp * (kFwdBlock / 32);
  int64_t s;
  int group;
  __device__ __forceinline__ FwdLayout() {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    s = (int64_t)blockIdx.x * kRaysPerBlock + warp * kRaysPerWarp + (lane % kRaysPerWarp);
    group = lane / kRaysPerWarp;
  }
};

template <int SPLIT, typename T, int ZB>
__device__ __forceinline__ void warp_reduce_rows(T (&acc)[ZB]) {
#pragma unroll
  for (int o = 32 / SPLIT; o < 32; o <<= 1) {
#pragma unroll
    for (int k = 0; k < ZB; ++k) acc[k] += __shfl_xor_sync(0xffffffffu, acc[k], o);
  }
}

// Reciprocal used by the float32 fan kernels: one hardware approximation
// (relative error ~1e-7, far inside the float32 tolerance); float64 keeps
// the reference's exact divisions.
__device__ __forceinline__ float fast_rcp(float v) { return __fdividef(1.0f, v); }

// ------------------------------------------------------------- Radon forward
// radon.cl:66-161.  One detector bin per SPLIT lanes, ZB slices per thread.
// ofs: 8 reals per angle (X, Y, offset, 1/max, weight, flip, -, -).
template <typename T, int SO, int IO, int ZB, int SPLIT, class Epi>
__global__ void __launch_bounds__(kFwdBlock)
radon_fwd_kernel(const T* __restrict__ img, const T* __restrict__ ofs, RadonGeo<T> g, Dims d,
                 Epi epi, double* __restrict__ partials, const int* __restrict__ skip) {
  __shared__ double red[kFwdBlock / 32];
  if (skip != nullptr && *skip) return;
  const FwdLayout<SPLIT> L;
  const int64_t s = L.s;
  const int64_t a = blockIdx.y;
  const int64_t z0 = (int64_t)blockIdx.z * ZB;
  const bool active = s < d.Ns;
  const int zn = (int)min((int64_t)ZB, d.Nz - z0);
  T acc[ZB];
#pragma unroll
  for (int k = 0; k < ZB; ++k) acc[k] = (T)0.;
  if (active) {
    const T* o8 = ofs + 8 * a;
    T ox = o8[0], oy = o8[1];
    const T oz = o8[2], ow = o8[3];
    const bool flip = o8[5] != (T)0.;
    int Nxx = (int)d.Nx, Nyy = (int)d.Ny;
    int64_t sx, sy, sz;
    img_strides<IO>(d, sx, sy, sz);
    int64_t step_x = sx, step_y = sy;
    if (flip) {
      T t = ox; ox = oy; oy = t;
      Nxx = (int)d.Ny;
      Nyy = (int)d.Nx;
      step_x = sy;
      step_y = sx;
    }
    const T* img0 = img + z0 * sz;
    const T fs = (T)(int)s;
    for (int y = L.group; y < Nyy; y += SPLIT) {
      const T dd = (T)y * oy + oz - fs;
      int x_low = (int)((-1 - dd) * ow);
      int x_high = (int)((1 - dd) * ow);
      if (ow < (T)0.) { int t = x_low; x_low = x_high; x_high = t; }
      x_low = max(x_low, 0);
      x_high = min(x_high, Nxx - 1);
      const T* p = img0 + (int64_t)y * step_y + (int64_t)x_low * step_x;
      for (int x = x_low; x <= x_high; ++x) {
        const T w = (T)1. - gabs((T)x * ox + dd);
        T v[ZB];
#pragma unroll
        for (int k = 0; k < ZB; ++k) v[k] = k < zn ? ldg(p + k * sz) : (T)0.;
        if (w > (T)0.) {
#pragma unroll
          for (int k = 0; k < ZB; ++k) acc[k] += w * v[k];
        }
        p += step_x;
      }
    }
  }
  if (SPLIT > 1) warp_reduce_rows<SPLIT>(acc);
  double part = 0.0;
  if (active && L.group == 0) {
#pragma unroll
    for (int k = 0; k < ZB; ++k) {
      if (k < zn) {
        const int64_t z = z0 + k;
        const T val = acc[k] * (T)g.delta_x * (T)g.delta_x / (T)g.delta_xi;
        part += epi(s, a, z, sino_index<SO>(s, a, z, d), val);
      }
    }
  }
  if (Epi::kReduce) {
    double t = block_sum(part, red);
    if (threadIdx.x == 0)
      partials[blockIdx.x + gridDim.x * ((int64_t)blockIdx.y + gridDim.y * (int64_t)blockIdx.z)] = t;
  }
}

// --------------------------------------------------------------- Fan forward
// fanbeam.cl:72-256.  Same layout as the Radon forward kernel.
template <typename T, int SO, int IO, int ZB, int SPLIT, class Epi>
__global__ void __launch_bounds__(kFwdBlock)
fan_fwd_kernel(const T* __restrict__ img, const T* __restrict__ ofs, const T* __restrict__ sdpd,
               FanGeo<T> g, Dims d, Epi epi, double* __restrict__ partials,
               const int* __restrict__ skip) {
  __shared__ double red[kFwdBlock / 32];
  if (skip != nullptr && *skip) return;
  const FwdLayout<SPLIT> L;
  const int64_t s = L.s;
  const int64_t a = blockIdx.y;
  const int64_t z0 = (int64_t)blockIdx.z * ZB;
  const bool active = s < d.Ns;
  const int zn = (int)min((int64_t)ZB, d.Nz - z0);
  T acc[ZB];
#pragma unroll
  for (int k = 0; k < ZB; ++k) acc[k] = (T)0.;
  const T R = g.R, dxi = g.delta_xi;
  if (active) {
    T midx = g.midx, midy = g.midy;
    T RE = g.RE;
    const T* o = ofs + 8 * a;
    T dx = o[0], dy = o[1], qx = o[2], qy = o[3];
    const T d0x = o[4], d0y = o[5];
    const T sr = (T)(int)s;
    const T fp = -g.mid_det + sr + 1;
    const T fm = -g.mid_det + sr - 1;
    T dpx = d0x + dx * fp - qx, dpy = d0y + dy * fp - qy;
    T dmx = d0x + dx * fm - qx, dmy = d0y + dy * fm - qy;
    T ddx = d0x - qx, ddy = d0y - qy;
    const T RR = R * R;
    ddx /= RR;
    ddy /= RR;
    const T xx2 = dxi * dxi;
    dx /= xx2;
    dy /= xx2;
    RE *= (T)1 / R;
    int Nyy = (int)d.Ny, Nxx = (int)d.Nx;
    int64_t sx, sy, sz;
    img_strides<IO>(d, sx, sy, sz);
    int64_t step_x = sx, step_y = sy;
    if (!(gabs(dpx) < gabs(dpy) && gabs(dmx) < gabs(dmy))) {
      T t;
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
    if ((qy) * (dmx - dpx) < (T)0.) {
      T t = dpx; dpx = dmx; dmx = t;
    }
    const T s_mid = sr - g.mid_det;
    const T hi_lim = (T)(Nxx - 1) - midx;
    const T lo_lim = -midx;
    const T* img0 = img + z0 * sz;
    for (int y = L.group; y < Nyy; y += SPLIT) {
      const T yr = (T)y;
      const T xhigh = qx + dpx * (yr - midy - qy);
      const T xlow = qx + dmx * (yr - midy - qy);
      const int xhi = (int)gfloor(gmin(hi_lim, xhigh) + midx);
      const int xlo = (int)gceil(gmax(lo_lim, xlow) + midx);
      if (xlo > xhi) continue;
      T t = ddx * ((T)xlo - midx) + ddy * (yr - midy) + RE;
      T ss = dx * ((T)xlo - midx) + dy * (yr - midy);
      const T* p = img0 + (int64_t)y * step_y + (int64_t)xlo * step_x;
      for (int x = xlo; x <= xhi; ++x) {
        T W;
        if constexpr (std::is_same<T, float>::value) {
          const float r = fast_rcp(t);
          W = (1.0f - fabsf(s_mid - ss * r)) * r;
        } else {
          const T xi = ss / t;
          W = ((T)1. - gabs(s_mid - xi)) / t;
        }
#pragma unroll
        for (int k = 0; k < ZB; ++k)
          if (k < zn) acc[k] += W * ldg(p + k * sz);
        p += step_x;
        t += ddx;
        ss += dx;
      }
    }
  }
  if (SPLIT > 1) warp_reduce_rows<SPLIT>(acc);
  double part = 0.0;
  if (active && L.group == 0) {
    const T sd = sdpd[s];
#pragma unroll
    for (int k = 0; k < ZB; ++k) {
      if (k < zn) {
        const int64_t z = z0 + k;
        const T val = acc[k] * sd / dxi * g.delta_x / R;
        part += epi(s, a, z, sino_index<SO>(s, a, z, d), val);
      }
    }
  }
  if (Epi::kReduce) {
    double t = block_sum(part, red);
    if (threadIdx.x == 0)
      partials[blockIdx.x + gridDim.x * ((int64_t)blockIdx.y + gridDim.y * (int64_t)blockIdx.z)] = t;
  }
}

// ------------------------------------------------------------ backprojection
// Block = 32 lanes along the contiguous pixel axis (x for F images, y for C
// images) x 8 thread rows.  With angle split ASPLIT, ASPLIT consecutive
// thread rows share one pixel row and take interleaved angles; their partial
// sums are added in a fixed order through shared memory (deterministic).
template <int ASPLIT>
struct BwdLayout {
  static constexpr int kRows = kBwdTileSlow / ASPLIT;
  int64_t fast, slow;
  int g;
  __device__ __forceinline__ BwdLayout() {
    g = threadIdx.y % ASPLIT;
    fast = (int64_t)blockIdx.x * kBwdTileFast + threadIdx.x;
    slow = (int64_t)blockIdx.y * kRows + threadIdx.y / ASPLIT;
  }
};

template <typename T, int ZB, int ASPLIT>
struct BwdReduce {
  T v[kBwdTileSlow][ZB][kBwdTileFast];
};
template <typename T, int ZB>
struct BwdReduce<T, ZB, 1> {};

template <typename T, int ZB, int ASPLIT>
__device__ __forceinline__ void bwd_combine(T (&acc)[ZB], BwdReduce<T, ZB, ASPLIT>& red, int g) {
  if constexpr (ASPLIT == 1) {
    return;
  } else {
  __syncthreads();
#pragma unroll
  for (int k = 0; k < ZB; ++k) red.v[threadIdx.y][k][threadIdx.x] = acc[k];
  __syncthreads();
  if (g == 0) {
#pragma unroll
    for (int k = 0; k < ZB; ++k) {
      T t = red.v[threadIdx.y][k][threadIdx.x];
#pragma unroll
      for (int j = 1; j < ASPLIT; ++j) t += red.v[threadIdx.y + j][k][threadIdx.x];
      acc[k] = t;
    }
  }
  }
}

// radon.cl:183-241.
template <typename T, int IO, int SO, int ZB, int ASPLIT, class Epi>
__global__ void __launch_bounds__(kBwdTileFast * kBwdTileSlow)
radon_bwd_kernel(const T* __restrict__ sino, const T* __restrict__ ofs, Dims d, Epi epi,
                 double* __restrict__ partials, const int* __restrict__ skip) {
  __shared__ RadonAngle<T> sang[kAngleChunk];
  __shared__ double red[kBwdTileFast * kBwdTileSlow / 32];
  __shared__ BwdReduce<T, ZB, ASPLIT> cred;
  if (skip != nullptr && *skip) return;
  const BwdLayout<ASPLIT> L;
  const int64_t x = IO == ORDER_F ? L.fast : L.slow;
  const int64_t y = IO == ORDER_F ? L.slow : L.fast;
  const int64_t z0 = (int64_t)blockIdx.z * ZB;
  const bool active = x < d.Nx && y < d.Ny;
  const int zn = (int)min((int64_t)ZB, d.Nz - z0);
  int64_t ss_, sa_, sz_;
  sino_strides<SO>(d, ss_, sa_, sz_);
  const T* sn = sino + z0 * sz_;
  const int Ns = (int)d.Ns;
  const T cx = (T)x, cy = (T)y;
  T acc[ZB];
#pragma unroll
  for (int k = 0; k < ZB; ++k) acc[k] = (T)0.;
  const int tid = threadIdx.x + kBwdTileFast * threadIdx.y;
  for (int a0 = 0; a0 < d.Na; a0 += kAngleChunk) {
    const int na = (int)min((int64_t)kAngleChunk, d.Na - a0);
    __syncthreads();
    for (int j = tid; j < na; j += kBwdTileFast * kBwdTileSlow) {
      const T* o = ofs + 8 * (int64_t)(a0 + j);
      RadonAngle<T> r;
      r.X = o[0];
      r.Y = o[1];
      r.off = o[2];
      r.w = o[4];
      sang[j] = r;
    }
    __syncthreads();
    if (active) {
      for (int j = L.g; j < na; j += ASPLIT) {
        const RadonAngle<T> r = sang[j];
        const T s = cx * r.X + cy * r.Y + r.off;
        const T fl = gfloor(s);
        int sm = (int)fl;
        int sp = sm + 1;
        T wp, wm;
        if constexpr (std::is_same<T, float>::value) {
          wp = s - fl;
          wm = 1.0f - wp;
        } else {
          wp = (T)1 - ((T)sp - s);
          wm = (T)1 - (s - (T)sm);
        }
        if (sm < 0 || sm >= Ns) { wm = (T)0.; sm = 0; }
        if (sp < 0 || sp >= Ns) { wp = (T)0.; sp = 0; }
        const int64_t base = (int64_t)(a0 + j) * sa_;
        const T* pm = sn + base + (int64_t)sm * ss_;
        const T* pp = sn + base + (int64_t)sp * ss_;
#pragma unroll
        for (int k = 0; k < ZB; ++k)
          if (k < zn) acc[k] += r.w * (wm * ldg(pm + k * sz_) + wp * ldg(pp + k * sz_));
      }
    }
  }
  bwd_combine<T, ZB, ASPLIT>(acc, cred, L.g);
  double part = 0.0;
  if (active && L.g == 0) {
#pragma unroll
    for (int k = 0; k < ZB; ++k)
      if (k < zn) part += epi(x, y, z0 + k, img_index<IO>(x, y, z0 + k, d), acc[k]);
  }
  if (Epi::kReduce) {
    double t = block_sum(part, red);
    if (tid == 0)
      partials[blockIdx.x + gridDim.x * ((int64_t)blockIdx.y + gridDim.y * (int64_t)blockIdx.z)] = t;
  }
}

// fanbeam.cl:290-391.  Per angle: detector direction scaled by 1/dxi^2,
// source-to-detector-foot direction scaled by 1/R^2, source position and
// angle weight (divided by R in the float32 path), staged in shared memory.
template <typename T>
struct alignas(sizeof(T) * 8) FanAngle {
  T ddx, ddy, dx, dy, qx, qy, w, wR;
};

template <typename T, int IO, int SO, int ZB, int ASPLIT, class Epi>
__global__ void __launch_bounds__(kBwdTileFast * kBwdTileSlow)
fan_bwd_kernel(const T* __restrict__ sino, const T* __restrict__ ofs, const T* __restrict__ sdpd,
               FanGeo<T> g, Dims d, Epi epi, double* __restrict__ partials,
               const int* __restrict__ skip) {
  __shared__ FanAngle<T> sang[kAngleChunk];
  __shared__ double red[kBwdTileFast * kBwdTileSlow / 32];
  __shared__ BwdReduce<T, ZB, ASPLIT> cred;
  if (skip != nullptr && *skip) return;
  const BwdLayout<ASPLIT> L;
  const int64_t x = IO == ORDER_F ? L.fast : L.slow;
  const int64_t y = IO == ORDER_F ? L.slow : L.fast;
  const int64_t z0 = (int64_t)blockIdx.z * ZB;
  const bool active = x < d.Nx && y < d.Ny;
  const int zn = (int)min((int64_t)ZB, d.Nz - z0);
  int64_t ss_, sa_, sz_;
  sino_strides<SO>(d, ss_, sa_, sz_);
  const T* sn = sino + z0 * sz_;
  const int Ns = (int)d.Ns;
  const T Px = (T)x - g.midx, Py = (T)y - g.midy;
  const T R = g.R;
  const T R_sqr_inv = (T)1. / (R * R);
  const T dxi_sqr_inv = (T)1. / (g.delta_xi * g.delta_xi);
  T acc[ZB];
#pragma unroll
  for (int k = 0; k < ZB; ++k) acc[k] = (T)0.;
  const int tid = threadIdx.x + kBwdTileFast * threadIdx.y;
  for (int a0 = 0; a0 < d.Na; a0 += kAngleChunk) {
    const int na = (int)min((int64_t)kAngleChunk, d.Na - a0);
    __syncthreads();
    for (int j = tid; j < na; j += kBwdTileFast * kBwdTileSlow) {
      const T* o = ofs + 8 * (int64_t)(a0 + j);
      FanAngle<T> r;
      r.qx = o[2];
      r.qy = o[3];
      r.ddx = (o[4] - o[2]) * R_sqr_inv;
      r.ddy = (o[5] - o[3]) * R_sqr_inv;
      r.dx = o[0] * dxi_sqr_inv;
      r.dy = o[1] * dxi_sqr_inv;
      r.w = o[6];
      r.wR = o[6] / R;
      sang[j] = r;
    }
    __syncthreads();
    if (active) {
      for (int j = L.g; j < na; j += ASPLIT) {
        const FanAngle<T> r = sang[j];
        const T pqx = Px - r.qx, pqy = Py - r.qy;
        const T t = r.ddx * pqx + r.ddy * pqy;
        const T ss = r.dx * pqx + r.dy * pqy;
        T xi, scale;
        if constexpr (std::is_same<T, float>::value) {
          const float inv = fast_rcp(t);
          xi = ss * inv + g.mid_det;
          scale = r.wR * inv;
        } else {
          xi = ss / t + g.mid_det;
          scale = (T)0.;
        }
        const T fl = gfloor(xi);
        int xim = (int)fl;
        int xip = xim + 1;
        T Wp, Wm;
        if constexpr (std::is_same<T, float>::value) {
          Wp = xi - fl;
          Wm = 1.0f - Wp;
        } else {
          Wp = (T)1. - ((T)xip - xi);
          Wm = (T)1. - (xi - (T)xim);
        }
        if (xim < 0 || xim >= Ns) { Wm = (T)0.; xim = 0; } else { Wm *= ldg(sdpd + xim); }
        if (xip < 0 || xip >= Ns) { Wp = (T)0.; xip = 0; } else { Wp *= ldg(sdpd + xip); }
        const int64_t base = (int64_t)(a0 + j) * sa_;
        const T* pm = sn + base + (int64_t)xim * ss_;
        const T* pp = sn + base + (int64_t)xip * ss_;
        if constexpr (std::is_same<T, float>::value) {
#pragma unroll
          for (int k = 0; k < ZB; ++k)
            if (k < zn) acc[k] += scale * (Wm * ldg(pm + k * sz_) + Wp * ldg(pp + k * sz_));
        } else {
          const T rt = R * t;
#pragma unroll
          for (int k = 0; k < ZB; ++k)
            if (k < zn) acc[k] += r.w * (Wm * ldg(pm + k * sz_) + Wp * ldg(pp + k * sz_)) / rt;
        }
      }
    }
  }
  bwd_combine<T, ZB, ASPLIT>(acc, cred, L.g);
  double part = 0.0;
  if (active && L.g == 0) {
#pragma unroll
    for (int k = 0; k < ZB; ++k)
      if (k < zn) part += epi(x, y, z0 + k, img_index<IO>(x, y, z0 + k, d), acc[k]);
  }
  if (Epi::kReduce) {
    double t = block_sum(part, red);
    if (tid == 0)
      partials[blockIdx.x + gridDim.x * ((int64_t)blockIdx.y + gridDim.y * (int64_t)blockIdx.z)] = t;
  }
}

}  // namespace gr
