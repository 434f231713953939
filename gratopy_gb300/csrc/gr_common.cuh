// Shared device definitions for the gratopy_gb300 CUDA kernels (sm_103a).
//
// Array layouts follow gratopy (radon.cl:28-31): order F = x fastest,
// order C = z fastest:
//   image   F: x + Nx (y + Ny z)      C: z + Nz (y + Ny x)
//   sinogram F: s + Ns (a + Na z)     C: z + Nz (a + Na s)
// All index arithmetic is 64-bit (volumes of 2048^2 x 64 exceed 2^31 cells).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace gr {

enum { ORDER_F = 0, ORDER_C = 1 };

struct Dims {
  int64_t Nx, Ny, Nz, Ns, Na;
  // the array a kernel gathers from is C-ordered with whole groups of 4
  // slices at 16-byte aligned addresses: 4 slices load as one float4
  bool vec4 = false;
};

template <int O>
__host__ __device__ __forceinline__ int64_t img_index(int64_t x, int64_t y, int64_t z,
                                                      const Dims& d) {
  return O == ORDER_F ? x + d.Nx * (y + d.Ny * z) : z + d.Nz * (y + d.Ny * x);
}

template <int O>
__host__ __device__ __forceinline__ int64_t sino_index(int64_t s, int64_t a, int64_t z,
                                                       const Dims& d) {
  return O == ORDER_F ? s + d.Ns * (a + d.Na * z) : z + d.Nz * (a + d.Na * s);
}

// Strides (in elements) of one step in x, y, z for the image and in s, a, z
// for the sinogram.
template <int O>
__host__ __device__ __forceinline__ void img_strides(const Dims& d, int64_t& sx, int64_t& sy,
                                                     int64_t& sz) {
  if (O == ORDER_F) {
    sx = 1;
    sy = d.Nx;
    sz = d.Nx * d.Ny;
  } else {
    sx = d.Nz * d.Ny;
    sy = d.Nz;
    sz = 1;
  }
}

template <int O>
__host__ __device__ __forceinline__ void sino_strides(const Dims& d, int64_t& ss, int64_t& sa,
                                                      int64_t& sz) {
  if (O == ORDER_F) {
    ss = 1;
    sa = d.Ns;
    sz = d.Ns * d.Na;
  } else {
    ss = d.Nz * d.Na;
    sa = d.Nz;
    sz = 1;
  }
}

template <typename T>
__device__ __forceinline__ T ldg(const T* p) {
  return __ldg(p);
}

// Exact floor/ceil/abs helpers per precision.
__device__ __forceinline__ float gfloor(float v) { return floorf(v); }
__device__ __forceinline__ double gfloor(double v) { return floor(v); }
__device__ __forceinline__ float gceil(float v) { return ceilf(v); }
__device__ __forceinline__ double gceil(double v) { return ceil(v); }
__device__ __forceinline__ float gabs(float v) { return fabsf(v); }
__device__ __forceinline__ double gabs(double v) { return fabs(v); }
__device__ __forceinline__ float gmin(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ double gmin(double a, double b) { return fmin(a, b); }
__device__ __forceinline__ float gmax(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ double gmax(double a, double b) { return fmax(a, b); }
__device__ __forceinline__ float ghypot(float a, float b) { return hypotf(a, b); }
__device__ __forceinline__ double ghypot(double a, double b) { return hypot(a, b); }

// Linear index of the current block in its grid.
__device__ __forceinline__ int64_t bid_linear() {
  return blockIdx.x + (int64_t)gridDim.x * ((int64_t)blockIdx.y + (int64_t)gridDim.y * blockIdx.z);
}

// Programmatic dependent launch (kernels launched by launch_pdl): wait until
// the kernel before this one in the stream has completed and its writes are
// visible (returns at once for a kernel launched without the attribute), and
// let the next kernel start launching.  The wait is the hardware's, bounded
// by the previous kernel's completion; it comes before any global access.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// Linear-interpolation (hat) weight of a detector bin at distance d from the
// ray, max(0, 1 - |d|).  1 - |d| never exceeds 1, so clamping it to [0, 1]
// gives the same value for every d (a NaN gives 0 both ways, and 1 - |d| is
// never -0 in round-to-nearest); the clamp is a saturating add.  The fan-beam
// orbit forward uses it (512^2 x 360 forward 1457-1473 -> 1485
// Gpixel-angle/s); the parallel-beam forwards keep fmaxf(0, .), which
// measured faster there (256^2 x 180 forward + back 729 against 685).
__device__ __forceinline__ float hat_weight(float d) { return __saturatef(1.0f - fabsf(d)); }

// Deterministic block-wide sum of one double per thread.  Every thread of the
// block must call it; the result is valid in thread 0.  `red` must hold one
// double per warp.
__device__ __forceinline__ double block_sum(double v, double* red) {
  const unsigned full = 0xffffffffu;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(full, v, o);
  const int nthreads = blockDim.x * blockDim.y * blockDim.z;
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int warp = tid >> 5, lane = tid & 31;
  const int nwarps = (nthreads + 31) >> 5;
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  // the warps' sums by one more warp reduction (a fixed order, five
  // dependent adds instead of one per warp)
  double t = 0.0;
  if (warp == 0) {
    t = lane < nwarps ? red[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(full, t, o);
  }
  return tid == 0 ? t : 0.0;
}

}  // namespace gr
