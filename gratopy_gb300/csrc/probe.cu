// Load-bandwidth probe of the L1 data path, the denominator of the gather
// roofline of the projection kernels (their operand loads hit L1/L2, not
// HBM).  Every thread streams float4 loads over a buffer small enough to
// stay resident in each SM's L1 and folds them into one sum, so the loads
// cannot be removed; bytes moved = blocks x threads x iterations x 16.
#include "gr_internal.cuh"

using namespace gr;

namespace {

constexpr int kProbeThreads = 256;

__global__ void __launch_bounds__(kProbeThreads)
l1_probe_kernel(float* __restrict__ out, const float4* __restrict__ buf, int n_vec, int iters) {
  const int mask = n_vec - 1;  // n_vec is a power of two
  int k = (threadIdx.x + blockIdx.x * 7) & mask;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll 8
  for (int it = 0; it < iters; ++it) {
    const float4 v = __ldg(buf + k);
    acc.x += v.x;
    acc.y += v.y;
    acc.z += v.z;
    acc.w += v.w;
    k = (k + kProbeThreads) & mask;
  }
  const float s = acc.x + acc.y + acc.z + acc.w;
  if (s == 1.2345f) out[blockIdx.x * kProbeThreads + threadIdx.x] = s;  // never true for the probe's zeros
}

}  // namespace

extern "C" {

int gr_probe_l1_bandwidth(float* out, const void* buf, int n_vec, int iters, int blocks,
                          void* stream) {
  if (out == nullptr || buf == nullptr || n_vec <= 0 || (n_vec & (n_vec - 1)) != 0 || iters <= 0 ||
      blocks <= 0)
    return GR_ERR_ARG;
  l1_probe_kernel<<<blocks, kProbeThreads, 0, as_stream(stream)>>>(
      out, static_cast<const float4*>(buf), n_vec, iters);
  return check_launch();
}

}  // extern "C"
