// Allocation-free variant of the CG forward step (q = A p and <W q, q>).
//
// Some callers cannot call cudaMalloc at the point where they need this
// step: code running while its stream is being captured into a CUDA graph
// (allocation is not a capturable operation), hosts whose device memory is
// owned and budgeted by another allocator, and latency-critical loops that
// cannot afford cudaMalloc's implicit device synchronisation.  For them,
// gr_forward_wsq_noalloc keeps the per-block partial sums of the reduction
// in a fixed device array of this library instead of caller-provided
// scratch.  The caller still passes its inputs and outputs.
#include <mutex>

#include "proj_impl.cuh"

namespace {

// Per-block partial sums: at most kMaxPartials doubles (512 KiB), resident on
// every GPU that loads this library until the process exits.  Every call
// shares this array and leaves its partials in it; calls that overlap on the
// GPU (concurrent streams, or several host threads) race on it.
constexpr size_t kMaxPartials = 65536;
__device__ __align__(256) double g_wsq_partials[kMaxPartials];

// Device address of g_wsq_partials, looked up once per device and kept for
// the life of the process.  In host code the symbol name is only a host-side
// stand-in, so kernels are always given this looked-up address.  A
// cudaDeviceReset destroys the context the address belongs to, and the kept
// address is not looked up again: this entry point must not be called on a
// device after a reset of that device.
constexpr int kMaxDevices = 64;
double* g_partials_addr[kMaxDevices] = {nullptr};
std::mutex g_setup_mutex;

int partials_address(double** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    gr::set_cuda_error(e);
    return GR_ERR_CUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) return GR_ERR_TOO_BIG;
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (g_partials_addr[dev] == nullptr) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_wsq_partials);
    if (e != cudaSuccess || p == nullptr) {
      gr::set_cuda_error(e);
      return GR_ERR_CUDA;
    }
    g_partials_addr[dev] = static_cast<double*>(p);
  }
  *out = g_partials_addr[dev];
  return GR_OK;
}

}  // namespace

extern "C" {

int gr_forward_wsq_noalloc(const gr_geometry* g, void* q, const void* p, const void* w,
                           double* out, int Nz, int order, void* stream) {
  if (g == nullptr || q == nullptr || p == nullptr || w == nullptr || out == nullptr ||
      !gr::valid_order(order) || !gr::valid_dtype(g->dtype))
    return GR_ERR_ARG;
  // sizes first: the partial count below is only meaningful for a valid geometry
  const int geo_rc = gr::launch::check_geometry(g);
  if (geo_rc != GR_OK) return geo_rc;
  if (Nz <= 0) return GR_ERR_SHAPE;
  const size_t n = gr_forward_partials(g, Nz);
  if (n == 0) return GR_ERR_ARG;
  if (n > kMaxPartials) return GR_ERR_TOO_BIG;
  double* partials = nullptr;
  int rc = partials_address(&partials);
  if (rc != GR_OK) return rc;
  rc = g->dtype == GR_F32
           ? gr::fwd_wsq<float>(g, q, p, w, partials, nullptr, Nz, order, stream)
           : gr::fwd_wsq<double>(g, q, p, w, partials, nullptr, Nz, order, stream);
  if (rc != GR_OK) return rc;
  return gr_sum_partials(out, partials, n, stream);
}

}  // extern "C"
