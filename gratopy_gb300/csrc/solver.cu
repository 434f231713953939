// Elementwise, reduction, TV-dual and CG-scalar kernels behind the C ABI.
//
// Reductions are two-stage and deterministic: a fixed grid of
// kDotBlocks blocks accumulates float64 partials with a grid-stride loop
// (warp shuffles + one shared-memory pass per block), and a single block adds
// the partials in a fixed order.  No atomics.
#include "gr_internal.cuh"

using namespace gr;

namespace gr {

static thread_local int g_last_cuda_error = 0;
void set_cuda_error(cudaError_t e) { g_last_cuda_error = (int)e; }

constexpr int kEwBlock = 256;
constexpr int kDotBlocks = 1216;  // 8 x 152 SMs
constexpr int kDotThreads = 256;
constexpr int kSumThreads = 1024;

inline unsigned ew_grid(size_t n) {
  size_t b = (n + kEwBlock - 1) / kEwBlock;
  if (b > 65535u * 64u) b = 65535u * 64u;
  return (unsigned)(b == 0 ? 1 : b);
}

template <typename T>
__global__ void weight_sino_kernel(T* __restrict__ out, const T* __restrict__ sino,
                                   const T* __restrict__ w, Dims d, int order, int divide) {
  const int64_t n = d.Ns * d.Na * d.Nz;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = order == ORDER_F ? (i / d.Ns) % d.Na : (i / d.Nz) % d.Na;
    out[i] = divide ? sino[i] / w[a] : sino[i] * w[a];
  }
}

template <typename T>
__global__ void equ_mul_add_kernel(T* __restrict__ rhs, T a, const T* __restrict__ x, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    rhs[i] += a * x[i];
}

template <typename T>
__global__ void mul_add_add_kernel(T* rhs, T a, const T* x, const T* __restrict__ y, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    rhs[i] = a * x[i] + y[i];
}

// Stage 1 of <a, b> (b == nullptr: plain sum of a).
template <typename T>
__global__ void __launch_bounds__(kDotThreads)
dot_partials_kernel(double* __restrict__ partials, const T* __restrict__ a, const T* __restrict__ b,
                    int64_t n) {
  __shared__ double red[kDotThreads / 32];
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)kDotThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kDotThreads)
    acc += b ? (double)a[i] * (double)b[i] : (double)a[i];
  const double t = block_sum(acc, red);
  if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

// Stage 2: fixed-order sum of n partials by one block.
__device__ double sum_partials_block(const double* __restrict__ partials, int64_t n, double* red) {
  double acc = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) acc += partials[i];
  return block_sum(acc, red);
}

__global__ void __launch_bounds__(kSumThreads)
sum_partials_kernel(double* __restrict__ out, const double* __restrict__ partials, int64_t n) {
  __shared__ double red[kSumThreads / 32];
  const double t = sum_partials_block(partials, n, red);
  if (threadIdx.x == 0) *out = t;
}

// total_variation.cl:54-93 then :150-167 on the same pixel:
// v <- v + sigma grad(u); v <- v / max(1, |v|).
template <typename T, int O>
__global__ void tv_dual_kernel(T* __restrict__ v, const T* __restrict__ u, float sigma,
                               float z_distance, Dims d) {
  const int64_t n = d.Nx * d.Ny * d.Nz;
  int64_t sx, sy, sz;
  img_strides<O>(d, sx, sy, sz);
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    int64_t x, y, z;
    if (O == ORDER_F) {
      x = i % d.Nx;
      y = (i / d.Nx) % d.Ny;
      z = i / (d.Nx * d.Ny);
    } else {
      z = i % d.Nz;
      y = (i / d.Nz) % d.Ny;
      x = i / (d.Nz * d.Ny);
    }
    const T* up = u + i;
    const T c = -up[0];
    T g0 = c, g1 = c, g2 = c;
    if (x < d.Nx - 1) g0 += up[sx]; else g0 = (T)0.;
    if (y < d.Ny - 1) g1 += up[sy]; else g1 = (T)0.;
    if (z < d.Nz - 1) g2 += up[sz]; else g2 = (T)0.;
    if (z_distance > 0) g2 /= z_distance; else g2 = (T)0.;
    T* vp = v + 4 * i;
    T v0 = vp[0] + sigma * g0;
    T v1 = vp[1] + sigma * g1;
    T v2 = vp[2] + sigma * g2;
    const T norm = ghypot(ghypot(v0, v1), v2);
    if (norm > (T)1.) {
      v0 /= norm;
      v1 /= norm;
      v2 /= norm;
    }
    vp[0] = v0;
    vp[1] = v1;
    vp[2] = v2;
  }
}

template <typename T>
__global__ void __launch_bounds__(kSumThreads)
cg_alpha_kernel(double* sc, const double* __restrict__ partials, int64_t n, double c,
                const int* skip) {
  __shared__ double red[kSumThreads / 32];
  pdl_wait();
  pdl_trigger();
  if (skip != nullptr && *skip) return;
  const double qwq = sum_partials_block(partials, n, red);
  if (threadIdx.x == 0) {
    const T alpha = (T)(c * (sc[GR_SC_SOLD] / qwq));
    sc[GR_SC_ALPHA] = (double)alpha;
  }
}

template <typename T>
__global__ void __launch_bounds__(kDotThreads)
cg_update_d_kernel(T* __restrict__ d, const T* __restrict__ q, const double* __restrict__ sc,
                   double* __restrict__ partials, int64_t n, const int* skip) {
  __shared__ double red[kDotThreads / 32];
  pdl_wait();
  pdl_trigger();
  if (skip != nullptr && *skip) return;
  const T na = -(T)sc[GR_SC_ALPHA];
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)kDotThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kDotThreads) {
    const T v = d[i] + na * q[i];
    d[i] = v;
    acc += (double)v * (double)v;
  }
  const double t = block_sum(acc, red);
  if (threadIdx.x == 0) partials[blockIdx.x] = t;
}

template <typename T>
__global__ void __launch_bounds__(kSumThreads)
cg_beta_kernel(double* sc, const double* __restrict__ snew_partials, int64_t n_snew,
               const double* __restrict__ d_partials, int64_t n_d, double epsilon, int* done) {
  __shared__ double red[kSumThreads / 32];
  pdl_wait();
  pdl_trigger();
  if (done != nullptr && *done) return;
  const double snew = sum_partials_block(snew_partials, n_snew, red);
  __syncthreads();
  const double dsq = sum_partials_block(d_partials, n_d, red);
  if (threadIdx.x == 0) {
    const T beta = (T)(snew / sc[GR_SC_SOLD]);
    sc[GR_SC_BETA] = (double)beta;
    sc[GR_SC_SOLD] = snew;
    sc[GR_SC_DSQ] = dsq;
    const double res = sqrt(dsq / sc[GR_SC_FSQ]);
    sc[GR_SC_RES] = res;
    if (done != nullptr && res < epsilon) *done = 1;
  }
}

template <typename T>
__global__ void cg_update_p_kernel(T* p, const T* __restrict__ snew, const double* __restrict__ sc,
                                   int64_t n, const int* skip) {
  pdl_wait();
  pdl_trigger();
  if (skip != nullptr && *skip) return;
  const T beta = (T)sc[GR_SC_BETA];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = beta * p[i] + snew[i];
}

template <typename T>
__global__ void scale_by_sum_kernel(T* img, const double* __restrict__ sc, int64_t n) {
  const T s = (T)sc[GR_SC_SUM];
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    img[i] /= s;
}

}  // namespace gr

extern "C" {

const char* gr_error_string(int code) {
  switch (code) {
    case GR_OK: return "success";
    case GR_ERR_ARG: return "invalid argument (null pointer, dtype, order or geometry kind)";
    case GR_ERR_SHAPE: return "array sizes do not match the geometry";
    case GR_ERR_CUDA: return "CUDA launch or runtime error (see gr_last_cuda_error)";
    case GR_ERR_TOO_BIG: return "size beyond a documented limit";
    default: return "unknown error code";
  }
}

int gr_last_cuda_error(void) { return gr::g_last_cuda_error; }

int gr_version(void) { return 1; }

#ifndef GR_SOURCE_HASH
#define GR_SOURCE_HASH "unknown"
#endif
const char* gr_source_hash(void) { return GR_SOURCE_HASH; }

int gr_weight_sinogram(void* out, const void* sino, const void* w, int dtype, int Ns, int Na,
                       int Nz, int order, int divide, void* stream) {
  if (!out || !sino || !w || !valid_dtype(dtype) || !valid_order(order)) return GR_ERR_ARG;
  if (Ns <= 0 || Na <= 0 || Nz <= 0) return GR_ERR_SHAPE;
  Dims d{0, 0, Nz, Ns, Na};
  const size_t n = (size_t)Ns * Na * Nz;
  cudaStream_t st = as_stream(stream);
  if (dtype == GR_F32)
    weight_sino_kernel<float><<<ew_grid(n), kEwBlock, 0, st>>>(
        (float*)out, (const float*)sino, (const float*)w, d, order, divide);
  else
    weight_sino_kernel<double><<<ew_grid(n), kEwBlock, 0, st>>>(
        (double*)out, (const double*)sino, (const double*)w, d, order, divide);
  return check_launch();
}

int gr_equ_mul_add(void* rhs, double a, const void* x, int dtype, size_t n, void* stream) {
  if (!rhs || !x || !valid_dtype(dtype)) return GR_ERR_ARG;
  if (n == 0) return GR_OK;
  cudaStream_t st = as_stream(stream);
  if (dtype == GR_F32)
    equ_mul_add_kernel<float><<<ew_grid(n), kEwBlock, 0, st>>>((float*)rhs, (float)a,
                                                                (const float*)x, (int64_t)n);
  else
    equ_mul_add_kernel<double><<<ew_grid(n), kEwBlock, 0, st>>>((double*)rhs, a, (const double*)x,
                                                                 (int64_t)n);
  return check_launch();
}

int gr_mul_add_add(void* rhs, double a, const void* x, const void* y, int dtype, size_t n,
                   void* stream) {
  if (!rhs || !x || !y || !valid_dtype(dtype)) return GR_ERR_ARG;
  if (n == 0) return GR_OK;
  cudaStream_t st = as_stream(stream);
  if (dtype == GR_F32)
    mul_add_add_kernel<float><<<ew_grid(n), kEwBlock, 0, st>>>(
        (float*)rhs, (float)a, (const float*)x, (const float*)y, (int64_t)n);
  else
    mul_add_add_kernel<double><<<ew_grid(n), kEwBlock, 0, st>>>(
        (double*)rhs, a, (const double*)x, (const double*)y, (int64_t)n);
  return check_launch();
}

size_t gr_dot_partials_count(void) { return (size_t)kDotBlocks; }

int gr_dot_partials(double* partials, const void* a, const void* b, int dtype, size_t n,
                    void* stream) {
  if (!partials || !a || !b || !valid_dtype(dtype)) return GR_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  if (dtype == GR_F32)
    dot_partials_kernel<float><<<kDotBlocks, kDotThreads, 0, st>>>(partials, (const float*)a,
                                                                   (const float*)b, (int64_t)n);
  else
    dot_partials_kernel<double><<<kDotBlocks, kDotThreads, 0, st>>>(partials, (const double*)a,
                                                                    (const double*)b, (int64_t)n);
  return check_launch();
}

int gr_sum_values_partials(double* partials, const void* a, int dtype, size_t n, void* stream) {
  if (!partials || !a || !valid_dtype(dtype)) return GR_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  if (dtype == GR_F32)
    dot_partials_kernel<float><<<kDotBlocks, kDotThreads, 0, st>>>(partials, (const float*)a,
                                                                   nullptr, (int64_t)n);
  else
    dot_partials_kernel<double><<<kDotBlocks, kDotThreads, 0, st>>>(partials, (const double*)a,
                                                                    nullptr, (int64_t)n);
  return check_launch();
}

int gr_sum_partials(double* out, const double* partials, size_t n, void* stream) {
  if (!out || !partials) return GR_ERR_ARG;
  sum_partials_kernel<<<1, kSumThreads, 0, as_stream(stream)>>>(out, partials, (int64_t)n);
  return check_launch();
}

int gr_tv_dual(void* v, const void* ubar, float sigma, float z_distance, int dtype, int Nx, int Ny,
               int Nz, int order, void* stream) {
  if (!v || !ubar || !valid_dtype(dtype) || !valid_order(order)) return GR_ERR_ARG;
  if (Nx <= 0 || Ny <= 0 || Nz <= 0) return GR_ERR_SHAPE;
  Dims d{Nx, Ny, Nz, 0, 0};
  const size_t n = (size_t)Nx * Ny * Nz;
  cudaStream_t st = as_stream(stream);
  return dispatch_orders(order, order, [&](auto o, auto) {
    constexpr int O = decltype(o)::value;
    if (dtype == GR_F32)
      tv_dual_kernel<float, O><<<ew_grid(n), kEwBlock, 0, st>>>((float*)v, (const float*)ubar,
                                                                 sigma, z_distance, d);
    else
      tv_dual_kernel<double, O><<<ew_grid(n), kEwBlock, 0, st>>>((double*)v, (const double*)ubar,
                                                                  sigma, z_distance, d);
    return check_launch();
  });
}

int gr_cg_alpha(double* sc, const double* partials, size_t n, double c, int dtype, const int* skip,
                void* stream) {
  if (!sc || !partials || !valid_dtype(dtype)) return GR_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  if (dtype == GR_F32)
    launch_pdl(cg_alpha_kernel<float>, dim3(1), dim3(kSumThreads), st, sc, partials, (int64_t)n,
               c, skip);
  else
    launch_pdl(cg_alpha_kernel<double>, dim3(1), dim3(kSumThreads), st, sc, partials, (int64_t)n,
               c, skip);
  return check_launch();
}

int gr_cg_update_d(void* d, const void* q, const double* sc, double* partials, int dtype, size_t n,
                   const int* skip, void* stream) {
  if (!d || !q || !sc || !partials || !valid_dtype(dtype)) return GR_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  if (dtype == GR_F32)
    launch_pdl(cg_update_d_kernel<float>, dim3(kDotBlocks), dim3(kDotThreads), st, (float*)d,
               (const float*)q, sc, partials, (int64_t)n, skip);
  else
    launch_pdl(cg_update_d_kernel<double>, dim3(kDotBlocks), dim3(kDotThreads), st, (double*)d,
               (const double*)q, sc, partials, (int64_t)n, skip);
  return check_launch();
}

int gr_cg_beta(double* sc, const double* snew_partials, size_t n_snew, const double* d_partials,
               size_t n_d, double epsilon, int dtype, int* done, void* stream) {
  if (!sc || !snew_partials || !d_partials || !valid_dtype(dtype)) return GR_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  if (dtype == GR_F32)
    launch_pdl(cg_beta_kernel<float>, dim3(1), dim3(kSumThreads), st, sc, snew_partials,
               (int64_t)n_snew, d_partials, (int64_t)n_d, epsilon, done);
  else
    launch_pdl(cg_beta_kernel<double>, dim3(1), dim3(kSumThreads), st, sc, snew_partials,
               (int64_t)n_snew, d_partials, (int64_t)n_d, epsilon, done);
  return check_launch();
}

int gr_cg_update_p(void* p, const void* snew, const double* sc, int dtype, size_t n,
                   const int* skip, void* stream) {
  if (!p || !snew || !sc || !valid_dtype(dtype)) return GR_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  if (dtype == GR_F32)
    launch_pdl(cg_update_p_kernel<float>, dim3(ew_grid(n)), dim3(kEwBlock), st, (float*)p,
               (const float*)snew, sc, (int64_t)n, skip);
  else
    launch_pdl(cg_update_p_kernel<double>, dim3(ew_grid(n)), dim3(kEwBlock), st, (double*)p,
               (const double*)snew, sc, (int64_t)n, skip);
  return check_launch();
}

int gr_scale_by_sum(void* img, const double* sc, int dtype, size_t n, void* stream) {
  if (!img || !sc || !valid_dtype(dtype)) return GR_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  if (dtype == GR_F32)
    scale_by_sum_kernel<float><<<ew_grid(n), kEwBlock, 0, st>>>((float*)img, sc, (int64_t)n);
  else
    scale_by_sum_kernel<double><<<ew_grid(n), kEwBlock, 0, st>>>((double*)img, sc, (int64_t)n);
  return check_launch();
}

}  // extern "C"
