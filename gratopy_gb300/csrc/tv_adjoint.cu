// Elementwise pieces of the adjoint (reverse mode) of one TV primal-dual
// iteration (total_variation.cl:54-167 + gratopy.py:2708-2717).  Forward map
// of one iteration k -> k+1 with state (U, Ubar, V, Lambda):
//   w = V + sigma grad(Ubar);                V'  = w / max(1, |w|)
//   Lambda' = mu2 (Lambda + sigma_l (A Ubar - f))
//   z = U + tau (div V' - n A* Lambda');     U'  = max(0, z);  Ubar' = 2 U' - U
// Given the adjoints (gU, gUbar, gV, gL) of the state k+1 these kernels
// produce, together with two projections (see gr_forward_angle_axpy and
// gr_backward_tv_adjoint), the adjoints of the state k and of f.
#include "gr_internal.cuh"

using namespace gr;

namespace {

constexpr int kBlock = 256;

inline unsigned grid_for(size_t n) {
  size_t b = (n + kBlock - 1) / kBlock;
  if (b > 65535u * 64u) b = 65535u * 64u;
  return (unsigned)(b == 0 ? 1 : b);
}

// gU1 = gU + 2 gUbar;  gz = [U' > 0] gU1;  gU_prev = gz - gUbar.
template <typename T>
__global__ void tv_adj_primal_kernel(T* __restrict__ gz, T* __restrict__ gu_prev,
                                     const T* __restrict__ gu, const T* __restrict__ gubar,
                                     const T* __restrict__ u_next, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const T g1 = gu[i] + (T)2 * gubar[i];
    const T z = u_next[i] > (T)0 ? g1 : (T)0;
    gz[i] = z;
    gu_prev[i] = z - gubar[i];
  }
}

// gV1 = gV - tau grad(gz);  gw = J_P(w)^T gV1 with w = V + sigma grad(Ubar):
// J_P = I inside the unit ball, (I - n n^T)/|w| outside (n = w/|w|).
template <typename T, int O>
__global__ void tv_adj_dual_kernel(T* __restrict__ gw, const T* __restrict__ gv,
                                   const T* __restrict__ gz, const T* __restrict__ v,
                                   const T* __restrict__ ubar, float sigma, float tau,
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
    // forward differences with gratopy's boundary and slice conventions
    T g0, g1, g2, h0, h1, h2;
    {
      const T c = -ubar[i];
      g0 = x < d.Nx - 1 ? c + ubar[i + sx] : (T)0;
      g1 = y < d.Ny - 1 ? c + ubar[i + sy] : (T)0;
      g2 = z < d.Nz - 1 ? c + ubar[i + sz] : (T)0;
      if (z_distance > 0) g2 /= z_distance; else g2 = (T)0;
    }
    {
      const T c = -gz[i];
      h0 = x < d.Nx - 1 ? c + gz[i + sx] : (T)0;
      h1 = y < d.Ny - 1 ? c + gz[i + sy] : (T)0;
      h2 = z < d.Nz - 1 ? c + gz[i + sz] : (T)0;
      if (z_distance > 0) h2 /= z_distance; else h2 = (T)0;
    }
    const T* vp = v + 4 * i;
    const T w0 = vp[0] + sigma * g0, w1 = vp[1] + sigma * g1, w2 = vp[2] + sigma * g2;
    const T* gp = gv + 4 * i;
    const T a0 = gp[0] - tau * h0, a1 = gp[1] - tau * h1, a2 = gp[2] - tau * h2;
    const T nrm = ghypot(ghypot(w0, w1), w2);
    T* op = gw + 4 * i;
    if (nrm > (T)1) {
      const T inv = (T)1 / nrm;
      const T n0 = w0 * inv, n1 = w1 * inv, n2 = w2 * inv;
      const T dot = n0 * a0 + n1 * a1 + n2 * a2;
      op[0] = (a0 - n0 * dot) * inv;
      op[1] = (a1 - n1 * dot) * inv;
      op[2] = (a2 - n2 * dot) * inv;
    } else {
      op[0] = a0;
      op[1] = a1;
      op[2] = a2;
    }
    op[3] = (T)0;
  }
}

// gL_prev = mu2 gL1;  gf += -mu2 sigma_l gL1.
template <typename T>
__global__ void tv_adj_lambda_kernel(T* __restrict__ gl_prev, T* __restrict__ gf,
                                     const T* __restrict__ gl1, float mu2, float sigma_l,
                                     int64_t n) {
  // the product of the two float32 factors in the array precision (a float
  // product would round it)
  const T c = (T)mu2 * (T)sigma_l;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const T g = gl1[i];
    gl_prev[i] = mu2 * g;
    gf[i] -= c * g;
  }
}

}  // namespace

extern "C" {

int gr_tv_adjoint_primal(void* gz, void* gu_prev, const void* gu, const void* gubar,
                         const void* u_next, int dtype, size_t n, void* stream) {
  if (!gz || !gu_prev || !gu || !gubar || !u_next || !valid_dtype(dtype)) return GR_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  if (dtype == GR_F32)
    tv_adj_primal_kernel<float><<<grid_for(n), kBlock, 0, st>>>(
        (float*)gz, (float*)gu_prev, (const float*)gu, (const float*)gubar,
        (const float*)u_next, (int64_t)n);
  else
    tv_adj_primal_kernel<double><<<grid_for(n), kBlock, 0, st>>>(
        (double*)gz, (double*)gu_prev, (const double*)gu, (const double*)gubar,
        (const double*)u_next, (int64_t)n);
  return check_launch();
}

int gr_tv_adjoint_dual(void* gw, const void* gv, const void* gz, const void* v, const void* ubar,
                       float sigma, float tau, float z_distance, int dtype, int Nx, int Ny, int Nz,
                       int order, void* stream) {
  if (!gw || !gv || !gz || !v || !ubar || !valid_dtype(dtype) || !valid_order(order))
    return GR_ERR_ARG;
  if (Nx <= 0 || Ny <= 0 || Nz <= 0) return GR_ERR_SHAPE;
  Dims d{Nx, Ny, Nz, 0, 0};
  const size_t n = (size_t)Nx * Ny * Nz;
  cudaStream_t st = as_stream(stream);
  return dispatch_orders(order, order, [&](auto o, auto) {
    constexpr int O = decltype(o)::value;
    if (dtype == GR_F32)
      tv_adj_dual_kernel<float, O><<<grid_for(n), kBlock, 0, st>>>(
          (float*)gw, (const float*)gv, (const float*)gz, (const float*)v, (const float*)ubar,
          sigma, tau, z_distance, d);
    else
      tv_adj_dual_kernel<double, O><<<grid_for(n), kBlock, 0, st>>>(
          (double*)gw, (const double*)gv, (const double*)gz, (const double*)v,
          (const double*)ubar, sigma, tau, z_distance, d);
    return check_launch();
  });
}

int gr_tv_adjoint_lambda(void* gl_prev, void* gf, const void* gl1, float mu2, float sigma_l,
                         int dtype, size_t n, void* stream) {
  if (!gl_prev || !gf || !gl1 || !valid_dtype(dtype)) return GR_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  if (dtype == GR_F32)
    tv_adj_lambda_kernel<float><<<grid_for(n), kBlock, 0, st>>>(
        (float*)gl_prev, (float*)gf, (const float*)gl1, mu2, sigma_l, (int64_t)n);
  else
    tv_adj_lambda_kernel<double><<<grid_for(n), kBlock, 0, st>>>(
        (double*)gl_prev, (double*)gf, (const double*)gl1, mu2, sigma_l, (int64_t)n);
  return check_launch();
}

}  // extern "C"
