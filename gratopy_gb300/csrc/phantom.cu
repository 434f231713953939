// Ellipse phantoms rasterised on the device: a stack of Nz slices, each the
// sum of its own K filled ellipses on the grid x = linspace(-1, 1, Nx),
// y = -linspace(-1, 1, Ny) (gratopy phantom.py:159-177).  Every operation is
// an explicitly rounded float64 operation in the order numpy evaluates the
// host rasteriser, so a slice equals the host image bit for bit.
#include "gr_internal.cuh"

using namespace gr;

namespace {

// numpy.linspace(-1, 1, n)[i]: i * (2 / (n - 1)) - 1, the last point exactly 1.
__device__ __forceinline__ double grid_point(int64_t i, int64_t n) {
  if (n == 1) return -1.0;
  if (i == n - 1) return 1.0;
  const double step = __ddiv_rn(2.0, (double)(n - 1));
  return __dadd_rn(__dmul_rn((double)i, step), -1.0);
}

// e: per slice K records (grey, a^2, b^2, xc, yc, cos theta, sin theta)
template <typename T, int O>
__global__ void ellipses_kernel(T* __restrict__ img, const double* __restrict__ e, int K, Dims d) {
  const int64_t n = d.Nx * d.Ny * d.Nz;
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
    const double X = grid_point(x, d.Nx);
    const double Y = -grid_point(y, d.Ny);
    const double* r = e + (int64_t)7 * K * z;
    double acc = 0.0;
    for (int k = 0; k < K; ++k, r += 7) {
      const double dx = __dsub_rn(X, r[3]), dy = __dsub_rn(Y, r[4]);
      const double u = __dadd_rn(__dmul_rn(dx, r[5]), __dmul_rn(dy, r[6]));
      const double v = __dsub_rn(__dmul_rn(dx, r[6]), __dmul_rn(dy, r[5]));
      const double q = __dadd_rn(__ddiv_rn(__dmul_rn(u, u), r[1]), __ddiv_rn(__dmul_rn(v, v), r[2]));
      if (q <= 1.0) acc = __dadd_rn(acc, r[0]);
    }
    img[i] = (T)acc;
  }
}

}  // namespace

extern "C" {

int gr_ellipses(void* img, const double* ellipses, int K, int Nx, int Ny, int Nz, int dtype,
                int order, void* stream) {
  if (img == nullptr || (K > 0 && ellipses == nullptr) || K < 0 || !valid_dtype(dtype) ||
      !valid_order(order))
    return GR_ERR_ARG;
  if (Nx <= 0 || Ny <= 0 || Nz <= 0) return GR_ERR_SHAPE;
  Dims d{Nx, Ny, Nz, 0, 0};
  const int64_t n = (int64_t)Nx * Ny * Nz;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 64) blocks = 152 * 64;
  cudaStream_t st = as_stream(stream);
  return dispatch_orders(order, order, [&](auto o, auto) {
    constexpr int O = decltype(o)::value;
    if (dtype == GR_F32)
      ellipses_kernel<float, O><<<(unsigned)blocks, 256, 0, st>>>((float*)img, ellipses, K, d);
    else
      ellipses_kernel<double, O><<<(unsigned)blocks, 256, 0, st>>>((double*)img, ellipses, K, d);
    return check_launch();
  });
}

}  // extern "C"
