// Sparse matrix of the forward projection in one launch.
//
// gratopy builds the matrix column by column: for every pixel it launches a
// "single line" kernel over the whole sinogram (radon.cl:263-341,
// fanbeam.cl:422-568) and keeps the positive entries (gratopy.py:2014-2155),
// Nx*Ny launches and host round trips.  A pixel has positive weight only in
// the (at most) two detector bins around its projected position, so here one
// thread per (pixel, angle) evaluates the single-line formula for those two
// bins and writes two (row, column, value) slots; entries that are not
// positive are written with value 0 and dropped by the caller.
#include "gr_internal.cuh"

using namespace gr;

namespace {

template <int O>
__device__ __forceinline__ int64_t pixel_pos(int64_t x, int64_t y, int64_t Nx, int64_t Ny) {
  return O == ORDER_F ? x + Nx * y : x * Ny + y;
}

template <int O>
__device__ __forceinline__ int64_t sino_pos(int64_t s, int64_t a, int64_t Ns, int64_t Na) {
  return O == ORDER_F ? s + Ns * a : s * Na + a;
}

// radon.cl:263-341 for bin s; 0 when the pixel does not contribute.
template <typename T>
__device__ T radon_single(int x, int y, int s, const T* o8, float delta_x, float delta_xi, int Nx,
                          int Ny) {
  T ox = o8[0], oy = o8[1];
  const T oz = o8[2], ow = o8[3];
  int Nxx = Nx;
  if (o8[5] != (T)0) {
    const T t = ox;
    ox = oy;
    oy = t;
    Nxx = Ny;
    const int ti = x;
    x = y;
    y = ti;
  }
  const T d = (T)y * oy + oz;
  int x_low = (int)(((T)(s - 1) - d) * ow);
  int x_high = (int)(((T)(s + 1) - d) * ow);
  if (ow < (T)0) {
    const int t = x_low;
    x_low = x_high;
    x_high = t;
  }
  x_low = max(x_low, 0);
  x_high = min(x_high, Nxx - 1);
  T acc = (T)0;
  if (x_low <= x && x <= x_high) {
    const T weight = (T)1 - gabs((T)x * ox + d - (T)s);
    if (weight > (T)0) acc = weight;
  }
  return acc * (T)delta_x * (T)delta_x / (T)delta_xi;
}

// fanbeam.cl:422-568 for bin s.
template <typename T>
__device__ T fan_single(int x, int y, int s, const T* o8, const T* sdpd, const double* geo) {
  T midx = (T)geo[3], midy = (T)geo[4];
  const T mid_det = (T)geo[5];
  const T R = (T)geo[0];
  T RE = (T)geo[1];
  const T delta_xi = (T)geo[2];
  const T delta_x = (T)geo[10];
  const int Nx = (int)geo[6], Ny = (int)geo[7];
  T dx = o8[0], dy = o8[1], qx = o8[2], qy = o8[3];
  const T d0x = o8[4], d0y = o8[5];
  T dpx = d0x + dx * (-mid_det + (T)(s + 1)) - qx, dpy = d0y + dy * (-mid_det + (T)(s + 1)) - qy;
  T dmx = d0x + dx * (-mid_det + (T)(s - 1)) - qx, dmy = d0y + dy * (-mid_det + (T)(s - 1)) - qy;
  T ddx = d0x - qx, ddy = d0y - qy;
  ddx /= R * R;
  ddy /= R * R;
  dx /= delta_xi * delta_xi;
  dy /= delta_xi * delta_xi;
  RE *= (T)1 / R;
  int Nxx = Nx;
  if (!(gabs(dpx) < gabs(dpy) && gabs(dmx) < gabs(dmy))) {
    T t;
    t = ddx; ddx = ddy; ddy = t;
    t = dx; dx = dy; dy = t;
    t = qx; qx = qy; qy = t;
    t = dpx; dpx = dpy; dpy = t;
    t = dmx; dmx = dmy; dmy = t;
    t = midx; midx = midy; midy = t;
    Nxx = Ny;
    const int ti = y;
    y = x;
    x = ti;
  }
  dpx /= dpy;
  dmx /= dmy;
  if (qy * (dmx - dpx) < (T)0) {
    const T t = dpx;
    dpx = dmx;
    dmx = t;
  }
  const T xhigh = qx + dpx * ((T)y - midy - qy);
  const T xlow = qx + dmx * ((T)y - midy - qy);
  const int xhighint = (int)gfloor(gmin((T)(Nxx - 1) - midx, xhigh) + midx);
  const int xlowint = (int)gceil(gmax(-midx, xlow) + midx);
  T acc = (T)0;
  if (xlowint <= x && x <= xhighint) {
    const T t = ddx * ((T)x - midx) + ddy * ((T)y - midy) + RE;
    const T ss = dx * ((T)x - midx) + dy * ((T)y - midy);
    const T xi = ss / t;
    acc = ((T)1 - gabs((T)s - xi - mid_det)) / (R * t);
  }
  return acc * sdpd[s] / delta_xi * delta_x;
}

template <typename T, int O>
__global__ void sparse_kernel(int64_t* __restrict__ rows, int64_t* __restrict__ cols,
                              T* __restrict__ vals, const T* __restrict__ ofs,
                              const T* __restrict__ sdpd, gr_geometry g) {
  const int64_t Nx = g.Nx, Ny = g.Ny, Ns = g.Ns, Na = g.Na;
  const int64_t n = Nx * Ny * Na;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t a = i % Na;
    const int64_t p = i / Na;
    const int x = (int)(p % Nx), y = (int)(p / Nx);
    const T* o8 = ofs + 8 * a;
    // the pixel's projected bin position picks the two candidate bins
    int f;
    if (g.kind == GR_RADON) {
      T ox = o8[0], oy = o8[1];
      int xx = x, yy = y;
      if (o8[5] != (T)0) {
        const T t = ox;
        ox = oy;
        oy = t;
        xx = y;
        yy = x;
      }
      f = (int)gfloor((T)xx * ox + ((T)yy * oy + o8[2]));
    } else {
      const T R = (T)g.geo[0], RE = (T)g.geo[1], dxi = (T)g.geo[2];
      const T px = (T)x - (T)g.geo[3], py = (T)y - (T)g.geo[4];
      const T t = ((o8[4] - o8[2]) * px + (o8[5] - o8[3]) * py) / (R * R) + RE / R;
      const T ss = (o8[0] * px + o8[1] * py) / (dxi * dxi);
      f = (int)gfloor(ss / t + (T)g.geo[5]);
    }
    for (int c = 0; c < 2; ++c) {
      const int s = f + c;
      T v = (T)0;
      if (s >= 0 && s < Ns)
        v = g.kind == GR_RADON ? radon_single<T>(x, y, s, o8, (float)g.geo[0], (float)g.geo[1],
                                                 (int)Nx, (int)Ny)
                               : fan_single<T>(x, y, s, o8, sdpd, g.geo);
      const int64_t slot = 2 * i + c;
      rows[slot] = (s >= 0 && s < Ns) ? sino_pos<O>(s, a, Ns, Na) : 0;
      cols[slot] = pixel_pos<O>(x, y, Nx, Ny);
      vals[slot] = v;
    }
  }
}

}  // namespace

extern "C" {

int gr_sparse_entries(const gr_geometry* g, int64_t* rows, int64_t* cols, void* vals, int order,
                      void* stream) {
  if (g == nullptr || rows == nullptr || cols == nullptr || vals == nullptr || g->ofs == nullptr ||
      !valid_order(order) || !valid_dtype(g->dtype) ||
      (g->kind != GR_RADON && g->kind != GR_FANBEAM) || (g->kind == GR_FANBEAM && !g->sdpd))
    return GR_ERR_ARG;
  if (g->Nx <= 0 || g->Ny <= 0 || g->Ns <= 0 || g->Na <= 0) return GR_ERR_SHAPE;
  const int64_t n = (int64_t)g->Nx * g->Ny * g->Na;
  int64_t blocks = (n + 255) / 256;
  if (blocks > 152 * 64) blocks = 152 * 64;
  cudaStream_t st = as_stream(stream);
  return dispatch_orders(order, order, [&](auto o, auto) {
    constexpr int O = decltype(o)::value;
    if (g->dtype == GR_F32)
      sparse_kernel<float, O><<<(unsigned)blocks, 256, 0, st>>>(
          rows, cols, static_cast<float*>(vals), static_cast<const float*>(g->ofs),
          static_cast<const float*>(g->sdpd), *g);
    else
      sparse_kernel<double, O><<<(unsigned)blocks, 256, 0, st>>>(
          rows, cols, static_cast<double*>(vals), static_cast<const double*>(g->ofs),
          static_cast<const double*>(g->sdpd), *g);
    return check_launch();
  });
}

}  // extern "C"
