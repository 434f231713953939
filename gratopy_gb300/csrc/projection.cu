// Launchers and C ABI for the projection kernels (plain and fused).
#include <cstdio>

#include "gr_internal.cuh"
#include "projection.cuh"

using namespace gr;

namespace {

int check_geometry(const gr_geometry* g) {
  if (g == nullptr || g->ofs == nullptr) return GR_ERR_ARG;
  if (g->kind != GR_RADON && g->kind != GR_FANBEAM) return GR_ERR_ARG;
  if (!valid_dtype(g->dtype)) return GR_ERR_ARG;
  if (g->kind == GR_FANBEAM && g->sdpd == nullptr) return GR_ERR_ARG;
  if (g->Nx <= 0 || g->Ny <= 0 || g->Ns <= 0 || g->Na <= 0) return GR_ERR_SHAPE;
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
RadonGeo<T> radon_geo(const double* geo) {
  RadonGeo<T> r;
  r.delta_x = (float)geo[0];
  r.delta_xi = (float)geo[1];
  return r;
}

template <typename T>
FanGeo<T> fan_geo(const double* geo) {
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

inline dim3 fwd_grid(const gr_geometry* g, int Nz) {
  const int ZB = zblock(Nz);
  return dim3((g->Ns + kFwdBlock - 1) / kFwdBlock, g->Na, (Nz + ZB - 1) / ZB);
}

inline dim3 bwd_grid(const gr_geometry* g, int Nz, int io) {
  const int ZB = zblock(Nz);
  const int fast = io == ORDER_F ? g->Nx : g->Ny;
  const int slow = io == ORDER_F ? g->Ny : g->Nx;
  return dim3((fast + kBwdTileFast - 1) / kBwdTileFast, (slow + kBwdTileSlow - 1) / kBwdTileSlow,
              (Nz + ZB - 1) / ZB);
}

template <typename T, int SO, int IO, int ZB, class Epi>
int launch_fwd_zb(const gr_geometry* g, const T* img, int Nz, Epi epi, double* partials,
                  const int* skip, cudaStream_t st) {
  const Dims d = dims_of(g, Nz);
  const dim3 grid = fwd_grid(g, Nz);
  if (g->kind == GR_RADON) {
    radon_fwd_kernel<T, SO, IO, ZB, Epi><<<grid, kFwdBlock, 0, st>>>(
        img, static_cast<const T*>(g->ofs), radon_geo<T>(g->geo), d, epi, partials, skip);
  } else {
    fan_fwd_kernel<T, SO, IO, ZB, Epi><<<grid, kFwdBlock, 0, st>>>(
        img, static_cast<const T*>(g->ofs), static_cast<const T*>(g->sdpd), fan_geo<T>(g->geo), d,
        epi, partials, skip);
  }
  return check_launch();
}

template <typename T, int SO, int IO, class Epi>
int launch_fwd(const gr_geometry* g, const void* img, int Nz, Epi epi, double* partials,
               const int* skip, void* stream) {
  int rc = check_geometry(g);
  if (rc) return rc;
  if (img == nullptr || Nz <= 0) return GR_ERR_ARG;
  if ((Nz + 3) / 4 > 65535) return GR_ERR_TOO_BIG;
  const T* im = static_cast<const T*>(img);
  if (Nz == 1) return launch_fwd_zb<T, SO, IO, 1>(g, im, Nz, epi, partials, skip, as_stream(stream));
  return launch_fwd_zb<T, SO, IO, 4>(g, im, Nz, epi, partials, skip, as_stream(stream));
}

template <typename T, int IO, int SO, int ZB, class Epi>
int launch_bwd_zb(const gr_geometry* g, const T* sino, int Nz, Epi epi, double* partials,
                  const int* skip, cudaStream_t st) {
  const Dims d = dims_of(g, Nz);
  const dim3 grid = bwd_grid(g, Nz, IO);
  const dim3 block(kBwdTileFast, kBwdTileSlow);
  if (g->kind == GR_RADON) {
    radon_bwd_kernel<T, IO, SO, ZB, Epi><<<grid, block, 0, st>>>(
        sino, static_cast<const T*>(g->ofs), d, epi, partials, skip);
  } else {
    fan_bwd_kernel<T, IO, SO, ZB, Epi><<<grid, block, 0, st>>>(
        sino, static_cast<const T*>(g->ofs), static_cast<const T*>(g->sdpd), fan_geo<T>(g->geo), d,
        epi, partials, skip);
  }
  return check_launch();
}

template <typename T, int IO, int SO, class Epi>
int launch_bwd(const gr_geometry* g, const void* sino, int Nz, Epi epi, double* partials,
               const int* skip, void* stream) {
  int rc = check_geometry(g);
  if (rc) return rc;
  if (sino == nullptr || Nz <= 0) return GR_ERR_ARG;
  if ((Nz + 3) / 4 > 65535) return GR_ERR_TOO_BIG;
  const T* sn = static_cast<const T*>(sino);
  if (Nz == 1) return launch_bwd_zb<T, IO, SO, 1>(g, sn, Nz, epi, partials, skip, as_stream(stream));
  return launch_bwd_zb<T, IO, SO, 4>(g, sn, Nz, epi, partials, skip, as_stream(stream));
}

// Fills a gr_geometry from the reference-style argument list.
gr_geometry make_geo(int kind, int dtype, const void* ofs, const void* sdpd, const double* geo) {
  gr_geometry g;
  g.kind = kind;
  g.dtype = dtype;
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

}  // namespace

extern "C" {

int gr_forward(const gr_geometry* g, void* sino, const void* img, int Nz, int sino_order,
               int img_order, void* stream) {
  if (g == nullptr || sino == nullptr) return GR_ERR_ARG;
  if (!valid_order(sino_order) || !valid_order(img_order)) return GR_ERR_ARG;
  return dispatch_orders(sino_order, img_order, [&](auto so, auto io) {
    if (g->dtype == GR_F32)
      return launch_fwd<float, decltype(so)::value, decltype(io)::value>(g, img, Nz, FwdStore<float>{static_cast<float*>(sino)},
                                           nullptr, nullptr, stream);
    return launch_fwd<double, decltype(so)::value, decltype(io)::value>(g, img, Nz, FwdStore<double>{static_cast<double*>(sino)},
                                          nullptr, nullptr, stream);
  });
}

int gr_backward(const gr_geometry* g, void* img, const void* sino, int Nz, int img_order,
                int sino_order, void* stream) {
  if (g == nullptr || img == nullptr) return GR_ERR_ARG;
  if (!valid_order(sino_order) || !valid_order(img_order)) return GR_ERR_ARG;
  return dispatch_orders(img_order, sino_order, [&](auto io, auto so) {
    if (g->dtype == GR_F32)
      return launch_bwd<float, decltype(io)::value, decltype(so)::value>(g, sino, Nz, BwdStore<float>{static_cast<float*>(img)},
                                           nullptr, nullptr, stream);
    return launch_bwd<double, decltype(io)::value, decltype(so)::value>(g, sino, Nz, BwdStore<double>{static_cast<double*>(img)},
                                          nullptr, nullptr, stream);
  });
}

int gr_radon_fwd(void* sino, const void* img, const void* ofs, const double* geo, int dtype,
                 int Ns, int Na, int Nz, int sino_order, int img_order, void* stream) {
  if (geo == nullptr) return GR_ERR_ARG;
  gr_geometry g = make_geo(GR_RADON, dtype, ofs, nullptr, geo);
  if (Ns != g.Ns || Na != g.Na) return GR_ERR_SHAPE;
  return gr_forward(&g, sino, img, Nz, sino_order, img_order, stream);
}

int gr_radon_bwd(void* img, const void* sino, const void* ofs, const double* geo, int dtype,
                 int Nx, int Ny, int Nz, int img_order, int sino_order, void* stream) {
  if (geo == nullptr) return GR_ERR_ARG;
  gr_geometry g = make_geo(GR_RADON, dtype, ofs, nullptr, geo);
  if (Nx != g.Nx || Ny != g.Ny) return GR_ERR_SHAPE;
  return gr_backward(&g, img, sino, Nz, img_order, sino_order, stream);
}

int gr_fan_fwd(void* sino, const void* img, const void* ofs, const void* sdpd, const double* geo,
               int dtype, int Ns, int Na, int Nz, int sino_order, int img_order, void* stream) {
  if (geo == nullptr) return GR_ERR_ARG;
  gr_geometry g = make_geo(GR_FANBEAM, dtype, ofs, sdpd, geo);
  if (Ns != g.Ns || Na != g.Na) return GR_ERR_SHAPE;
  return gr_forward(&g, sino, img, Nz, sino_order, img_order, stream);
}

int gr_fan_bwd(void* img, const void* sino, const void* ofs, const void* sdpd, const double* geo,
               int dtype, int Nx, int Ny, int Nz, int img_order, int sino_order, void* stream) {
  if (geo == nullptr) return GR_ERR_ARG;
  gr_geometry g = make_geo(GR_FANBEAM, dtype, ofs, sdpd, geo);
  if (Nx != g.Nx || Ny != g.Ny) return GR_ERR_SHAPE;
  return gr_backward(&g, img, sino, Nz, img_order, sino_order, stream);
}

size_t gr_forward_partials(const gr_geometry* g, int Nz) {
  if (g == nullptr || Nz <= 0) return 0;
  const dim3 grid = fwd_grid(g, Nz);
  return (size_t)grid.x * grid.y * grid.z;
}

size_t gr_backward_partials(const gr_geometry* g, int Nz, int order) {
  if (g == nullptr || Nz <= 0 || !valid_order(order)) return 0;
  const dim3 grid = bwd_grid(g, Nz, order);
  return (size_t)grid.x * grid.y * grid.z;
}

int gr_forward_residual(const gr_geometry* g, void* r, const void* u, const void* f, int Nz,
                        int order, void* stream) {
  if (g == nullptr || r == nullptr || f == nullptr || !valid_order(order)) return GR_ERR_ARG;
  return dispatch_orders(order, order, [&](auto so, auto io) {
    if (g->dtype == GR_F32)
      return launch_fwd<float, decltype(so)::value, decltype(io)::value>(
          g, u, Nz, FwdResidual<float>{static_cast<float*>(r), static_cast<const float*>(f)},
          nullptr, nullptr, stream);
    return launch_fwd<double, decltype(so)::value, decltype(io)::value>(
        g, u, Nz, FwdResidual<double>{static_cast<double*>(r), static_cast<const double*>(f)},
        nullptr, nullptr, stream);
  });
}

int gr_backward_axpy(const gr_geometry* g, void* u, const void* r, double a, int Nz, int order,
                     void* stream) {
  if (g == nullptr || u == nullptr || !valid_order(order)) return GR_ERR_ARG;
  return dispatch_orders(order, order, [&](auto io, auto so) {
    if (g->dtype == GR_F32)
      return launch_bwd<float, decltype(io)::value, decltype(so)::value>(g, r, Nz, BwdAxpy<float>{static_cast<float*>(u), (float)a},
                                           nullptr, nullptr, stream);
    return launch_bwd<double, decltype(io)::value, decltype(so)::value>(g, r, Nz, BwdAxpy<double>{static_cast<double*>(u), a},
                                          nullptr, nullptr, stream);
  });
}

int gr_forward_lambda(const gr_geometry* g, void* lambda, const void* u, const void* f,
                      float sigma, float mu2, int Nz, int order, void* stream) {
  if (g == nullptr || lambda == nullptr || f == nullptr || !valid_order(order)) return GR_ERR_ARG;
  return dispatch_orders(order, order, [&](auto so, auto io) {
    if (g->dtype == GR_F32)
      return launch_fwd<float, decltype(so)::value, decltype(io)::value>(
          g, u, Nz,
          FwdLambda<float>{static_cast<float*>(lambda), static_cast<const float*>(f), sigma, mu2},
          nullptr, nullptr, stream);
    return launch_fwd<double, decltype(so)::value, decltype(io)::value>(
        g, u, Nz,
        FwdLambda<double>{static_cast<double*>(lambda), static_cast<const double*>(f), sigma, mu2},
        nullptr, nullptr, stream);
  });
}

int gr_backward_tv_primal(const gr_geometry* g, void* u, void* ubar, const void* v,
                          const void* lambda, float tau, float norming, float z_distance, int Nz,
                          int order, void* stream) {
  if (g == nullptr || u == nullptr || ubar == nullptr || v == nullptr || !valid_order(order))
    return GR_ERR_ARG;
  const Dims d = dims_of(g, Nz);
  return dispatch_orders(order, order, [&](auto io, auto so) {
    if (g->dtype == GR_F32) {
      BwdTVPrimal<float, decltype(io)::value> e{static_cast<float*>(u), static_cast<float*>(ubar),
                                 static_cast<const float*>(v), d, tau, norming, z_distance};
      return launch_bwd<float, decltype(io)::value, decltype(so)::value>(g, lambda, Nz, e, nullptr, nullptr, stream);
    }
    BwdTVPrimal<double, decltype(io)::value> e{static_cast<double*>(u), static_cast<double*>(ubar),
                                static_cast<const double*>(v), d, tau, norming, z_distance};
    return launch_bwd<double, decltype(io)::value, decltype(so)::value>(g, lambda, Nz, e, nullptr, nullptr, stream);
  });
}

int gr_forward_wsq(const gr_geometry* g, void* q, const void* p, const void* w, double* partials,
                   const int* skip, int Nz, int order, void* stream) {
  if (g == nullptr || q == nullptr || w == nullptr || partials == nullptr || !valid_order(order))
    return GR_ERR_ARG;
  return dispatch_orders(order, order, [&](auto so, auto io) {
    if (g->dtype == GR_F32)
      return launch_fwd<float, decltype(so)::value, decltype(io)::value>(
          g, p, Nz,
          FwdStoreWeightedSq<float>{static_cast<float*>(q), static_cast<const float*>(w)},
          partials, skip, stream);
    return launch_fwd<double, decltype(so)::value, decltype(io)::value>(
        g, p, Nz,
        FwdStoreWeightedSq<double>{static_cast<double*>(q), static_cast<const double*>(w)},
        partials, skip, stream);
  });
}

int gr_backward_cg(const gr_geometry* g, void* snew, const void* d, void* x, const void* p,
                   const double* alpha, double* partials, const int* skip, int Nz, int order,
                   void* stream) {
  if (g == nullptr || snew == nullptr || x == nullptr || p == nullptr || alpha == nullptr ||
      partials == nullptr || !valid_order(order))
    return GR_ERR_ARG;
  return dispatch_orders(order, order, [&](auto io, auto so) {
    if (g->dtype == GR_F32)
      return launch_bwd<float, decltype(io)::value, decltype(so)::value>(
          g, d, Nz,
          BwdCG<float>{static_cast<float*>(snew), static_cast<float*>(x),
                       static_cast<const float*>(p), alpha},
          partials, skip, stream);
    return launch_bwd<double, decltype(io)::value, decltype(so)::value>(
        g, d, Nz,
        BwdCG<double>{static_cast<double*>(snew), static_cast<double*>(x),
                      static_cast<const double*>(p), alpha},
        partials, skip, stream);
  });
}

int gr_backward_sum(const gr_geometry* g, void* img, const void* sino, double* partials, int Nz,
                    int order, void* stream) {
  if (g == nullptr || img == nullptr || partials == nullptr || !valid_order(order))
    return GR_ERR_ARG;
  return dispatch_orders(order, order, [&](auto io, auto so) {
    if (g->dtype == GR_F32)
      return launch_bwd<float, decltype(io)::value, decltype(so)::value>(g, sino, Nz, BwdStoreSum<float>{static_cast<float*>(img)},
                                           partials, nullptr, stream);
    return launch_bwd<double, decltype(io)::value, decltype(so)::value>(g, sino, Nz,
                                          BwdStoreSum<double>{static_cast<double*>(img)}, partials,
                                          nullptr, stream);
  });
}

}  // extern "C"
