// Typed projection entry points, explicitly instantiated per precision in
// proj_plain_f32.cu / proj_plain_f64.cu / proj_fused_f32.cu /
// proj_fused_f64.cu and called by the C ABI in capi.cu.
#pragma once

#include "proj_launch.cuh"

namespace gr {

// Plain projections (any order pair).
template <typename T>
int fwd_plain(const gr_geometry* g, void* sino, const void* img, int Nz, int so, int io,
              void* stream);
template <typename T>
int bwd_plain(const gr_geometry* g, void* img, const void* sino, int Nz, int io, int so,
              void* stream);

// Fused solver steps (image and sinogram share `order`).
template <typename T>
int fwd_residual(const gr_geometry* g, void* r, const void* u, const void* f, int Nz, int order,
                 void* stream);
template <typename T>
int bwd_axpy(const gr_geometry* g, void* u, const void* r, double a, int Nz, int order,
             void* stream);
template <typename T>
int fwd_lambda(const gr_geometry* g, void* lambda, const void* u, const void* f, float sigma,
               float mu2, int Nz, int order, void* stream);
template <typename T>
int bwd_tv_primal(const gr_geometry* g, void* u, void* ubar, const void* v, const void* lambda,
                  float tau, float norming, float z_distance, int Nz, int order, void* stream);
template <typename T>
int fwd_wsq(const gr_geometry* g, void* q, const void* p, const void* w, double* partials,
            const int* skip, int Nz, int order, void* stream);
template <typename T>
int bwd_cg(const gr_geometry* g, void* snew, const void* d, void* x, const void* p,
           const double* alpha, double* partials, const int* skip, int Nz, int order,
           void* stream);
template <typename T>
int bwd_sum(const gr_geometry* g, void* img, const void* sino, double* partials, int Nz, int order,
            void* stream);
template <typename T>
int fwd_angle_axpy(const gr_geometry* g, void* out, const void* base, const void* u,
                   const void* w, double c, int Nz, int order, void* stream);
template <typename T>
int bwd_tv_adjoint(const gr_geometry* g, void* out, const void* lambda, const void* gw, double c1,
                   float sigma, float z_distance, int Nz, int order, void* stream);

#ifdef GR_DEFINE_PLAIN
template <typename T>
int fwd_plain(const gr_geometry* g, void* sino, const void* img, int Nz, int so, int io,
              void* stream) {
  return dispatch_orders(so, io, [&](auto so_, auto io_) {
    return launch::launch_fwd<T, decltype(so_)::value, decltype(io_)::value>(
        g, img, Nz, FwdStore<T>{static_cast<T*>(sino)}, nullptr, nullptr, stream);
  });
}

template <typename T>
int bwd_plain(const gr_geometry* g, void* img, const void* sino, int Nz, int io, int so,
              void* stream) {
  return dispatch_orders(io, so, [&](auto io_, auto so_) {
    return launch::launch_bwd<T, decltype(io_)::value, decltype(so_)::value>(
        g, sino, Nz, BwdStore<T>{static_cast<T*>(img)}, nullptr, nullptr, stream);
  });
}
#endif

#ifdef GR_DEFINE_FUSED
template <class F>
inline int dispatch_order(int order, F&& f) {
  if (order == ORDER_F) return f(IC<ORDER_F>{});
  if (order == ORDER_C) return f(IC<ORDER_C>{});
  return GR_ERR_ARG;
}

template <typename T>
int fwd_residual(const gr_geometry* g, void* r, const void* u, const void* f, int Nz, int order,
                 void* stream) {
  return dispatch_order(order, [&](auto o) {
    constexpr int O = decltype(o)::value;
    return launch::launch_fwd<T, O, O>(
        g, u, Nz, FwdResidual<T>{static_cast<T*>(r), static_cast<const T*>(f)}, nullptr, nullptr,
        stream);
  });
}

template <typename T>
int bwd_axpy(const gr_geometry* g, void* u, const void* r, double a, int Nz, int order,
             void* stream) {
  return dispatch_order(order, [&](auto o) {
    constexpr int O = decltype(o)::value;
    return launch::launch_bwd<T, O, O>(g, r, Nz, BwdAxpy<T>{static_cast<T*>(u), (T)a}, nullptr,
                                       nullptr, stream);
  });
}

template <typename T>
int fwd_lambda(const gr_geometry* g, void* lambda, const void* u, const void* f, float sigma,
               float mu2, int Nz, int order, void* stream) {
  return dispatch_order(order, [&](auto o) {
    constexpr int O = decltype(o)::value;
    return launch::launch_fwd<T, O, O>(
        g, u, Nz, FwdLambda<T>{static_cast<T*>(lambda), static_cast<const T*>(f), sigma, mu2},
        nullptr, nullptr, stream);
  });
}

template <typename T>
int bwd_tv_primal(const gr_geometry* g, void* u, void* ubar, const void* v, const void* lambda,
                  float tau, float norming, float z_distance, int Nz, int order, void* stream) {
  const Dims d = launch::dims_of(g, Nz);
  return dispatch_order(order, [&](auto o) {
    constexpr int O = decltype(o)::value;
    BwdTVPrimal<T, O> e{static_cast<T*>(u), static_cast<T*>(ubar), static_cast<const T*>(v), d,
                        tau, norming, z_distance};
    return launch::launch_bwd<T, O, O>(g, lambda, Nz, e, nullptr, nullptr, stream);
  });
}

template <typename T>
int fwd_wsq(const gr_geometry* g, void* q, const void* p, const void* w, double* partials,
            const int* skip, int Nz, int order, void* stream) {
  return dispatch_order(order, [&](auto o) {
    constexpr int O = decltype(o)::value;
    return launch::launch_fwd<T, O, O>(
        g, p, Nz, FwdStoreWeightedSq<T>{static_cast<T*>(q), static_cast<const T*>(w)}, partials,
        skip, stream);
  });
}

template <typename T>
int bwd_cg(const gr_geometry* g, void* snew, const void* d, void* x, const void* p,
           const double* alpha, double* partials, const int* skip, int Nz, int order,
           void* stream) {
  return dispatch_order(order, [&](auto o) {
    constexpr int O = decltype(o)::value;
    return launch::launch_bwd<T, O, O>(
        g, d, Nz,
        BwdCG<T>{static_cast<T*>(snew), static_cast<T*>(x), static_cast<const T*>(p), alpha},
        partials, skip, stream);
  });
}

template <typename T>
int bwd_sum(const gr_geometry* g, void* img, const void* sino, double* partials, int Nz, int order,
            void* stream) {
  return dispatch_order(order, [&](auto o) {
    constexpr int O = decltype(o)::value;
    return launch::launch_bwd<T, O, O>(g, sino, Nz, BwdStoreSum<T>{static_cast<T*>(img)}, partials,
                                       nullptr, stream);
  });
}

template <typename T>
int fwd_angle_axpy(const gr_geometry* g, void* out, const void* base, const void* u,
                   const void* w, double c, int Nz, int order, void* stream) {
  return dispatch_order(order, [&](auto o) {
    constexpr int O = decltype(o)::value;
    return launch::launch_fwd<T, O, O>(
        g, u, Nz,
        FwdAngleAxpy<T>{static_cast<T*>(out), static_cast<const T*>(base),
                        static_cast<const T*>(w), (T)c},
        nullptr, nullptr, stream);
  });
}

template <typename T>
int bwd_tv_adjoint(const gr_geometry* g, void* out, const void* lambda, const void* gw, double c1,
                   float sigma, float z_distance, int Nz, int order, void* stream) {
  const Dims d = launch::dims_of(g, Nz);
  return dispatch_order(order, [&](auto o) {
    constexpr int O = decltype(o)::value;
    BwdTVAdjoint<T, O> e{static_cast<T*>(out), static_cast<const T*>(gw), d, (T)c1, sigma,
                         z_distance};
    return launch::launch_bwd<T, O, O>(g, lambda, Nz, e, nullptr, nullptr, stream);
  });
}
#endif

}  // namespace gr
