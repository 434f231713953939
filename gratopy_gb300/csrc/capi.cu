// C ABI of the projection entry points (include/gratopy_gb300.h): argument
// validation and dispatch on precision to the typed launchers.
#include "proj_impl.cuh"

using namespace gr;

namespace {

inline bool same_order_ok(const gr_geometry* g, int order) {
  return g != nullptr && valid_order(order) && valid_dtype(g->dtype);
}

}  // namespace

extern "C" {

int gr_forward(const gr_geometry* g, void* sino, const void* img, int Nz, int sino_order,
               int img_order, void* stream) {
  if (g == nullptr || sino == nullptr) return GR_ERR_ARG;
  if (!valid_order(sino_order) || !valid_order(img_order)) return GR_ERR_ARG;
  if (g->dtype == GR_F32) return fwd_plain<float>(g, sino, img, Nz, sino_order, img_order, stream);
  if (g->dtype == GR_F64) return fwd_plain<double>(g, sino, img, Nz, sino_order, img_order, stream);
  return GR_ERR_ARG;
}

int gr_backward(const gr_geometry* g, void* img, const void* sino, int Nz, int img_order,
                int sino_order, void* stream) {
  if (g == nullptr || img == nullptr) return GR_ERR_ARG;
  if (!valid_order(sino_order) || !valid_order(img_order)) return GR_ERR_ARG;
  if (g->dtype == GR_F32) return bwd_plain<float>(g, img, sino, Nz, img_order, sino_order, stream);
  if (g->dtype == GR_F64) return bwd_plain<double>(g, img, sino, Nz, img_order, sino_order, stream);
  return GR_ERR_ARG;
}

int gr_radon_fwd(void* sino, const void* img, const void* ofs, const double* geo, int dtype,
                 int Ns, int Na, int Nz, int sino_order, int img_order, void* stream) {
  if (geo == nullptr) return GR_ERR_ARG;
  gr_geometry g = launch::make_geo(GR_RADON, dtype, ofs, nullptr, geo);
  if (Ns != g.Ns || Na != g.Na) return GR_ERR_SHAPE;
  return gr_forward(&g, sino, img, Nz, sino_order, img_order, stream);
}

int gr_radon_bwd(void* img, const void* sino, const void* ofs, const double* geo, int dtype,
                 int Nx, int Ny, int Nz, int img_order, int sino_order, void* stream) {
  if (geo == nullptr) return GR_ERR_ARG;
  gr_geometry g = launch::make_geo(GR_RADON, dtype, ofs, nullptr, geo);
  if (Nx != g.Nx || Ny != g.Ny) return GR_ERR_SHAPE;
  return gr_backward(&g, img, sino, Nz, img_order, sino_order, stream);
}

int gr_fan_fwd(void* sino, const void* img, const void* ofs, const void* sdpd, const double* geo,
               int dtype, int Ns, int Na, int Nz, int sino_order, int img_order, void* stream) {
  if (geo == nullptr) return GR_ERR_ARG;
  gr_geometry g = launch::make_geo(GR_FANBEAM, dtype, ofs, sdpd, geo);
  if (Ns != g.Ns || Na != g.Na) return GR_ERR_SHAPE;
  return gr_forward(&g, sino, img, Nz, sino_order, img_order, stream);
}

int gr_fan_bwd(void* img, const void* sino, const void* ofs, const void* sdpd, const double* geo,
               int dtype, int Nx, int Ny, int Nz, int img_order, int sino_order, void* stream) {
  if (geo == nullptr) return GR_ERR_ARG;
  gr_geometry g = launch::make_geo(GR_FANBEAM, dtype, ofs, sdpd, geo);
  if (Nx != g.Nx || Ny != g.Ny) return GR_ERR_SHAPE;
  return gr_backward(&g, img, sino, Nz, img_order, sino_order, stream);
}

size_t gr_work_bytes(const gr_geometry* g, int Nz) {
  if (Nz <= 0 || launch::check_geometry(g) != GR_OK) return 0;
  return launch::orbit_work_bytes(g, Nz);
}

int gr_orbit_kinds(const gr_geometry* g, int Nz) {
  if (g == nullptr || Nz <= 0 || launch::check_geometry(g) != GR_OK) return 0;
  int k = 0;
  if (launch::use_quarter(g, Nz) || launch::use_radon_orbit_fwd(g, Nz)) k |= 1;
  if (launch::use_quarter_bwd(g, Nz) || launch::use_radon_orbit_bwd(g, Nz)) k |= 2;
  return k;
}

size_t gr_geometry_size(void) { return sizeof(gr_geometry); }

size_t gr_forward_partials(const gr_geometry* g, int Nz) {
  if (g == nullptr || Nz <= 0) return 0;
  const dim3 grid = launch::fwd_grid(g, Nz, launch::fwd_split(g, Nz));
  return (size_t)grid.x * grid.y * grid.z;
}

size_t gr_backward_partials(const gr_geometry* g, int Nz, int order) {
  if (g == nullptr || Nz <= 0 || !valid_order(order)) return 0;
  const dim3 grid = launch::bwd_grid(g, Nz, order, launch::bwd_split(g, Nz));
  return (size_t)grid.x * grid.y * grid.z;
}

#define GR_TYPED(call_f32, call_f64) \
  (g->dtype == GR_F32 ? (call_f32) : (call_f64))

int gr_forward_residual(const gr_geometry* g, void* r, const void* u, const void* f, int Nz,
                        int order, void* stream) {
  if (!same_order_ok(g, order) || r == nullptr || f == nullptr) return GR_ERR_ARG;
  return GR_TYPED(fwd_residual<float>(g, r, u, f, Nz, order, stream),
                  fwd_residual<double>(g, r, u, f, Nz, order, stream));
}

int gr_backward_axpy(const gr_geometry* g, void* u, const void* r, double a, int Nz, int order,
                     void* stream) {
  if (!same_order_ok(g, order) || u == nullptr) return GR_ERR_ARG;
  return GR_TYPED(bwd_axpy<float>(g, u, r, a, Nz, order, stream),
                  bwd_axpy<double>(g, u, r, a, Nz, order, stream));
}

int gr_forward_lambda(const gr_geometry* g, void* lambda, const void* u, const void* f,
                      float sigma, float mu2, int Nz, int order, void* stream) {
  if (!same_order_ok(g, order) || lambda == nullptr || f == nullptr) return GR_ERR_ARG;
  return GR_TYPED(fwd_lambda<float>(g, lambda, u, f, sigma, mu2, Nz, order, stream),
                  fwd_lambda<double>(g, lambda, u, f, sigma, mu2, Nz, order, stream));
}

int gr_backward_tv_primal(const gr_geometry* g, void* u, void* ubar, const void* v,
                          const void* lambda, float tau, float norming, float z_distance, int Nz,
                          int order, void* stream) {
  if (!same_order_ok(g, order) || u == nullptr || ubar == nullptr || v == nullptr)
    return GR_ERR_ARG;
  return GR_TYPED(
      bwd_tv_primal<float>(g, u, ubar, v, lambda, tau, norming, z_distance, Nz, order, stream),
      bwd_tv_primal<double>(g, u, ubar, v, lambda, tau, norming, z_distance, Nz, order, stream));
}

int gr_forward_wsq(const gr_geometry* g, void* q, const void* p, const void* w, double* partials,
                   const int* skip, int Nz, int order, void* stream) {
  if (!same_order_ok(g, order) || q == nullptr || w == nullptr || partials == nullptr)
    return GR_ERR_ARG;
  return GR_TYPED(fwd_wsq<float>(g, q, p, w, partials, skip, Nz, order, stream),
                  fwd_wsq<double>(g, q, p, w, partials, skip, Nz, order, stream));
}

int gr_backward_cg(const gr_geometry* g, void* snew, const void* d, void* x, const void* p,
                   const double* alpha, double* partials, const int* skip, int Nz, int order,
                   void* stream) {
  if (!same_order_ok(g, order) || snew == nullptr || x == nullptr || p == nullptr ||
      alpha == nullptr || partials == nullptr)
    return GR_ERR_ARG;
  return GR_TYPED(bwd_cg<float>(g, snew, d, x, p, alpha, partials, skip, Nz, order, stream),
                  bwd_cg<double>(g, snew, d, x, p, alpha, partials, skip, Nz, order, stream));
}

int gr_backward_sum(const gr_geometry* g, void* img, const void* sino, double* partials, int Nz,
                    int order, void* stream) {
  if (!same_order_ok(g, order) || img == nullptr || partials == nullptr) return GR_ERR_ARG;
  return GR_TYPED(bwd_sum<float>(g, img, sino, partials, Nz, order, stream),
                  bwd_sum<double>(g, img, sino, partials, Nz, order, stream));
}

int gr_forward_angle_axpy(const gr_geometry* g, void* out, const void* base, const void* u,
                          const void* w, double c, int Nz, int order, void* stream) {
  if (!same_order_ok(g, order) || out == nullptr || u == nullptr || w == nullptr) return GR_ERR_ARG;
  return GR_TYPED(fwd_angle_axpy<float>(g, out, base, u, w, c, Nz, order, stream),
                  fwd_angle_axpy<double>(g, out, base, u, w, c, Nz, order, stream));
}

int gr_backward_tv_adjoint(const gr_geometry* g, void* out, const void* lambda, const void* gw,
                           double c1, float sigma, float z_distance, int Nz, int order,
                           void* stream) {
  if (!same_order_ok(g, order) || out == nullptr || lambda == nullptr || gw == nullptr)
    return GR_ERR_ARG;
  return GR_TYPED(
      bwd_tv_adjoint<float>(g, out, lambda, gw, c1, sigma, z_distance, Nz, order, stream),
      bwd_tv_adjoint<double>(g, out, lambda, gw, c1, sigma, z_distance, Nz, order, stream));
}

}  // extern "C"
