// Projections with fused solver epilogues, double instantiation.
#define GR_DEFINE_FUSED
#include "proj_impl.cuh"

namespace gr {
template int fwd_residual<double>(const gr_geometry*, void*, const void*, const void*, int, int, void*);
template int bwd_axpy<double>(const gr_geometry*, void*, const void*, double, int, int, void*);
template int fwd_lambda<double>(const gr_geometry*, void*, const void*, const void*, float, float, int,
                            int, void*);
template int bwd_tv_primal<double>(const gr_geometry*, void*, void*, const void*, const void*, float,
                               float, float, int, int, void*);
template int fwd_wsq<double>(const gr_geometry*, void*, const void*, const void*, double*, const int*,
                         int, int, void*);
template int bwd_cg<double>(const gr_geometry*, void*, const void*, void*, const void*, const double*,
                        double*, const int*, int, int, void*);
template int bwd_sum<double>(const gr_geometry*, void*, const void*, double*, int, int, void*);
template int fwd_angle_axpy<double>(const gr_geometry*, void*, const void*, const void*, const void*,
                                double, int, int, void*);
template int bwd_tv_adjoint<double>(const gr_geometry*, void*, const void*, const void*, double, float,
                                float, int, int, void*);
}  // namespace gr
