// Projections with fused solver epilogues, float instantiation.
#define GR_DEFINE_FUSED
#include "proj_impl.cuh"

namespace gr {
template int fwd_residual<float>(const gr_geometry*, void*, const void*, const void*, int, int, void*);
template int bwd_axpy<float>(const gr_geometry*, void*, const void*, double, int, int, void*);
template int fwd_lambda<float>(const gr_geometry*, void*, const void*, const void*, float, float, int,
                            int, void*);
template int bwd_tv_primal<float>(const gr_geometry*, void*, void*, const void*, const void*, float,
                               float, float, int, int, void*);
template int fwd_wsq<float>(const gr_geometry*, void*, const void*, const void*, double*, const int*,
                         int, int, void*);
template int bwd_cg<float>(const gr_geometry*, void*, const void*, void*, const void*, const double*,
                        double*, const int*, int, int, void*);
template int bwd_sum<float>(const gr_geometry*, void*, const void*, double*, int, int, void*);
template int fwd_angle_axpy<float>(const gr_geometry*, void*, const void*, const void*, const void*,
                                double, int, int, void*);
template int bwd_tv_adjoint<float>(const gr_geometry*, void*, const void*, const void*, double, float,
                                float, int, int, void*);
}  // namespace gr
