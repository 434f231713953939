// Plain forward/backprojection launches, double instantiation.
#define GR_DEFINE_PLAIN
#include "proj_impl.cuh"

namespace gr {
template int fwd_plain<double>(const gr_geometry*, void*, const void*, int, int, int, void*);
template int bwd_plain<double>(const gr_geometry*, void*, const void*, int, int, int, void*);
}  // namespace gr
