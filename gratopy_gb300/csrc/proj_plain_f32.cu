// Plain forward/backprojection launches, float instantiation.
#define GR_DEFINE_PLAIN
#include "proj_impl.cuh"

namespace gr {
template int fwd_plain<float>(const gr_geometry*, void*, const void*, int, int, int, void*);
template int bwd_plain<float>(const gr_geometry*, void*, const void*, int, int, int, void*);
}  // namespace gr
