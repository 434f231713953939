// Internal helpers shared by the translation units behind the C ABI.
#pragma once

#include <type_traits>

#include "../../include/gratopy_gb300.h"
#include "gr_common.cuh"

namespace gr {

void set_cuda_error(cudaError_t e);

inline int check_launch() {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_cuda_error(e);
    return GR_ERR_CUDA;
  }
  return GR_OK;
}

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Launch with programmatic stream serialization: the kernel may start
// launching once every block of the kernel before it has called
// pdl_trigger (or exited), and waits in pdl_wait until that kernel has
// completed and its writes are visible.  The kernel calls pdl_wait before
// any access to global memory.  Errors are left for check_launch.
template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t st,
                       Args&&... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = 0;
  cfg.stream = st;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  (void)cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

template <int V>
using IC = std::integral_constant<int, V>;

// Calls f(IC<so>{}, IC<io>{}) for the runtime order pair.
template <class F>
inline int dispatch_orders(int so, int io, F&& f) {
  if (so == ORDER_F && io == ORDER_F) return f(IC<ORDER_F>{}, IC<ORDER_F>{});
  if (so == ORDER_F && io == ORDER_C) return f(IC<ORDER_F>{}, IC<ORDER_C>{});
  if (so == ORDER_C && io == ORDER_F) return f(IC<ORDER_C>{}, IC<ORDER_F>{});
  if (so == ORDER_C && io == ORDER_C) return f(IC<ORDER_C>{}, IC<ORDER_C>{});
  return GR_ERR_ARG;
}

inline bool valid_order(int o) { return o == ORDER_F || o == ORDER_C; }
inline bool valid_dtype(int t) { return t == GR_F32 || t == GR_F64; }

}  // namespace gr
