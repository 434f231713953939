// Batched reconstruction: many float32 2-D problems (Radon or fan beam, any
// size, Landweber / CG / TV) advance one iteration per sequence of
// persistent launches.  Each launch strides over a flat work list of
// (problem, tile) pairs, so one launch covers every problem in the batch and
// the GPU stays full even when single problems are far too small to fill it.
// The per-problem solver step is selected at run time by the epilogue.
#include "proj_launch.cuh"

using namespace gr;

namespace {

constexpr int kSinoChunk = 256;

struct BatchFwdEpi {
  static constexpr bool kReduce = true;
  const gr_batch_problem* P;
  int mode;
  __device__ __forceinline__ double operator()(int64_t, int64_t a, int64_t, int64_t i,
                                               float v) const {
    if (mode == GR_BATCH_NORMEST) {
      P->s1[i] = v;
      return 0.0;
    }
    switch (P->solver) {
      case GR_SOLVER_LANDWEBER:
        P->s1[i] = v - P->f[i];
        return 0.0;
      case GR_SOLVER_CG: {
        P->s1[i] = v;
        const float wv = v * P->w[a];
        return (double)wv * (double)v;
      }
      default:
        P->s1[i] = (P->s1[i] + P->a1 * (v - P->f[i])) * P->a2;
        return 0.0;
    }
  }
};

struct BatchBwdEpi {
  static constexpr bool kReduce = true;
  const gr_batch_problem* P;
  int mode;
  __device__ __forceinline__ double operator()(int64_t x, int64_t y, int64_t, int64_t i,
                                               float v) const {
    if (mode == GR_BATCH_NORMEST) {
      P->img[i] = v;
      return (double)v;
    }
    if (mode == GR_BATCH_CG_INIT) {
      P->i1[i] = v;
      P->i2[i] = v;
      return (double)v * (double)v;
    }
    switch (P->solver) {
      case GR_SOLVER_LANDWEBER:
        P->img[i] += P->a0 * v;
        return 0.0;
      case GR_SOLVER_CG: {
        P->i2[i] = v;
        const float alpha = (float)P->sc[GR_SC_ALPHA];
        P->img[i] += alpha * P->i1[i];
        return (double)v * (double)v;
      }
      default: {
        // total_variation.cl:108-148 + extragradient (2-D: no z term)
        const int64_t Nx = P->Nx, Ny = P->Ny;
        const float* vp = P->v4 + 4 * i;
        float v0 = vp[0], v1 = vp[1];
        if (x == Nx - 1) v0 = 0.0f;
        if (x > 0) v0 -= vp[-4 + 0];
        if (y == Ny - 1) v1 = 0.0f;
        if (y > 0) v1 -= vp[-4 * Nx + 1];
        const float uo = P->img[i];
        const float un = fmaxf(0.0f, uo + P->a3 * (v0 + v1 + 0.0f - P->a4 * v));
        P->img[i] = un;
        P->i1[i] = 2.0f * un - uo;
        return 0.0;
      }
    }
  }
};

__device__ __forceinline__ Dims dims2(const gr_batch_problem& P) {
  Dims d;
  d.Nx = P.Nx;
  d.Ny = P.Ny;
  d.Nz = 1;
  d.Ns = P.Ns;
  d.Na = P.Na;
  return d;
}

__device__ __forceinline__ FanGeo<float> fan_of(const gr_batch_problem& P) {
  FanGeo<float> g;
  g.R = P.geo[0];
  g.RE = P.geo[1];
  g.delta_xi = P.geo[2];
  g.midx = P.geo[3];
  g.midy = P.geo[4];
  g.mid_det = P.geo[5];
  g.delta_x = P.geo[6];
  return g;
}

template <int SPLIT>
__device__ __forceinline__ double fwd_item(const gr_batch_problem& P, int tile, int mode) {
  const uint3 bid = make_uint3(tile % P.fwd_tiles_x, tile / P.fwd_tiles_x, 0);
  const float* in = (mode == GR_BATCH_NORMEST || P.solver == GR_SOLVER_LANDWEBER) ? P.img : P.i1;
  const BatchFwdEpi e{&P, mode};
  if (P.kind == GR_RADON) {
    RadonGeo<float> g;
    g.delta_x = P.geo[0];
    g.delta_xi = P.geo[1];
    return fast::radon_fwd_fast_tile<ORDER_F, ORDER_F, 1, SPLIT, BatchFwdEpi>(in, P.ofs, g,
                                                                             dims2(P), e, bid);
  }
  return fast::fan_fwd_fast_tile<ORDER_F, ORDER_F, 1, SPLIT, BatchFwdEpi>(in, P.ofs, P.sdpd,
                                                                         fan_of(P), dims2(P), e,
                                                                         bid);
}

__global__ void __launch_bounds__(kFwdBlock)
batch_forward_kernel(const gr_batch_problem* __restrict__ probs, const int2* __restrict__ items,
                     int n, int mode) {
  __shared__ double red[32];
  for (int it = blockIdx.x; it < n; it += gridDim.x) {
    const int2 item = items[it];
    const gr_batch_problem& P = probs[item.x];
    double part;
    switch (P.fwd_split) {
      case 1: part = fwd_item<1>(P, item.y, mode); break;
      case 2: part = fwd_item<2>(P, item.y, mode); break;
      case 4: part = fwd_item<4>(P, item.y, mode); break;
      default: part = fwd_item<8>(P, item.y, mode); break;
    }
    const double t = block_sum(part, red);
    if (threadIdx.x == 0) P.fwd_part[item.y] = t;
  }
}

// Forward over orbits (problems of kind KIND with orbit bit 1; items of
// other problems are skipped): a tile covers a pair of base angles, the orbit
// members gathered from the image, with the lanes per group of the per-call
// orbit forwards (4 x fwd_split parallel beam, 2 x fan beam).  One kernel
// per kind keeps each at its own register count.
template <int KIND, int SPLIT>
__device__ __forceinline__ double fwd_orbit_item(const gr_batch_problem& P, int tile, int mode) {
  const uint3 bid = make_uint3(tile % P.fwd_tiles_x, tile / P.fwd_tiles_x, 0);
  const float* in = (mode == GR_BATCH_NORMEST || P.solver == GR_SOLVER_LANDWEBER) ? P.img : P.i1;
  const BatchFwdEpi e{&P, mode};
  const fast::QuarterMaps qm = launch::quarter_maps_of(P.sym_map);
  if constexpr (KIND == GR_RADON) {
    RadonGeo<float> g;
    g.delta_x = P.geo[0];
    g.delta_xi = P.geo[1];
    return fast::radon_fwd_quarter_tile<ORDER_F, ORDER_F, 4 * SPLIT, false, 1, BatchFwdEpi>(
        in, nullptr, P.ofs, g, dims2(P), qm, e, bid, 0);
  } else {
    return fast::fan_fwd_quarter_tile<ORDER_F, ORDER_F, 2 * SPLIT, false, false, BatchFwdEpi>(
        in, nullptr, P.ofs, P.sdpd, fan_of(P), dims2(P), qm, e, bid, 0);
  }
}

template <int KIND>
__global__ void __launch_bounds__(kFwdBlock)
batch_forward_orbit_kernel(const gr_batch_problem* __restrict__ probs,
                           const int2* __restrict__ items, int n, int mode) {
  __shared__ double red[32];
  for (int it = blockIdx.x; it < n; it += gridDim.x) {
    const int2 item = items[it];
    const gr_batch_problem& P = probs[item.x];
    if (P.kind != KIND || !(P.orbit & 1)) continue;  // uniform per block
    double part;
    switch (P.fwd_split) {
      case 1: part = fwd_orbit_item<KIND, 1>(P, item.y, mode); break;
      case 2: part = fwd_orbit_item<KIND, 2>(P, item.y, mode); break;
      case 4: part = fwd_orbit_item<KIND, 4>(P, item.y, mode); break;
      default: part = fwd_orbit_item<KIND, 8>(P, item.y, mode); break;
    }
    const double t = block_sum(part, red);
    if (threadIdx.x == 0) P.fwd_part[item.y] = t;
  }
}

constexpr int kBatchPY = 2;  // pixels per thread of the batched backprojection

__global__ void __launch_bounds__(kBwdTileFast * kBwdTileSlow / kBatchPY)
batch_backward_kernel(const gr_batch_problem* __restrict__ probs, const int2* __restrict__ items,
                      int n, int mode) {
  __shared__ double red[32];
  for (int it = blockIdx.x; it < n; it += gridDim.x) {
    const int2 item = items[it];
    const gr_batch_problem& P = probs[item.x];
    const uint3 bid = make_uint3(item.y % P.bwd_tiles_x, item.y / P.bwd_tiles_x, 0);
    const float* in;
    if (mode == GR_BATCH_NORMEST) in = P.s1;
    else if (mode == GR_BATCH_CG_INIT) in = P.s2;
    else in = P.solver == GR_SOLVER_CG ? P.s2 : P.s1;
    const BatchBwdEpi e{&P, mode};
    double part;
    if (P.kind == GR_RADON)
      part = fast::radon_bwd_fast_tile<ORDER_F, ORDER_F, 1, 1, kBatchPY, BatchBwdEpi>(
          in, P.ofs, dims2(P), e, bid);
    else
      part = fast::fan_bwd_fast_tile<ORDER_F, ORDER_F, 1, 1, kBatchPY, BatchBwdEpi>(
          in, P.ofs, P.sdpd, fan_of(P), dims2(P), e, bid);
    const double t = block_sum(part, red);
    if (threadIdx.x + blockDim.x * threadIdx.y == 0) P.bwd_part[item.y] = t;
  }
}

// Backprojection over pixel orbits (problems of kind KIND with orbit bit 2;
// items of other problems are skipped): a tile is 32 quadrant pixels, each
// thread row one of 8 angle groups, as the per-call orbit backprojections
// without scratch.
constexpr int kBatchOrbitG = 8;

template <int KIND>
__global__ void __launch_bounds__(kBwdTileFast * kBwdTileSlow)
batch_backward_orbit_kernel(const gr_batch_problem* __restrict__ probs,
                            const int2* __restrict__ items, int n, int mode) {
  __shared__ double red[32];
  for (int it = blockIdx.x; it < n; it += gridDim.x) {
    const int2 item = items[it];
    const gr_batch_problem& P = probs[item.x];
    if (P.kind != KIND || !(P.orbit & 2)) continue;  // uniform per block
    const uint3 bid = make_uint3(item.y % P.obwd_tiles_x, item.y / P.obwd_tiles_x, 0);
    const float* in;
    if (mode == GR_BATCH_NORMEST) in = P.s1;
    else if (mode == GR_BATCH_CG_INIT) in = P.s2;
    else in = P.solver == GR_SOLVER_CG ? P.s2 : P.s1;
    const BatchBwdEpi e{&P, mode};
    const fast::QuarterMaps qm = launch::quarter_maps_of(P.sym_map);
    double part;
    if constexpr (KIND == GR_RADON)
      part = fast::radon_bwd_orbit_tile<ORDER_F, ORDER_F, kBatchOrbitG, false, BatchBwdEpi>(
          nullptr, in, P.ofs, dims2(P), qm, e, bid, 0);
    else
      part = fast::fan_bwd_orbit_tile<ORDER_F, ORDER_F, kBatchOrbitG, BatchBwdEpi>(
          in, P.ofs, P.sdpd, fan_of(P), dims2(P), qm, e, bid, 0);
    const double t = block_sum(part, red);
    if (threadIdx.x + blockDim.x * threadIdx.y == 0) P.bwd_part[item.y] = t;
  }
}

// One thread per pixel of a 32 x 8 backprojection tile.
__global__ void __launch_bounds__(kBwdTileFast * kBwdTileSlow)
batch_image_kernel(const gr_batch_problem* __restrict__ probs, const int2* __restrict__ items,
                   int n, int mode) {
  for (int it = blockIdx.x; it < n; it += gridDim.x) {
    const int2 item = items[it];
    const gr_batch_problem& P = probs[item.x];
    const int64_t x = (int64_t)(item.y % P.bwd_tiles_x) * kBwdTileFast + threadIdx.x;
    const int64_t y = (int64_t)(item.y / P.bwd_tiles_x) * kBwdTileSlow + threadIdx.y;
    if (x >= P.Nx || y >= P.Ny) continue;
    const int64_t i = x + P.Nx * y;
    if (mode == GR_BATCH_NORMEST) {
      P.img[i] /= (float)P.sc[GR_SC_SUM];
    } else if (P.solver == GR_SOLVER_CG) {
      P.i1[i] = (float)P.sc[GR_SC_BETA] * P.i1[i] + P.i2[i];
    } else if (P.solver == GR_SOLVER_TV) {
      // total_variation.cl:54-93 + :150-167 (2-D: no z term)
      const float c = -P.i1[i];
      const float g0 = x < P.Nx - 1 ? c + P.i1[i + 1] : 0.0f;
      const float g1 = y < P.Ny - 1 ? c + P.i1[i + P.Nx] : 0.0f;
      float* vp = P.v4 + 4 * i;
      float v0 = vp[0] + P.a0 * g0, v1 = vp[1] + P.a0 * g1, v2 = vp[2] + P.a0 * 0.0f;
      const float nrm = hypotf(hypotf(v0, v1), v2);
      if (nrm > 1.0f) {
        v0 /= nrm;
        v1 /= nrm;
        v2 /= nrm;
      }
      vp[0] = v0;
      vp[1] = v1;
      vp[2] = v2;
    }
  }
}

__global__ void __launch_bounds__(kSinoChunk)
batch_sino_kernel(const gr_batch_problem* __restrict__ probs, const int2* __restrict__ items,
                  int n, int mode) {
  for (int it = blockIdx.x; it < n; it += gridDim.x) {
    const int2 item = items[it];
    const gr_batch_problem& P = probs[item.x];
    const int64_t i = (int64_t)item.y * kSinoChunk + threadIdx.x;
    if (i >= (int64_t)P.Ns * P.Na) continue;
    if (mode == GR_BATCH_MAIN && P.solver == GR_SOLVER_CG) {
      const float na = -(float)P.sc[GR_SC_ALPHA];
      P.s2[i] = P.s2[i] + na * P.s1[i];
    }
  }
}

__device__ double sum_parts(const double* __restrict__ p, int64_t n, double* red) {
  double acc = 0.0;
  for (int64_t k = threadIdx.x; k < n; k += blockDim.x) acc += p[k];
  return block_sum(acc, red);
}

__global__ void __launch_bounds__(1024)
batch_scalar_kernel(const gr_batch_problem* __restrict__ probs, const int* __restrict__ ids,
                    int mode, int phase) {
  __shared__ double red[32];
  const gr_batch_problem& P = probs[ids[blockIdx.x]];
  const int64_t n_fwd = (int64_t)P.fwd_tiles_x * P.fwd_tiles_y;
  const int64_t n_bwd = (P.orbit & 2) ? (int64_t)P.obwd_tiles_x * P.obwd_tiles_y
                                      : (int64_t)P.bwd_tiles_x * P.bwd_tiles_y;
  double* sc = P.sc;
  if (phase == 0) {
    if (mode != GR_BATCH_MAIN || P.solver != GR_SOLVER_CG) return;
    const double qwq = sum_parts(P.fwd_part, n_fwd, red);
    if (threadIdx.x == 0) sc[GR_SC_ALPHA] = (double)(float)(P.cg_c * (sc[GR_SC_SOLD] / qwq));
    return;
  }
  const double s = sum_parts(P.bwd_part, n_bwd, red);
  if (threadIdx.x != 0) return;
  if (mode == GR_BATCH_NORMEST) {
    sc[GR_SC_SUM] = s;
  } else if (mode == GR_BATCH_CG_INIT) {
    sc[GR_SC_SOLD] = s;
    sc[GR_SC_BETA] = 0.0;
  } else if (P.solver == GR_SOLVER_CG) {
    sc[GR_SC_BETA] = (double)(float)(s / sc[GR_SC_SOLD]);
    sc[GR_SC_SOLD] = s;
  }
}

// grid <= 0: one wave of resident blocks (SMs x blocks per SM at the
// kernel's occupancy), so the blocks stride over the work list in lockstep.
int resident_grid(void (*k)(const gr_batch_problem*, const int2*, int, int), dim3 block) {
  int dev = 0, sms = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0)
    sms = 152;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, (int)(block.x * block.y * block.z),
                                                    0) != cudaSuccess || per_sm <= 0)
    per_sm = 4;
  return sms * per_sm;
}

int launch_items(void (*k)(const gr_batch_problem*, const int2*, int, int), dim3 block,
                 const gr_batch_problem* probs, const int* items, int n, int mode, int grid,
                 void* stream) {
  if (n < 0) return GR_ERR_ARG;
  if (n == 0) return GR_OK;
  if (probs == nullptr || items == nullptr) return GR_ERR_ARG;
  if (grid <= 0) grid = resident_grid(k, block);
  const int g = grid < n ? grid : n;
  k<<<g, block, 0, as_stream(stream)>>>(probs, reinterpret_cast<const int2*>(items), n, mode);
  return check_launch();
}

}  // namespace

extern "C" {

size_t gr_batch_problem_size(void) { return sizeof(gr_batch_problem); }

int gr_batch_forward(const gr_batch_problem* probs, const int* items, int n, int mode, int grid,
                     void* stream) {
  return launch_items(batch_forward_kernel, dim3(kFwdBlock), probs, items, n, mode, grid, stream);
}

int gr_batch_backward(const gr_batch_problem* probs, const int* items, int n, int mode, int grid,
                      void* stream) {
  return launch_items(batch_backward_kernel, dim3(kBwdTileFast, kBwdTileSlow / kBatchPY), probs,
                      items, n, mode, grid, stream);
}

int gr_batch_forward_orbit(const gr_batch_problem* probs, const int* items, int n, int mode,
                           int kind, int grid, void* stream) {
  if (kind != GR_RADON && kind != GR_FANBEAM) return GR_ERR_ARG;
  return launch_items(kind == GR_RADON ? batch_forward_orbit_kernel<GR_RADON>
                                       : batch_forward_orbit_kernel<GR_FANBEAM>,
                      dim3(kFwdBlock), probs, items, n, mode, grid, stream);
}

int gr_batch_backward_orbit(const gr_batch_problem* probs, const int* items, int n, int mode,
                            int kind, int grid, void* stream) {
  if (kind != GR_RADON && kind != GR_FANBEAM) return GR_ERR_ARG;
  return launch_items(kind == GR_RADON ? batch_backward_orbit_kernel<GR_RADON>
                                       : batch_backward_orbit_kernel<GR_FANBEAM>,
                      dim3(kBwdTileFast, kBwdTileSlow), probs, items, n, mode, grid, stream);
}

int gr_batch_image_step(const gr_batch_problem* probs, const int* items, int n, int mode,
                        int grid, void* stream) {
  return launch_items(batch_image_kernel, dim3(kBwdTileFast, kBwdTileSlow), probs, items, n, mode,
                      grid, stream);
}

int gr_batch_sino_step(const gr_batch_problem* probs, const int* items, int n, int mode, int grid,
                       void* stream) {
  return launch_items(batch_sino_kernel, dim3(kSinoChunk), probs, items, n, mode, grid, stream);
}

int gr_batch_scalars(const gr_batch_problem* probs, const int* prob_ids, int n, int mode,
                     int phase, void* stream) {
  if (n < 0) return GR_ERR_ARG;
  if (n == 0) return GR_OK;
  if (probs == nullptr || prob_ids == nullptr) return GR_ERR_ARG;
  batch_scalar_kernel<<<n, 1024, 0, as_stream(stream)>>>(probs, prob_ids, mode, phase);
  return check_launch();
}

}  // extern "C"
