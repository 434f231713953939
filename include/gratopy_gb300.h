/*
 * gratopy_gb300 -- C ABI of the GB300 (sm_103a) projection and
 * reconstruction kernels.
 *
 * Conventions
 *  - Every pointer argument named like an array (sino, img, ofs, ...) is a
 *    DEVICE pointer owned by the caller; scalars and `const double* geo`
 *    are host values.  Nothing here allocates or frees memory.
 *  - `stream` is a cudaStream_t passed as void*; every call is
 *    asynchronous on it and returns 0 (GR_OK) or an error code; nothing
 *    throws across the ABI.  gr_error_string() names a code.
 *  - dtype: GR_F32 or GR_F64.  order: GR_ORDER_F (x / detector fastest) or
 *    GR_ORDER_C (z fastest), as in gratopy's pos_img_f / pos_img_c
 *    (gratopy radon.cl:28-31).  Images are (Nx, Ny, Nz), sinograms
 *    (Ns, Na, Nz); Nz = 1 for 2-D data.
 *  - Per-angle table `ofs`: 8 reals per angle, angle-major (gratopy's
 *    ofs_dict arrays in Fortran order); `sdpd`: Ns reals (fan beam only).
 *    gratopy builds them in radon_struct (gratopy.py:380-578) and
 *    fanbeam_struct (gratopy.py:706-1003).
 */
#ifndef GRATOPY_GB300_H
#define GRATOPY_GB300_H

#include <stddef.h>

#if defined(__GNUC__)
#define GR_API __attribute__((visibility("default")))
#else
#define GR_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

enum { GR_F32 = 0, GR_F64 = 1 };
enum { GR_ORDER_F = 0, GR_ORDER_C = 1 };
enum { GR_RADON = 0, GR_FANBEAM = 1 };

enum {
  GR_OK = 0,
  GR_ERR_ARG = 1,      /* null pointer, bad dtype/order/kind */
  GR_ERR_SHAPE = 2,    /* sizes inconsistent with the geometry */
  GR_ERR_CUDA = 3,     /* a CUDA launch or runtime call failed */
  GR_ERR_TOO_BIG = 4   /* size beyond a documented limit */
};

/* Geometry of one projection problem.  geo[] holds gratopy's
 * Geometryinformation vector in float64:
 *   Radon (6):  [delta_x, delta_s, Nx, Ny, Ns, Na]           (gratopy.py:556-560)
 *   Fan  (11):  [R, RE, ds/dx, x_mid, y_mid, s_mid, Nx, Ny, Ns, Na, delta_x]
 *                                                          (gratopy.py:970-986) */
typedef struct gr_geometry {
  int kind;          /* GR_RADON | GR_FANBEAM */
  int dtype;         /* GR_F32 | GR_F64: precision of ofs/sdpd and of the data */
  int Nx, Ny, Ns, Na;
  const void* ofs;   /* device: 8*Na reals */
  const void* sdpd;  /* device: Ns reals (fan) or NULL (Radon) */
  double geo[11];
  /* Launch shape (0 = automatic): lanes per detector bin in the forward
   * projection and angle groups per pixel in the backprojection; each must
   * be 1, 2, 4 or 8.  Chosen by the autotuner.  The quarter-turn forward
   * (sym = 4) runs twice fwd_split lanes per group of bins. */
  int fwd_split, bwd_split;
  /* Quarter-turn symmetry (no counterpart in the reference): 4 when the
   * angles a + m*Na/4 see the (square, centred) pixel grid as angle a sees it
   * after m quarter turns, else 0.  sym_map[m-1] = (axx, axy, ayx, ayy, cx,
   * cy): pixel (x, y) of angle a is pixel (cx + axx x + axy y, cy + ayx x +
   * ayy y) of angle a + m*Na/4.  The float32 fan-beam forward projection of
   * single slices then shares each pixel's interpolation weights across the
   * four angles.  2 for a parallel-beam geometry with Na angles equispaced
   * over [0, pi) (Na even), a centred square image and a centred detector:
   * sym_map[0..2] are then the lookups S^-1, -I, -S^-1 (S the quarter turn
   * with which angle k + Na/2 sees the grid as angle k does) that give the
   * outputs (s, k + Na/2), (Ns-1-s, k), (Ns-1-s, k + Na/2) from the weights
   * of angle k; the float32 projections of single slices then run over these
   * orbits when `work` holds their copies, and so does the forward projection
   * of stacks from 32 * 2^20 pixel-angles per slice, slice by slice.  Set by
   * the Python layer after checking the geometry. */
  int sym;
  int sym_map[3][6];
  /* Mirror symmetry of a quarter-turn symmetric fan-beam geometry (sym = 4;
   * no counterpart in the reference): nonzero when angle (mirror_pair - b)
   * mod Na sees pixel mirror_map(P) as angle b sees P, with the detector
   * reversed (bin s <-> Ns - 1 - s), for every angle b.  mirror_map is a
   * reflection through the image centre in the sym_map format.  The float32
   * forward projection that reads the orbit copy then walks only the bins
   * s < ceil(Ns/2) and fills their mirrored bins from the same weights.
   * Ignored unless sym = 4.  Set by the Python layer after checking the
   * geometry; 0 in a zeroed descriptor. */
  int mirror;
  int mirror_pair;
  int mirror_map[6];
  /* Device scratch (no counterpart in the reference) that a call may use
   * while it runs, stream-ordered, 16-byte aligned: the quarter-turn orbit
   * kernels keep interleaved copies of their input there (the forward: the
   * four orbit pixels of every pixel; the backprojection: the four sinogram
   * rows of every angle orbit).  gr_work_bytes gives the size for a number
   * of slices; a stack is copied in chunks of as many slices as the scratch
   * holds.  NULL or smaller than one slice's copy: the kernels read their
   * input directly.  Calls that may run at the same time must not share
   * it. */
  void* work;
  size_t work_bytes;
} gr_geometry;

GR_API const char* gr_error_string(int code);
/* Scratch bytes the projections of g on Nz slices can use (gr_geometry.work;
 * at most 8 slices' copies); 0 when they use none. */
GR_API size_t gr_work_bytes(const gr_geometry* g, int Nz);
/* Which projections of g on Nz slices run over orbits (no counterpart in the
 * reference): bit 1 the forward, bit 2 the backprojection; 0 for none or an
 * invalid geometry.  Stacks' orbit forward needs g's scratch (gr_work_bytes). */
GR_API int gr_orbit_kinds(const gr_geometry* g, int Nz);
/* sizeof(gr_geometry), for bindings that mirror the struct. */
GR_API size_t gr_geometry_size(void);
/* Last CUDA error seen by this library on the calling thread (cudaError_t). */
GR_API int gr_last_cuda_error(void);
GR_API int gr_version(void);
/* Hex SHA-256 of the sources this library was compiled from (csrc/*.cu,
 * csrc/*.cuh, this header and the build recipe), so a binding can refuse a
 * library left over from other sources. */
GR_API const char* gr_source_hash(void);

/* ---- The four projection kernels, argument order as gratopy's kernels ----
 * radon.cl:66-161    radon_{T}_{so}{io}(sino, img, ofs, Geometryinformation) */
GR_API int gr_radon_fwd(void* sino, const void* img, const void* ofs, const double* geo,
                 int dtype, int Ns, int Na, int Nz, int sino_order, int img_order,
                 void* stream);
/* radon.cl:183-241   radon_ad_{T}_{io}{so}(img, sino, ofs, Geometryinformation) */
GR_API int gr_radon_bwd(void* img, const void* sino, const void* ofs, const double* geo,
                 int dtype, int Nx, int Ny, int Nz, int img_order, int sino_order,
                 void* stream);
/* fanbeam.cl:72-256  fanbeam_{T}_{so}{io}(sino, img, ofs, sdpd, Geometryinformation) */
GR_API int gr_fan_fwd(void* sino, const void* img, const void* ofs, const void* sdpd,
               const double* geo, int dtype, int Ns, int Na, int Nz, int sino_order,
               int img_order, void* stream);
/* fanbeam.cl:290-391 fanbeam_ad_{T}_{io}{so}(img, sino, ofs, sdpd, Geometryinformation) */
GR_API int gr_fan_bwd(void* img, const void* sino, const void* ofs, const void* sdpd,
               const double* geo, int dtype, int Nx, int Ny, int Nz, int img_order,
               int sino_order, void* stream);

/* ---- Geometry-generic projections (dispatch on g->kind) ----
 * gratopy.py:1655-1685 (ProjectionSettings.forwardprojection/backprojection) */
GR_API int gr_forward(const gr_geometry* g, void* sino, const void* img, int Nz, int sino_order,
               int img_order, void* stream);
GR_API int gr_backward(const gr_geometry* g, void* img, const void* sino, int Nz, int img_order,
                int sino_order, void* stream);

/* ---- Projections with a fused solver epilogue (image and sinogram share
 * one order) ----
 * Landweber (gratopy.py:2432-2444): r = A u - f  and  u += a * A^T r */
GR_API int gr_forward_residual(const gr_geometry* g, void* r, const void* u, const void* f, int Nz,
                        int order, void* stream);
GR_API int gr_backward_axpy(const gr_geometry* g, void* u, const void* r, double a, int Nz, int order,
                     void* stream);
/* TV data dual step (total_variation.cl:95-106 on A u):
 * lambda = (lambda + sigma (A u - f)) * mu2 */
GR_API int gr_forward_lambda(const gr_geometry* g, void* lambda, const void* u, const void* f,
                      float sigma, float mu2, int Nz, int order, void* stream);
/* TV primal step (total_variation.cl:108-148 + gratopy.py:2708-2717 on A^T lambda):
 * u_new = max(0, u + tau (div v - norming A^T lambda)); ubar = 2 u_new - u; u = u_new */
GR_API int gr_backward_tv_primal(const gr_geometry* g, void* u, void* ubar, const void* v,
                          const void* lambda, float tau, float norming, float z_distance,
                          int Nz, int order, void* stream);
/* CG (gratopy.py:2521-2542): q = A p with block partials of <W q, q>;
 * snew = A^T d, x += alpha p with block partials of <snew, snew>.
 * `skip` (device int, may be NULL) makes the launch a no-op when nonzero. */
GR_API int gr_forward_wsq(const gr_geometry* g, void* q, const void* p, const void* w,
                   double* partials, const int* skip, int Nz, int order, void* stream);
GR_API int gr_backward_cg(const gr_geometry* g, void* snew, const void* d, void* x, const void* p,
                   const double* alpha, double* partials, const int* skip, int Nz, int order,
                   void* stream);
/* No counterpart in the reference: gr_forward_wsq without caller scratch, for
 * callers that cannot allocate device memory where they run this step (code
 * inside a CUDA graph capture, hosts whose device memory is budgeted by
 * another allocator, loops that cannot take cudaMalloc's implicit sync).
 * Writes q = A p and *out = <W q, q> (device double).  The block partials
 * live in a static device array of this library: at most 65536 of them
 * (gr_forward_partials(g, Nz) <= 65536, else GR_ERR_TOO_BIG); 512 KiB is
 * held on every GPU that loads the library until exit.  The first call on
 * each device looks that array's address up (cudaGetSymbolAddress), so make
 * it before any stream capture; the address is kept for the life of the
 * process, so after a cudaDeviceReset of a device this entry point must not
 * be called on that device again.  All calls share the array: calls that
 * overlap on the GPU (several streams, several host threads) race, so the
 * caller serialises them, for example on one stream.  Invalid sizes return
 * GR_ERR_SHAPE before the partial count is checked. */
GR_API int gr_forward_wsq_noalloc(const gr_geometry* g, void* q, const void* p, const void* w,
                                  double* out, int Nz, int order, void* stream);
/* Transposes for differentiation (no counterpart in the reference, which
 * has no gradients): out = base + c * w[a] * (A u), base may be NULL.  With
 * c = (ds/dx)/dx and w the angle weights this is the plain transpose of
 * gratopy's backprojection; the plain transpose of the forward projection is
 * gr_backward with the per-angle weights of ofs replaced by dx/(ds/dx). */
GR_API int gr_forward_angle_axpy(const gr_geometry* g, void* out, const void* base, const void* u,
                                 const void* w, double c, int Nz, int order, void* stream);
/* Adjoint of one TV primal-dual iteration (reverse mode through
 * total_variation.cl:54-167): out = c1 * (A^T lambda) - sigma * div(gw) on
 * the image, with A^T from an adjoint geometry as above. */
GR_API int gr_backward_tv_adjoint(const gr_geometry* g, void* out, const void* lambda,
                                  const void* gw, double c1, float sigma, float z_distance, int Nz,
                                  int order, void* stream);
/* Elementwise parts of the TV adjoint (csrc/tv_adjoint.cu):
 * gz = [u_next > 0] (gu + 2 gubar), gu_prev = gz - gubar */
GR_API int gr_tv_adjoint_primal(void* gz, void* gu_prev, const void* gu, const void* gubar,
                                const void* u_next, int dtype, size_t n, void* stream);
/* gw = J_P(w)^T (gv - tau grad gz), w = v + sigma grad ubar (4 reals/pixel) */
GR_API int gr_tv_adjoint_dual(void* gw, const void* gv, const void* gz, const void* v,
                              const void* ubar, float sigma, float tau, float z_distance, int dtype,
                              int Nx, int Ny, int Nz, int order, void* stream);
/* gl_prev = mu2 gl1, gf -= mu2 sigma_l gl1 (sinogram-sized) */
GR_API int gr_tv_adjoint_lambda(void* gl_prev, void* gf, const void* gl1, float mu2, float sigma_l,
                                int dtype, size_t n, void* stream);
/* normest (gratopy.py:2366-2376): img = A^T sino with block partials of sum(img). */
GR_API int gr_backward_sum(const gr_geometry* g, void* img, const void* sino, double* partials,
                    int Nz, int order, void* stream);
/* Number of block partials the reducing launches above write. */
GR_API size_t gr_forward_partials(const gr_geometry* g, int Nz);
GR_API size_t gr_backward_partials(const gr_geometry* g, int Nz, int order);

/* ---- Elementwise and reduction kernels ---- */
/* utilities.cl:38-67 multiply/divide: out = sino * w[a]  (or / w[a]) */
GR_API int gr_weight_sinogram(void* out, const void* sino, const void* w, int dtype, int Ns, int Na,
                       int Nz, int order, int divide, void* stream);
/* utilities.cl:69-73 equ_mul_add: rhs += a x */
GR_API int gr_equ_mul_add(void* rhs, double a, const void* x, int dtype, size_t n, void* stream);
/* utilities.cl:75-80 mul_add_add: rhs = a x + y */
GR_API int gr_mul_add_add(void* rhs, double a, const void* x, const void* y, int dtype, size_t n,
                   void* stream);
/* Deterministic float64 dot product <a, b> (b may equal a), two stages:
 * gr_dot_partials writes gr_dot_partials_count() block partials, then
 * gr_sum_partials adds n partials in a fixed order into *out (device). */
GR_API size_t gr_dot_partials_count(void);
GR_API int gr_dot_partials(double* partials, const void* a, const void* b, int dtype, size_t n,
                    void* stream);
GR_API int gr_sum_partials(double* out, const double* partials, size_t n, void* stream);
/* Plain sum of n reals (normest's clarray.sum), same two-stage scheme. */
GR_API int gr_sum_values_partials(double* partials, const void* a, int dtype, size_t n, void* stream);

/* ---- TV dual step (total_variation.cl:54-93 + :150-167 fused):
 * v = P_{|.|<=1}(v + sigma grad(ubar)); v holds 4 reals per pixel. */
GR_API int gr_tv_dual(void* v, const void* ubar, float sigma, float z_distance, int dtype, int Nx,
               int Ny, int Nz, int order, void* stream);

/* ---- Sparse matrix of the forward projection (gratopy.py:2014-2155) ----
 * One launch over (pixel, angle): the single-line formula of radon.cl:263-341
 * / fanbeam.cl:422-568 for the two bins around the pixel's projection.
 * rows, cols, vals: 2*Nx*Ny*Na slots each (vals of g's dtype); slot 2*i+c,
 * i = a + Na*(x + Nx*y), holds (sinogram position, pixel position, value) in
 * `order`'s linear indexing; value 0 marks a slot without an entry. */
GR_API int gr_sparse_entries(const gr_geometry* g, int64_t* rows, int64_t* cols, void* vals,
                             int order, void* stream);

/* ---- Measurement (no counterpart in the reference) ----
 * L1 load-bandwidth probe: `blocks` blocks of 256 threads each stream `iters`
 * float4 loads from buf (n_vec float4, a power of two, small enough to stay
 * in L1); bytes moved = blocks * 256 * iters * 16.  out: blocks*256 floats,
 * written only in a case that cannot occur for a zero buffer. */
GR_API int gr_probe_l1_bandwidth(float* out, const void* buf, int n_vec, int iters, int blocks,
                                 void* stream);

/* ---- Ellipse phantoms on the device (gratopy phantom.py:159-177) ----
 * img: Nx x Ny x Nz in `order`; slice z is the sum of its K ellipses, given as
 * 7 doubles each (grey, a^2, b^2, xc, yc, cos theta, sin theta) at
 * ellipses[7*K*z ...], on the grid x = linspace(-1,1,Nx), y = -linspace(-1,1,Ny).
 * Rounded float64 arithmetic in numpy's order: equal to the host rasteriser. */
GR_API int gr_ellipses(void* img, const double* ellipses, int K, int Nx, int Ny, int Nz, int dtype,
                       int order, void* stream);

/* ---- Batched reconstruction (no counterpart in the reference) ----
 * Many float32 2-D problems of different sizes, geometries and solvers
 * advance together: each phase of an iteration is ONE persistent launch
 * whose blocks stride over a work list of (problem, tile) pairs covering
 * every problem.  Descriptors, work lists and buffers are device memory
 * owned by the caller; Fortran order throughout. */
enum { GR_SOLVER_LANDWEBER = 0, GR_SOLVER_CG = 1, GR_SOLVER_TV = 2 };
enum { GR_BATCH_NORMEST = 0, GR_BATCH_MAIN = 1, GR_BATCH_CG_INIT = 2 };
typedef struct gr_batch_problem {
  int kind, Nx, Ny, Ns, Na, solver;
  int fwd_split;               /* 1, 2, 4 or 8 lanes per group of detector bins */
  int fwd_tiles_x;             /* forward tiles per angle */
  int bwd_tiles_x, bwd_tiles_y;/* backprojection tiles (32 x 8 pixels) */
  const float* ofs;            /* 8*Na */
  const float* sdpd;           /* Ns (fan) */
  const float* w;              /* angle weights, Na */
  float geo[8];                /* Radon: dx, dxi (float); fan: R, RE, dxi, midx, midy, mid_det, dx */
  const float* f;              /* data sinogram */
  float* img;                  /* iterate: normest image / Landweber u / CG x / TV U */
  float* s1;                   /* normest sino / Landweber residual / CG q / TV lambda */
  float* s2;                   /* CG d */
  float* i1;                   /* CG p / TV ubar */
  float* i2;                   /* CG snew */
  float* v4;                   /* TV dual, 4 reals per pixel */
  double* sc;                  /* GR_SC_COUNT scalars */
  double* fwd_part;            /* fwd_tiles_x * Na partials */
  double* bwd_part;            /* bwd_tiles_x * bwd_tiles_y partials */
  float a0, a1, a2, a3, a4;    /* Landweber: a0 = -w;  TV: sigma, sigma_l, mu2, tau, norming */
  double cg_c;                 /* CG: dx^2/ds */
  /* Orbit tiles (no counterpart in the reference), as gr_orbit_kinds gives
   * them for the problem's gr_geometry: bit 1 the forward runs over the
   * orbits of sym_map (fwd_tiles_x bin tiles of 128-thread blocks per pair of
   * base angles, gathering the orbit members from the image); bit 2 the
   * backprojection does (gr_batch_backward_orbit over the quadrant's
   * obwd_tiles_x x obwd_tiles_y tiles of 32 x 1 pixels, 8 angle groups). */
  int orbit;
  int sym;                     /* 4: fan-beam quarter turns, 2: parallel-beam half circle */
  int fwd_tiles_y;             /* forward tile rows: Na, or base-angle pairs with bit 1 */
  int obwd_tiles_x, obwd_tiles_y;
  int sym_map[3][6];
} gr_batch_problem;
/* sizeof(gr_batch_problem), so bindings can check their struct layout. */
GR_API size_t gr_batch_problem_size(void);
/* items: 2*n ints (problem index, tile index); grid: persistent block count,
 * or <= 0 for one wave of resident blocks at the kernel's occupancy.
 * gr_batch_forward / gr_batch_backward take the problems without orbit bit 1
 * / bit 2; gr_batch_forward_orbit / gr_batch_backward_orbit those with it,
 * one geometry kind (GR_RADON or GR_FANBEAM) per call (items of other
 * problems are skipped). */
GR_API int gr_batch_forward(const gr_batch_problem* probs, const int* items, int n, int mode,
                            int grid, void* stream);
GR_API int gr_batch_backward(const gr_batch_problem* probs, const int* items, int n, int mode,
                             int grid, void* stream);
GR_API int gr_batch_forward_orbit(const gr_batch_problem* probs, const int* items, int n,
                                  int mode, int kind, int grid, void* stream);
GR_API int gr_batch_backward_orbit(const gr_batch_problem* probs, const int* items, int n,
                                   int mode, int kind, int grid, void* stream);
/* image-sized elementwise step over backprojection tiles: normest scaling,
 * CG p = beta p + snew, TV dual update */
GR_API int gr_batch_image_step(const gr_batch_problem* probs, const int* items, int n, int mode,
                               int grid, void* stream);
/* sinogram-sized elementwise step (CG d -= alpha q) over chunks of 256 bins */
GR_API int gr_batch_sino_step(const gr_batch_problem* probs, const int* items, int n, int mode,
                              int grid, void* stream);
/* per-problem scalar step, one block per listed problem (phase 0: after the
 * forward launch, phase 1: after the backprojection) */
GR_API int gr_batch_scalars(const gr_batch_problem* probs, const int* prob_ids, int n, int mode,
                            int phase, void* stream);

/* ---- Device-resident solver scalars ----
 * sc is a device array of GR_SC_COUNT doubles; see the GR_SC_* slots. */
enum {
  GR_SC_SOLD = 0,   /* <s_old, s_old> */
  GR_SC_ALPHA = 1,  /* CG step, rounded to the data precision */
  GR_SC_BETA = 2,   /* CG direction weight, rounded to the data precision */
  GR_SC_DSQ = 3,    /* <d, d> */
  GR_SC_FSQ = 4,    /* <sino, sino> */
  GR_SC_RES = 5,    /* relative residual */
  GR_SC_SUM = 6,    /* normest: current sum of the iterate */
  GR_SC_COUNT = 8
};
/* CG scalar steps (gratopy.py:2523-2547):
 * alpha = c * sold / sum(partials)           (c = delta_x^2 / delta_s)
 * d -= alpha q  (+ block partials of <d, d>)
 * sold <- sum(snew partials), beta = snew/sold, residual, done flag
 * p = beta p + snew */
GR_API int gr_cg_alpha(double* sc, const double* partials, size_t n, double c, int dtype,
                const int* skip, void* stream);
GR_API int gr_cg_update_d(void* d, const void* q, const double* sc, double* partials, int dtype,
                   size_t n, const int* skip, void* stream);
GR_API int gr_cg_beta(double* sc, const double* snew_partials, size_t n_snew,
               const double* d_partials, size_t n_d, double epsilon, int dtype, int* done,
               void* stream);
GR_API int gr_cg_update_p(void* p, const void* snew, const double* sc, int dtype, size_t n,
                   const int* skip, void* stream);
/* normest: img /= (real) sc[GR_SC_SUM] */
GR_API int gr_scale_by_sum(void* img, const double* sc, int dtype, size_t n, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* GRATOPY_GB300_H */
