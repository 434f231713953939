/*
 * Oracle (test infrastructure only, never on the product path): plain-C CPU
 * restatement of gratopy's OpenCL kernels, used by tests/ as the checker,
 * by bench.py as the timed CPU baseline and by __graft_entry__.smoke().
 *
 * Reference kernels restated (file:line in the gratopy project):
 *   radon.cl:66-161      radon_{T}_{so}{io}        -> or_radon_fwd_*
 *   radon.cl:183-241     radon_ad_{T}_{io}{so}     -> or_radon_bwd_*
 *   fanbeam.cl:72-256    fanbeam_{T}_{so}{io}      -> or_fan_fwd_*
 *   fanbeam.cl:290-391   fanbeam_ad_{T}_{io}{so}   -> or_fan_bwd_*
 *   total_variation.cl:54-167                      -> or_tv_*
 *   utilities.cl:38-80                             -> or_weight_sino_*, or_equ_mul_add_*, or_mul_add_add_*
 * Built with -ffp-contract=off so every product and sum rounds as written.
 */
#include <math.h>
#include <stddef.h>

static inline size_t pos_img(int order, size_t x, size_t y, size_t z, size_t Nx,
                             size_t Ny, size_t Nz) {
  return order == 0 ? x + Nx * (y + Ny * z) : z + Nz * (y + Ny * x);
}
static inline size_t pos_sino(int order, size_t s, size_t a, size_t z,
                              size_t Ns, size_t Na, size_t Nz) {
  return order == 0 ? s + Ns * (a + Na * z) : z + Nz * (a + Na * s);
}

int or_version(void) { return 1; }

#define REAL float
#define SFX f32
#define FABS fabsf
#define FLOOR floorf
#define CEIL ceilf
#define FMIN fminf
#define FMAX fmaxf
#define HYPOT hypotf
#include "gr_oracle_impl.h"
#undef REAL
#undef SFX
#undef FABS
#undef FLOOR
#undef CEIL
#undef FMIN
#undef FMAX
#undef HYPOT

#define REAL double
#define SFX f64
#define FABS fabs
#define FLOOR floor
#define CEIL ceil
#define FMIN fmin
#define FMAX fmax
#define HYPOT hypot
#include "gr_oracle_impl.h"
