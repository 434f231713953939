/*
 * Oracle (test infrastructure only): CPU restatement of gratopy's OpenCL
 * kernels, instantiated once per precision by gr_oracle.c with
 *   REAL  = float | double
 *   SFX   = f32   | f64
 * Every function follows the reference kernel arithmetic statement by
 * statement (same evaluation order, same int/float conversions, same
 * float-typed scale factors), one loop iteration per OpenCL work-item, and
 * parallelises over output elements with OpenMP to mirror the NDRange.
 *
 * Orders: 0 = "F" (x fastest), 1 = "C" (z fastest); see radon.cl:28-31.
 * Nothing outside tests/, bench.py's CPU baseline and smoke() may use this.
 */

#define CAT_(a, b) a##_##b
#define CAT(a, b) CAT_(a, b)
#define FN(name) CAT(name, SFX)

/* radon.cl:66-161 -- parallel-beam forward projection (ray-driven gather). */
void FN(or_radon_fwd)(REAL *sino, const REAL *img, const REAL *ofs,
                      const REAL *geo, int Ns, int Na, int Nz, int sino_order,
                      int img_order, int nthreads) {
  const int Nx = (int)geo[2];
  const int Ny = (int)geo[3];
  const float delta_x = (float)geo[0];
  const float delta_xi = (float)geo[1];
#pragma omp parallel for collapse(3) schedule(static) num_threads(nthreads)
  for (int z = 0; z < Nz; z++)
    for (int a = 0; a < Na; a++)
      for (int s = 0; s < Ns; s++) {
        int ss = s;
        const REAL *o8 = ofs + 8 * (size_t)a;
        REAL ox = o8[0], oy = o8[1], oz = o8[2], ow = o8[3];
        REAL reverse_mask = o8[5];
        int Nxx = Nx, Nyy = Ny, horizontal = 1;
        if (reverse_mask != (REAL)0.) {
          horizontal = 0;
          REAL t = ox;
          ox = oy;
          oy = t;
          Nxx = Ny;
          Nyy = Nx;
        }
        REAL acc = (REAL)0.;
        const REAL *img0 = img + pos_img(img_order, 0, 0, z, Nx, Ny, Nz);
        ptrdiff_t stride_x = horizontal == 1
                                 ? (ptrdiff_t)pos_img(img_order, 1, 0, 0, Nx, Ny, Nz)
                                 : (ptrdiff_t)pos_img(img_order, 0, 1, 0, Nx, Ny, Nz);
        for (int y = 0; y < Nyy; y++) {
          REAL d = (REAL)y * oy + oz - (REAL)ss;
          int x_low = (int)((-1 - d) * ow);
          int x_high = (int)((1 - d) * ow);
          if (ow < (REAL)0.) {
            int trade = x_low;
            x_low = x_high;
            x_high = trade;
          }
          x_low = x_low > 0 ? x_low : 0;
          x_high = x_high < Nxx - 1 ? x_high : Nxx - 1;
          const REAL *p;
          if (horizontal == 1)
            p = img0 + pos_img(img_order, (size_t)x_low, y, 0, Nx, Ny, Nz);
          else
            p = img0 + pos_img(img_order, y, (size_t)x_low, 0, Nx, Ny, Nz);
          for (int x = x_low; x <= x_high; x++) {
            REAL weight = (REAL)1. - FABS((REAL)x * ox + d);
            if (weight > (REAL)0.) acc += weight * p[0];
            p += stride_x;
          }
        }
        sino[pos_sino(sino_order, s, a, z, Ns, Na, Nz)] =
            acc * delta_x * delta_x / delta_xi;
      }
}

/* radon.cl:183-241 -- parallel-beam backprojection (2-tap interpolation). */
void FN(or_radon_bwd)(REAL *img, const REAL *sino, const REAL *ofs,
                      const REAL *geo, int Nx, int Ny, int Nz, int img_order,
                      int sino_order, int nthreads) {
  const int Ns = (int)geo[4];
  const int Na = (int)geo[5];
#pragma omp parallel for collapse(3) schedule(static) num_threads(nthreads)
  for (int z = 0; z < Nz; z++)
    for (int y = 0; y < Ny; y++)
      for (int x = 0; x < Nx; x++) {
        REAL acc = (REAL)0.;
        REAL cx = (REAL)x, cy = (REAL)y;
        const REAL *sn = sino + pos_sino(sino_order, 0, 0, z, Ns, Na, Nz);
        for (int a = 0; a < Na; a++) {
          const REAL *o = ofs + 8 * (size_t)a;
          REAL Delta_phi = o[4];
          REAL s = cx * o[0] + cy * o[1] + o[2];
          int sm = (int)FLOOR(s);
          int sp = sm + 1;
          REAL weightp = 1 - ((REAL)sp - s);
          REAL weightm = 1 - (s - (REAL)sm);
          if (sm < 0 || sm >= Ns) {
            weightm = (REAL)0.;
            sm = 0;
          }
          if (sp < 0 || sp >= Ns) {
            weightp = (REAL)0.;
            sp = 0;
          }
          acc += Delta_phi * (weightm * sn[pos_sino(sino_order, sm, a, 0, Ns, Na, Nz)] +
                              weightp * sn[pos_sino(sino_order, sp, a, 0, Ns, Na, Nz)]);
        }
        img[pos_img(img_order, x, y, z, Nx, Ny, Nz)] = acc;
      }
}

/* fanbeam.cl:72-256 -- fan-beam forward projection. */
void FN(or_fan_fwd)(REAL *sino, const REAL *img, const REAL *ofs,
                    const REAL *sdpd, const REAL *geo, int Ns, int Na, int Nz,
                    int sino_order, int img_order, int nthreads) {
  const int Nx = (int)geo[6];
  const int Ny = (int)geo[7];
#pragma omp parallel for collapse(3) schedule(static) num_threads(nthreads)
  for (int z = 0; z < Nz; z++)
    for (int a = 0; a < Na; a++)
      for (int s = 0; s < Ns; s++) {
        REAL midx = geo[3], midy = geo[4];
        REAL midpoint_det = geo[5];
        REAL R = geo[0], RE = geo[1], delta_xi = geo[2], delta_x = geo[10];
        const REAL *o = ofs + 8 * (size_t)a;
        REAL dx = o[0], dy = o[1];
        REAL qx = o[2], qy = o[3];
        REAL d0x = o[4], d0y = o[5];
        REAL acc = (REAL)0.;
        REAL sr = (REAL)s;
        REAL fp = -midpoint_det + sr + 1;
        REAL fm = -midpoint_det + sr - 1;
        REAL dpx = d0x + dx * fp - qx, dpy = d0y + dy * fp - qy;
        REAL dmx = d0x + dx * fm - qx, dmy = d0y + dy * fm - qy;
        REAL ddx = d0x - qx, ddy = d0y - qy;
        REAL RR = R * R;
        ddx /= RR;
        ddy /= RR;
        REAL xx2 = delta_xi * delta_xi;
        dx /= xx2;
        dy /= xx2;
        RE *= 1 / R;
        int Nyy = Ny, Nxx = Nx, horizontal;
        if (FABS(dpx) < FABS(dpy) && FABS(dmx) < FABS(dmy)) {
          horizontal = 1;
        } else {
          horizontal = 0;
          REAL t;
          t = ddx; ddx = ddy; ddy = t;
          t = dx; dx = dy; dy = t;
          t = qx; qx = qy; qy = t;
          t = dpx; dpx = dpy; dpy = t;
          t = dmx; dmx = dmy; dmy = t;
          t = midx; midx = midy; midy = t;
          Nyy = Nx;
          Nxx = Ny;
        }
        dpx /= dpy;
        dmx /= dmy;
        REAL xlow = qx - dmx * (qy + midy);
        REAL xhigh = qx - dpx * (qy + midy);
        if ((qy) * (dmx - dpx) < (REAL)0.) {
          REAL trade = xhigh;
          xhigh = xlow;
          xlow = trade;
          trade = dpx;
          dpx = dmx;
          dmx = trade;
        }
        REAL s_midpoint_det = sr - midpoint_det;
        const REAL *img0 = img + pos_img(img_order, 0, 0, z, Nx, Ny, Nz);
        ptrdiff_t stride_x = (horizontal != 0)
                                 ? (ptrdiff_t)pos_img(img_order, 1, 0, 0, Nx, Ny, Nz)
                                 : (ptrdiff_t)pos_img(img_order, 0, 1, 0, Nx, Ny, Nz);
        for (int y = 0; y < Nyy; y++) {
          REAL yr = (REAL)y;
          xhigh = qx + dpx * (yr - midy - qy);
          xlow = qx + dmx * (yr - midy - qy);
          REAL hi_lim = (REAL)(Nxx - 1) - midx;
          REAL lo_lim = -midx;
          int xhighint = (int)FLOOR(FMIN(hi_lim, xhigh) + midx);
          int xlowint = (int)CEIL(FMAX(lo_lim, xlow) + midx);
          REAL t = ddx * ((REAL)xlowint - midx) + ddy * (yr - midy) + RE;
          REAL ss = dx * ((REAL)xlowint - midx) + dy * (yr - midy);
          const REAL *p;
          if (xlowint > xhighint) continue;
          if (horizontal != 0)
            p = img0 + pos_img(img_order, (size_t)xlowint, y, 0, Nx, Ny, Nz);
          else
            p = img0 + pos_img(img_order, y, (size_t)xlowint, 0, Nx, Ny, Nz);
          for (int x = xlowint; x <= xhighint; x++) {
            REAL xi = ss / t;
            REAL Weight = ((REAL)1. - FABS(s_midpoint_det - xi)) / t;
            acc += Weight * p[0];
            p += stride_x;
            t += ddx;
            ss += dx;
          }
        }
        sino[pos_sino(sino_order, s, a, z, Ns, Na, Nz)] =
            acc * sdpd[s] / delta_xi * delta_x / R;
      }
}

/* fanbeam.cl:290-391 -- fan-beam backprojection. */
void FN(or_fan_bwd)(REAL *img, const REAL *sino, const REAL *ofs,
                    const REAL *sdpd, const REAL *geo, int Nx, int Ny, int Nz,
                    int img_order, int sino_order, int nthreads) {
  const int Ns = (int)geo[8];
  const int Na = (int)geo[9];
#pragma omp parallel for collapse(3) schedule(static) num_threads(nthreads)
  for (int z = 0; z < Nz; z++)
    for (int yy = 0; yy < Ny; yy++)
      for (int xx = 0; xx < Nx; xx++) {
        REAL midx = geo[3], midy = geo[4];
        REAL midpoint_det = geo[5];
        REAL delta_xi = geo[2];
        REAL R = geo[0];
        REAL Px = (REAL)xx - midx, Py = (REAL)yy - midy;
        REAL acc = (REAL)0.;
        const REAL *sn = sino + pos_sino(sino_order, 0, 0, z, Ns, Na, Nz);
        REAL R_sqr_inv = (REAL)1. / (R * R);
        REAL delta_xi_sqr_inv = (REAL)1. / (delta_xi * delta_xi);
        for (int a = 0; a < Na; a++) {
          const REAL *o = ofs + 8 * (size_t)a;
          REAL dx = o[0], dy = o[1];
          REAL qx = o[2], qy = o[3];
          REAL d0x = o[4], d0y = o[5];
          REAL ddx = d0x - qx, ddy = d0y - qy;
          REAL Delta_Phi = o[6];
          ddx *= R_sqr_inv;
          ddy *= R_sqr_inv;
          dx *= delta_xi_sqr_inv;
          dy *= delta_xi_sqr_inv;
          REAL pqx = Px - qx, pqy = Py - qy;
          REAL t = ddx * pqx + ddy * pqy;
          REAL ss = dx * pqx + dy * pqy;
          REAL xi = ss / t + midpoint_det;
          int xim = (int)FLOOR(xi);
          int xip = xim + 1;
          REAL Weightp = (REAL)1. - ((REAL)xip - xi);
          REAL Weightm = (REAL)1. - (xi - (REAL)xim);
          if (xim < 0 || xim >= Ns) {
            Weightm = (REAL)0.;
            xim = 0;
          } else {
            Weightm *= sdpd[xim];
          }
          if (xip < 0 || xip >= Ns) {
            Weightp = (REAL)0.;
            xip = 0;
          } else {
            Weightp *= sdpd[xip];
          }
          acc += Delta_Phi *
                 (Weightm * sn[pos_sino(sino_order, xim, a, 0, Ns, Na, Nz)] +
                  Weightp * sn[pos_sino(sino_order, xip, a, 0, Ns, Na, Nz)]) /
                 (R * t);
        }
        img[pos_img(img_order, xx, yy, z, Nx, Ny, Nz)] = acc;
      }
}

/* total_variation.cl:54-93 -- v += sigma * grad(u); v holds 4 reals/pixel. */
void FN(or_tv_update_v)(REAL *v, const REAL *u, float sigma, float z_distance,
                        int Nx, int Ny, int Nz, int order, int nthreads) {
  ptrdiff_t sx = (ptrdiff_t)pos_img(order, 1, 0, 0, Nx, Ny, Nz);
  ptrdiff_t sy = (ptrdiff_t)pos_img(order, 0, 1, 0, Nx, Ny, Nz);
  ptrdiff_t sz = (ptrdiff_t)pos_img(order, 0, 0, 1, Nx, Ny, Nz);
#pragma omp parallel for collapse(3) schedule(static) num_threads(nthreads)
  for (int z = 0; z < Nz; z++)
    for (int y = 0; y < Ny; y++)
      for (int x = 0; x < Nx; x++) {
        size_t i = pos_img(order, x, y, z, Nx, Ny, Nz);
        const REAL *up = u + i;
        REAL v0 = -up[0], v1 = -up[0], v2 = -up[0];
        if (x < Nx - 1) v0 += up[sx]; else v0 = (REAL)0.;
        if (y < Ny - 1) v1 += up[sy]; else v1 = (REAL)0.;
        if (z < Nz - 1) v2 += up[sz]; else v2 = (REAL)0.;
        if (z_distance > 0) v2 /= z_distance; else v2 = (REAL)0.;
        REAL *vp = v + 4 * i;
        vp[0] += sigma * v0;
        vp[1] += sigma * v1;
        vp[2] += sigma * v2;
      }
}

/* total_variation.cl:150-167 -- pointwise projection onto the unit ball. */
void FN(or_tv_normv)(REAL *v, size_t n, int nthreads) {
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (size_t i = 0; i < n; i++) {
    REAL *vp = v + 4 * i;
    REAL norm = HYPOT(HYPOT(vp[0], vp[1]), vp[2]);
    if (norm > (REAL)1.) {
      vp[0] /= norm;
      vp[1] /= norm;
      vp[2] /= norm;
    }
  }
}

/* total_variation.cl:95-106 -- lambda = (lambda + sigma (Ku - f)) * mu''. */
void FN(or_tv_update_lambda)(REAL *lambda, const REAL *Ku, const REAL *f,
                             float sigma, float sigmap1inv, size_t n,
                             int nthreads) {
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (size_t i = 0; i < n; i++)
    lambda[i] = (lambda[i] + sigma * (Ku[i] - f[i])) * sigmap1inv;
}

/* total_variation.cl:108-148 -- u = max(0, u_ + tau (div v - norming K*l)). */
void FN(or_tv_update_u)(REAL *u, const REAL *u_, const REAL *v,
                        const REAL *Kstarlambda, float tau, float norming,
                        float z_distance, int Nx, int Ny, int Nz, int order,
                        int nthreads) {
  ptrdiff_t sx = (ptrdiff_t)pos_img(order, 1, 0, 0, Nx, Ny, Nz);
  ptrdiff_t sy = (ptrdiff_t)pos_img(order, 0, 1, 0, Nx, Ny, Nz);
  ptrdiff_t sz = (ptrdiff_t)pos_img(order, 0, 0, 1, Nx, Ny, Nz);
#pragma omp parallel for collapse(3) schedule(static) num_threads(nthreads)
  for (int z = 0; z < Nz; z++)
    for (int y = 0; y < Ny; y++)
      for (int x = 0; x < Nx; x++) {
        size_t i = pos_img(order, x, y, z, Nx, Ny, Nz);
        const REAL *vp = v + 4 * i;
        REAL v0 = vp[0], v1 = vp[1], v2 = vp[2];
        if (x == Nx - 1) v0 = (REAL)0.;
        if (x > 0) v0 -= vp[-4 * sx + 0];
        if (y == Ny - 1) v1 = (REAL)0.;
        if (y > 0) v1 -= vp[-4 * sy + 1];
        if (z == Nz - 1) v2 = (REAL)0.;
        if (z > 0) v2 -= vp[-4 * sz + 2];
        if (z_distance > 0) v2 /= z_distance; else v2 = 0;
        REAL val = u_[i] + tau * (v0 + v1 + v2 - norming * Kstarlambda[i]);
        u[i] = FMAX((REAL)0., val);
      }
}

/* gratopy.py:2708-2717 -- u = 2.0f*u_ - u (ElementwiseKernel). */
void FN(or_tv_extra)(const REAL *u_, REAL *u, size_t n, int nthreads) {
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (size_t i = 0; i < n; i++) u[i] = 2.0f * u_[i] - u[i];
}

/* utilities.cl:38-67 -- sinogram angle weighting (multiply or divide). */
void FN(or_weight_sino)(REAL *out, const REAL *sino, const REAL *w, int Ns,
                        int Na, int Nz, int order, int divide, int nthreads) {
#pragma omp parallel for collapse(3) schedule(static) num_threads(nthreads)
  for (int z = 0; z < Nz; z++)
    for (int a = 0; a < Na; a++)
      for (int s = 0; s < Ns; s++) {
        size_t i = pos_sino(order, s, a, z, Ns, Na, Nz);
        out[i] = divide ? sino[i] / w[a] : sino[i] * w[a];
      }
}

/* utilities.cl:69-73 -- rhs += a * x. */
void FN(or_equ_mul_add)(REAL *rhs, REAL a, const REAL *x, size_t n,
                        int nthreads) {
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (size_t i = 0; i < n; i++) rhs[i] += a * x[i];
}

/* utilities.cl:75-80 -- rhs = a * x + y. */
void FN(or_mul_add_add)(REAL *rhs, REAL a, const REAL *x, const REAL *y,
                        size_t n, int nthreads) {
#pragma omp parallel for schedule(static) num_threads(nthreads)
  for (size_t i = 0; i < n; i++) rhs[i] = a * x[i] + y[i];
}

/* FP64 dot product (the reduction the GPU path uses for CG/Landweber). */
double FN(or_dot_f64)(const REAL *a, const REAL *b, size_t n, int nthreads) {
  double acc = 0.0;
#pragma omp parallel for reduction(+ : acc) schedule(static) num_threads(nthreads)
  for (size_t i = 0; i < n; i++) acc += (double)a[i] * (double)b[i];
  return acc;
}

#undef FN
#undef CAT
#undef CAT_
