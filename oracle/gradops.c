/*
 * gradops.c -- CPU restatement of the gradient-type operators of the PN-PN
 * splitting step (TEST INFRASTRUCTURE ONLY: the oracle the device operators
 * are checked against; never linked into the product).  Arithmetic in the
 * reference's order (mxm sums over the inner index left to right, products
 * and sums unfused: built with -ffp-contract=off).
 *
 *   wgradm1  core/navier1.f:4170-4230  weak gradient (opgrad for PN-PN)
 *   cdtp     core/navier1.f:330-470    D^T x, the PN-PN (ifsplit) 3-D branch
 *   dudxyz   core/navier1.f:1156-1220  strong derivative du/dx_isd
 *   op_curl  core/plan4.f:368-430      curl, averaged when ifavg
 *
 * rst: the metric terms rxm1..tzm1 as nine arrays of n (rx ry rz sx sy sz tx
 * ty tz, ref_geom_rst); jac: jacm1.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "nekref.h"

void ref_zwgll(double *z, double *w, int np);
void ref_dgll(double *d, double *dt, const double *zin, int nz);

static void dmat(int nx1, double *d, double *dt, double *w3) {
  double z[32], w[32];
  ref_zwgll(z, w, nx1);
  ref_dgll(d, dt, z, nx1);
  if (w3)
    for (int k = 0; k < nx1; ++k)
      for (int j = 0; j < nx1; ++j)
        for (int i = 0; i < nx1; ++i) w3[i + nx1 * (j + nx1 * k)] = w[i] * w[j] * w[k];
}

void ref_wgradm1(int nx1, int nel, double *ux, double *uy, double *uz, const double *u,
                 const double *rst) {
  const int nxyz = nx1 * nx1 * nx1;
  const int64_t n = (int64_t)nxyz * nel;
  double d[1024], dt[1024];
  double *w3 = (double *)malloc(sizeof(double) * nxyz);
  double *ur = (double *)malloc(sizeof(double) * 3 * nxyz), *us = ur + nxyz, *ut = us + nxyz;
  dmat(nx1, d, dt, w3);
  const double *rx = rst, *ry = rst + n, *rz = rst + 2 * n, *sx = rst + 3 * n, *sy = rst + 4 * n,
               *sz = rst + 5 * n, *tx = rst + 6 * n, *ty = rst + 7 * n, *tz = rst + 8 * n;
  for (int e = 0; e < nel; ++e) {
    const int64_t o = (int64_t)nxyz * e;
    ref_local_grad3(ur, us, ut, u + o, nx1 - 1, d, dt);
    for (int i = 0; i < nxyz; ++i) {
      const int64_t p = o + i;
      ux[p] = w3[i] * (ur[i] * rx[p] + us[i] * sx[p] + ut[i] * tx[p]);
      uy[p] = w3[i] * (ur[i] * ry[p] + us[i] * sy[p] + ut[i] * ty[p]);
      uz[p] = w3[i] * (ur[i] * rz[p] + us[i] * sz[p] + ut[i] * tz[p]);
    }
  }
  free(w3);
  free(ur);
}

/* isd = 1, 2, 3: the metric terms of x, y or z (rm2 = rxm1 ... as cdtp's
 * callers pass them) */
void ref_cdtp(int nx1, int nel, double *dtx, const double *x, const double *rst,
              const double *jac, const double *bm1, int isd) {
  const int nxyz = nx1 * nx1 * nx1;
  const int64_t n = (int64_t)nxyz * nel;
  double d[1024], dt[1024];
  double *wx = (double *)malloc(sizeof(double) * 5 * nxyz);
  double *ta = wx + nxyz, *tb = ta + nxyz, *tc = tb + nxyz, *wk = tc + nxyz;
  dmat(nx1, d, dt, NULL);
  const double *rm = rst + (int64_t)(isd - 1) * n, *sm = rst + (int64_t)(isd + 2) * n,
               *tm = rst + (int64_t)(isd + 5) * n;
  for (int e = 0; e < nel; ++e) {
    const int64_t o = (int64_t)nxyz * e;
    for (int i = 0; i < nxyz; ++i) {
      wx[i] = bm1[o + i] * x[o + i]; /* col3 */
      wx[i] = wx[i] / jac[o + i];    /* invcol2 */
    }
    for (int i = 0; i < nxyz; ++i) {
      ta[i] = wx[i] * rm[o + i];
      tb[i] = wx[i] * sm[o + i];
      tc[i] = wx[i] * tm[o + i];
    }
    ref_local_grad3_t(dtx + o, ta, tb, tc, nx1 - 1, d, dt, wk);
  }
  free(wx);
}

void ref_dudxyz(int nx1, int nel, double *du, const double *u, const double *rst,
                const double *jac, int isd) {
  const int nxyz = nx1 * nx1 * nx1;
  const int64_t n = (int64_t)nxyz * nel;
  double d[1024], dt[1024];
  double *ur = (double *)malloc(sizeof(double) * 3 * nxyz), *us = ur + nxyz, *ut = us + nxyz;
  dmat(nx1, d, dt, NULL);
  const double *rm = rst + (int64_t)(isd - 1) * n, *sm = rst + (int64_t)(isd + 2) * n,
               *tm = rst + (int64_t)(isd + 5) * n;
  for (int e = 0; e < nel; ++e) {
    const int64_t o = (int64_t)nxyz * e;
    ref_local_grad3(ur, us, ut, u + o, nx1 - 1, d, dt);
    for (int i = 0; i < nxyz; ++i) {
      double v = ur[i] * rm[o + i];    /* col2 */
      v = v + us[i] * sm[o + i];       /* addcol3 */
      v = v + ut[i] * tm[o + i];       /* addcol3 */
      const double jacmi = 1.0 / jac[o + i];
      du[o + i] = v * jacmi;           /* col2 by jacmi */
    }
  }
  free(ur);
}

void ref_op_curl(const ref_ops *ops, double *w1, double *w2, double *w3, const double *u1,
                 const double *u2, const double *u3, int ifavg, const double *rst,
                 const double *jac, const double *bm1, const double *binv) {
  const int nx1 = ref_ops_nx1(ops), nel = ref_ops_nel(ops);
  const int64_t n = ref_ops_n(ops);
  double *a = (double *)malloc(sizeof(double) * 2 * n), *b = a + n;
  ref_dudxyz(nx1, nel, a, u3, rst, jac, 2);
  ref_dudxyz(nx1, nel, b, u2, rst, jac, 3);
  for (int64_t i = 0; i < n; ++i) w1[i] = a[i] - b[i];
  ref_dudxyz(nx1, nel, a, u1, rst, jac, 3);
  ref_dudxyz(nx1, nel, b, u3, rst, jac, 1);
  for (int64_t i = 0; i < n; ++i) w2[i] = a[i] - b[i];
  ref_dudxyz(nx1, nel, a, u2, rst, jac, 1);
  ref_dudxyz(nx1, nel, b, u1, rst, jac, 2);
  for (int64_t i = 0; i < n; ++i) w3[i] = a[i] - b[i];
  if (ifavg) {
    double *w[3] = {w1, w2, w3};
    for (int c = 0; c < 3; ++c) {
      for (int64_t i = 0; i < n; ++i) w[c][i] = w[c][i] * bm1[i];
      ref_dssum(ops, w[c]);
      for (int64_t i = 0; i < n; ++i) w[c][i] = w[c][i] * binv[i];
    }
  }
  free(a);
}

/* ---- the splitting step's residuals ---------------------------------------- */

/* cresvsp (core/plan4.f:264-306), PN-PN without the stress formulation:
 * resv = -A(h1, h2) v - wgradm1(pr - vdiff qtl / 3) + bf, per component. */
void ref_cresvsp(const ref_ops *ops, double *r1, double *r2, double *r3, const double *vx,
                 const double *vy, const double *vz, const double *h1, const double *h2,
                 const double *vdiff, const double *qtl, const double *pr, const double *bfx,
                 const double *bfy, const double *bfz, const double *rst) {
  const int nx1 = ref_ops_nx1(ops), nel = ref_ops_nel(ops);
  const int64_t n = ref_ops_n(ops);
  double *ta = (double *)malloc(sizeof(double) * 4 * n), *t1 = ta + n, *t2 = t1 + n, *t3 = t2 + n;
  double *r[3] = {r1, r2, r3};
  const double *v[3] = {vx, vy, vz}, *bf[3] = {bfx, bfy, bfz};
  for (int c = 0; c < 3; ++c) ref_axhelm(ops, r[c], v[c], h1, h2); /* ophx */
  for (int c = 0; c < 3; ++c)
    for (int64_t i = 0; i < n; ++i) r[c][i] = -r[c][i];             /* opchsgn */
  const double scale = -1. / 3.;
  for (int64_t i = 0; i < n; ++i) {
    ta[i] = vdiff[i] * qtl[i];       /* col3 */
    ta[i] = scale * ta[i] + pr[i];   /* add2s1 */
  }
  ref_wgradm1(nx1, nel, t1, t2, t3, ta, rst); /* opgrad */
  const double *t[3] = {t1, t2, t3};
  for (int c = 0; c < 3; ++c)
    for (int64_t i = 0; i < n; ++i) {
      r[c][i] = r[c][i] - t[c][i];   /* opsub2 */
      r[c][i] = r[c][i] + bf[c][i];  /* opadd2 */
    }
  free(ta);
}

/* cresvsp_weak (core/plan4.f:308-361), the velocity residual of the stress
 * formulation's branch of plan4 (:84-86): the pressure enters through its
 * weak gradient (cdtp of pr per direction) instead of the strong one,
 * resv = -A(h1, h2) v - (wgradm1(scale vdiff qtl) - cdtp(pr)) + bf, per
 * component, with scale = 2/3 (stress formulation) or -1/3. */
void ref_cresvsp_weak(const ref_ops *ops, double *r1, double *r2, double *r3, const double *vx,
                      const double *vy, const double *vz, const double *h1, const double *h2,
                      const double *vdiff, const double *qtl, const double *pr,
                      const double *bfx, const double *bfy, const double *bfz,
                      const double *rst, const double *jac, const double *bm1, int stress) {
  const int nx1 = ref_ops_nx1(ops), nel = ref_ops_nel(ops);
  const int64_t n = ref_ops_n(ops);
  double *ta = (double *)malloc(sizeof(double) * 5 * n), *t1 = ta + n, *t2 = t1 + n,
         *t3 = t2 + n, *wa = t3 + n;
  double *r[3] = {r1, r2, r3};
  const double *v[3] = {vx, vy, vz}, *bf[3] = {bfx, bfy, bfz};
  for (int c = 0; c < 3; ++c) ref_axhelm(ops, r[c], v[c], h1, h2); /* ophx */
  for (int c = 0; c < 3; ++c)
    for (int64_t i = 0; i < n; ++i) r[c][i] = -r[c][i];             /* opchsgn */
  const double scale = stress ? 2. / 3. : -1. / 3.;
  for (int64_t i = 0; i < n; ++i) {
    ta[i] = vdiff[i] * qtl[i]; /* col3 */
    ta[i] = ta[i] * scale;     /* cmult */
  }
  ref_wgradm1(nx1, nel, t1, t2, t3, ta, rst); /* opgrad */
  double *t[3] = {t1, t2, t3};
  for (int c = 0; c < 3; ++c) {
    ref_cdtp(nx1, nel, wa, pr, rst, jac, bm1, c + 1);           /* cdtp(wa, pr, r/s/t x|y|z m1) */
    for (int64_t i = 0; i < n; ++i) t[c][i] = t[c][i] - wa[i];  /* sub2 */
  }
  for (int c = 0; c < 3; ++c)
    for (int64_t i = 0; i < n; ++i) {
      r[c][i] = r[c][i] - t[c][i];   /* opsub2 */
      r[c][i] = r[c][i] + bf[c][i];  /* opadd2 */
    }
  free(ta);
}

/* ---- the stress formulation's coupled velocity operator and solve --------- */

/* axsf_e_3d over every element (core/subs1.f:2031-2116, the default "fast"
 * path of axhmsf, :1240-1315, for a fluid, matmod = 0): the velocity gradient
 * from local_grad3 and the metric terms, the symmetric strain times
 * h1 w3 / J, contracted back with the metric terms and local_grad3_t, plus
 * h2 B u per component. */
void ref_axsf(const ref_ops *ops, double *au, double *av, double *aw, const double *u,
              const double *v, const double *w, const double *h1, const double *h2,
              const double *rst, const double *jac, const double *bm1) {
  const int nx1 = ref_ops_nx1(ops), nel = (int)(ref_ops_n(ops) / ((int64_t)nx1 * nx1 * nx1));
  const int nxyz = nx1 * nx1 * nx1;
  const int64_t n = ref_ops_n(ops);
  double d[1024], dt[1024];
  double *w3 = (double *)malloc(sizeof(double) * nxyz);
  double *ur = (double *)malloc(sizeof(double) * 10 * nxyz); /* ur(i, 3, 3) + work */
  double *wk = ur + 9 * nxyz;
  dmat(nx1, d, dt, w3);
  const double *rx = rst, *ry = rst + n, *rz = rst + 2 * n, *sx = rst + 3 * n, *sy = rst + 4 * n,
               *sz = rst + 5 * n, *tx = rst + 6 * n, *ty = rst + 7 * n, *tz = rst + 8 * n;
#define UR(i, a, b) ur[(i) + nxyz * ((a) + 3 * (b))]
  for (int e = 0; e < nel; ++e) {
    const int64_t o = (int64_t)nxyz * e;
    ref_local_grad3(&UR(0, 0, 0), &UR(0, 1, 0), &UR(0, 2, 0), u + o, nx1 - 1, d, dt);
    ref_local_grad3(&UR(0, 0, 1), &UR(0, 1, 1), &UR(0, 2, 1), v + o, nx1 - 1, d, dt);
    ref_local_grad3(&UR(0, 0, 2), &UR(0, 1, 2), &UR(0, 2, 2), w + o, nx1 - 1, d, dt);
    for (int i = 0; i < nxyz; ++i) {
      const int64_t q = o + i;
      const double u1 = UR(i, 0, 0) * rx[q] + UR(i, 1, 0) * sx[q] + UR(i, 2, 0) * tx[q];
      const double u2 = UR(i, 0, 0) * ry[q] + UR(i, 1, 0) * sy[q] + UR(i, 2, 0) * ty[q];
      const double u3 = UR(i, 0, 0) * rz[q] + UR(i, 1, 0) * sz[q] + UR(i, 2, 0) * tz[q];
      const double v1 = UR(i, 0, 1) * rx[q] + UR(i, 1, 1) * sx[q] + UR(i, 2, 1) * tx[q];
      const double v2 = UR(i, 0, 1) * ry[q] + UR(i, 1, 1) * sy[q] + UR(i, 2, 1) * ty[q];
      const double v3 = UR(i, 0, 1) * rz[q] + UR(i, 1, 1) * sz[q] + UR(i, 2, 1) * tz[q];
      const double w1 = UR(i, 0, 2) * rx[q] + UR(i, 1, 2) * sx[q] + UR(i, 2, 2) * tx[q];
      const double w2 = UR(i, 0, 2) * ry[q] + UR(i, 1, 2) * sy[q] + UR(i, 2, 2) * ty[q];
      const double ww3 = UR(i, 0, 2) * rz[q] + UR(i, 1, 2) * sz[q] + UR(i, 2, 2) * tz[q];
      const double dj = h1[q] * w3[i] * (1.0 / jac[q]);
      const double s11 = dj * (u1 + u1), s12 = dj * (u2 + v1), s13 = dj * (u3 + w1);
      const double s21 = dj * (v1 + u2), s22 = dj * (v2 + v2), s23 = dj * (v3 + w2);
      const double s31 = dj * (w1 + u3), s32 = dj * (w2 + v3), s33 = dj * (ww3 + ww3);
      UR(i, 0, 0) = rx[q] * s11 + ry[q] * s12 + rz[q] * s13;
      UR(i, 1, 0) = sx[q] * s11 + sy[q] * s12 + sz[q] * s13;
      UR(i, 2, 0) = tx[q] * s11 + ty[q] * s12 + tz[q] * s13;
      UR(i, 0, 1) = rx[q] * s21 + ry[q] * s22 + rz[q] * s23;
      UR(i, 1, 1) = sx[q] * s21 + sy[q] * s22 + sz[q] * s23;
      UR(i, 2, 1) = tx[q] * s21 + ty[q] * s22 + tz[q] * s23;
      UR(i, 0, 2) = rx[q] * s31 + ry[q] * s32 + rz[q] * s33;
      UR(i, 1, 2) = sx[q] * s31 + sy[q] * s32 + sz[q] * s33;
      UR(i, 2, 2) = tx[q] * s31 + ty[q] * s32 + tz[q] * s33;
    }
    ref_local_grad3_t(au + o, &UR(0, 0, 0), &UR(0, 1, 0), &UR(0, 2, 0), nx1 - 1, d, dt, wk);
    ref_local_grad3_t(av + o, &UR(0, 0, 1), &UR(0, 1, 1), &UR(0, 2, 1), nx1 - 1, d, dt, wk);
    ref_local_grad3_t(aw + o, &UR(0, 0, 2), &UR(0, 1, 2), &UR(0, 2, 2), nx1 - 1, d, dt, wk);
    for (int i = 0; i < nxyz; ++i) {
      const int64_t q = o + i;
      au[q] = au[q] + h2[q] * bm1[q] * u[q];
      av[q] = av[q] + h2[q] * bm1[q] * v[q];
      aw[q] = aw[q] + h2[q] * bm1[q] * w[q];
    }
  }
#undef UR
  free(w3);
  free(ur);
}

/* hmhzsf (core/subs1.f:1093-1147) without the projection onto previous
 * solutions (param(94) = 0): rmask (the volume masks of qmask, :1800-1860),
 * opdssum, u = 0, chktcgs (:1149-1238), then cggosf (:2-165): Jacobi-PCG on
 * the coupled system with dpc the sum of the three setprec diagonals and the
 * loop capped at 200 iterations, as the reference sets it.  tol is the
 * absolute tolerance on sqrt(sum binv mult |r|^2 / vol).  Sums run serially
 * over the points.  Returns the iteration count (-1: the cap was reached). */
static double sf_wdot(int64_t n, const double *a1, const double *a2, const double *a3,
                      const double *b1, const double *b2, const double *b3, const double *wt) {
  double s = 0.0;
  for (int64_t i = 0; i < n; ++i) s = s + wt[i] * (a1[i] * b1[i] + a2[i] * b2[i] + a3[i] * b3[i]);
  return s;
}

int ref_hmhzsf(const ref_ops *ops, double *u1, double *u2, double *u3, double *r1, double *r2,
               double *r3, const double *h1, const double *h2, const double *m1,
               const double *m2, const double *m3, const double *mult, const double *binv,
               const double *rst, const double *jac, const double *bm1, double vol, double tin,
               double *rbn0, double *rbn2) {
  const int64_t n = ref_ops_n(ops);
  double *r[3] = {r1, r2, r3}, *u[3] = {u1, u2, u3};
  const double *m[3] = {m1, m2, m3};
  double *buf = (double *)malloc(sizeof(double) * 11 * n);
  double *dpc = buf, *wa = buf + n, *p[3] = {buf + 2 * n, buf + 3 * n, buf + 4 * n},
         *pp[3] = {buf + 5 * n, buf + 6 * n, buf + 7 * n},
         *ap[3] = {buf + 8 * n, buf + 9 * n, buf + 10 * n};
  for (int c = 0; c < 3; ++c) {
    for (int64_t i = 0; i < n; ++i) r[c][i] = r[c][i] * m[c][i]; /* rmask */
    ref_dssum(ops, r[c]);                                          /* opdssum */
    for (int64_t i = 0; i < n; ++i) u[c][i] = 0.0;
  }
  /* chktcgs (EIGAA = 0: ACONDNO = 10; FP64: EPS = 1e-13) */
  double tol = tin;
  {
    for (int64_t i = 0; i < n; ++i) wa[i] = r1[i] * r1[i] + r2[i] * r2[i] + r3[i] * r3[i];
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s = s + wa[i] * binv[i] * mult[i];
    const double rmin = 1e-13 * sqrt(s / vol);
    if (tol < rmin) tol = rmin;
    double b1 = 0.0, b2 = 0.0;
    for (int64_t i = 0; i < n; ++i) {
      wa[i] = m1[i] + m2[i] + m3[i];
      b1 = b1 + wa[i] * mult[i];
      b2 = b2 + mult[i];
    }
    if (fabs(b1 - 3.0 * b2) < 0.1) {
      double o = 0.0;
      for (int64_t i = 0; i < n; ++i) o = o + (r1[i] + r2[i] + r3[i]) * mult[i];
      const double tolmin = fabs(o / 3.0) * 10.0;
      if (tol < tolmin) tol = tolmin;
    }
  }
  /* cggosf */
  int iters = -1;
  double rbnorm;
  {
    for (int64_t i = 0; i < n; ++i) wa[i] = r1[i] * r1[i] + r2[i] * r2[i] + r3[i] * r3[i];
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s = s + wa[i] * binv[i] * mult[i];
    rbnorm = sqrt(s / vol);
  }
  *rbn0 = rbnorm;
  if (rbnorm < tol * tol) {
    *rbn2 = rbnorm;
    free(buf);
    return 0;
  }
  ref_setprec(ops, dpc, h1, h2);
  for (int64_t i = 0; i < n; ++i) dpc[i] = (dpc[i] + dpc[i]) + dpc[i]; /* isd = 1, 2, 3 */
  for (int c = 0; c < 3; ++c)
    for (int64_t i = 0; i < n; ++i) {
      pp[c][i] = dpc[i] * r[c][i];
      p[c][i] = 0.0 + pp[c][i];
    }
  double rpp1 = sf_wdot(n, p[0], p[1], p[2], r1, r2, r3, mult);
  for (int iter = 1; iter <= 200; ++iter) {
    ref_axsf(ops, ap[0], ap[1], ap[2], p[0], p[1], p[2], h1, h2, rst, jac, bm1);
    for (int c = 0; c < 3; ++c) {
      for (int64_t i = 0; i < n; ++i) ap[c][i] = ap[c][i] * m[c][i]; /* rmask */
      ref_dssum(ops, ap[c]);                                            /* opdssum */
    }
    const double pap = sf_wdot(n, p[0], p[1], p[2], ap[0], ap[1], ap[2], mult);
    const double alpha = rpp1 / pap;
    for (int c = 0; c < 3; ++c)
      for (int64_t i = 0; i < n; ++i) {
        u[c][i] = u[c][i] + alpha * p[c][i];
        r[c][i] = r[c][i] + (-alpha) * ap[c][i];
      }
    for (int64_t i = 0; i < n; ++i) wa[i] = r1[i] * r1[i] + r2[i] * r2[i] + r3[i] * r3[i];
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s = s + wa[i] * binv[i] * mult[i];
    rbnorm = sqrt(s / vol);
    if (iter == 1) *rbn0 = rbnorm;
    if (rbnorm < tol) {
      iters = iter;
      break;
    }
    for (int c = 0; c < 3; ++c)
      for (int64_t i = 0; i < n; ++i) pp[c][i] = dpc[i] * r[c][i];
    for (int64_t i = 0; i < n; ++i) wa[i] = r1[i] * pp[0][i] + r2[i] * pp[1][i] + r3[i] * pp[2][i];
    const double rpp2 = rpp1;
    rpp1 = 0.0;
    for (int64_t i = 0; i < n; ++i) rpp1 = rpp1 + wa[i] * mult[i];
    const double beta = rpp1 / rpp2;
    for (int c = 0; c < 3; ++c)
      for (int64_t i = 0; i < n; ++i) p[c][i] = beta * p[c][i] + pp[c][i];
  }
  *rbn2 = rbnorm;
  free(buf);
  return iters;
}

/* crespsp (core/plan4.f:99-260), PN-PN without the stress formulation: the
 * face terms on the faces fbc marks (6 per element, preprocessor order: 0
 * none, 1 'V'/'v'/'MV'/'mv', 2 'shl', 3 'SYM'; fbc null: none); the pressure right-hand side
 * from the curl-curl of the extrapolated velocity, qtl, the pressure's own
 * operator, the forcing, and dtbd = bd(1)/dt; the mean removed when
 * null_space (ortho). */
/* The face term of crespsp (core/plan4.f:219-258) on face f (preprocessor
 * order 1..6) of element e: w = (b1 unx + b2 uny + b3 unz) area (times dtbd
 * for type 1) subtracted at the face points.  Normals and areas as area3 and
 * unitvec form them (core/coef.f:1354-1445): the cross product of the face's
 * tangent derivatives is the r-, s- or t-cofactor triple up to its sign
 * (outward: - on faces 1, 4, 5, + on 2, 3, 6), its length times the two
 * GLL weights is the area, the triple over its length the unit normal. */
static void face_term(int nx1, int64_t n, int64_t e, int f, int type, double *respr,
                      const double *b1, const double *b2, const double *b3, const double *rst,
                      const double *w, double dtbd) {
  const int N = nx1 - 1;
  const int64_t eo = e * (int64_t)nx1 * nx1 * nx1;
  const int d = (f == 2 || f == 4) ? 0 : (f == 1 || f == 3) ? 1 : 2; /* r, s, t */
  const double sg = (f == 1 || f == 4 || f == 5) ? -1.0 : 1.0;
  for (int b = 0; b < nx1; ++b)
    for (int a = 0; a < nx1; ++a) {
      int i, j, k;
      double wt;
      if (d == 0) { i = f == 2 ? N : 0; j = a; k = b; wt = w[a] * w[b]; }
      else if (d == 1) { i = a; j = f == 3 ? N : 0; k = b; wt = w[a] * w[b]; }
      else { i = a; j = b; k = f == 6 ? N : 0; wt = w[a] * w[b]; }
      const int64_t p = eo + i + nx1 * (j + nx1 * k);
      const double c1 = rst[(int64_t)(3 * d) * n + p], c2 = rst[(int64_t)(3 * d + 1) * n + p],
                   c3 = rst[(int64_t)(3 * d + 2) * n + p];
      const double len = sqrt(c1 * c1 + c2 * c2 + c3 * c3);
      double nx = sg * c1, ny = sg * c2, nz = sg * c3;
      if (len != 0.0) {
        nx = nx / len;
        ny = ny / len;
        nz = nz / len;
      }
      const double area = len * wt;
      double v = b1[p] * nx;      /* faccl3 */
      v = v + b2[p] * ny;         /* add2 */
      v = v + b3[p] * nz;
      v = v * area;               /* faccl2 */
      if (type == 1) v = v * dtbd; /* cmult */
      respr[p] = respr[p] - v;    /* sub2 */
    }
}

void ref_crespsp(const ref_ops *ops, double *respr, const double *vxe, const double *vye,
                 const double *vze, const double *pr, const double *qtl, const double *vdiff,
                 const double *vtrans, const double *bfx, const double *bfy, const double *bfz,
                 const double *bm1, const double *binv, double dtbd, int null_space,
                 const double *rst, const double *jac, const double *vx, const double *vy,
                 const double *vz, const int *fbc, const double *w) {
  const int nx1 = ref_ops_nx1(ops), nel = ref_ops_nel(ops);
  const int64_t n = ref_ops_n(ops);
  double *buf = (double *)malloc(sizeof(double) * 9 * n);
  double *ta[3] = {buf, buf + n, buf + 2 * n}, *wa[3] = {buf + 3 * n, buf + 4 * n, buf + 5 * n};
  double *w1 = buf + 6 * n, *w2 = buf + 7 * n, *w3 = buf + 8 * n;
  const double *bf[3] = {bfx, bfy, bfz};
  ref_op_curl(ops, ta[0], ta[1], ta[2], vxe, vye, vze, 1, rst, jac, bm1, binv);
  ref_op_curl(ops, wa[0], wa[1], wa[2], ta[0], ta[1], ta[2], 1, rst, jac, bm1, binv);
  for (int c = 0; c < 3; ++c)
    for (int64_t i = 0; i < n; ++i) wa[c][i] = wa[c][i] * bm1[i]; /* opcolv */
  ref_wgradm1(nx1, nel, ta[0], ta[1], ta[2], qtl, rst);            /* opgrad */
  const double scale = -4. / 3.;
  for (int c = 0; c < 3; ++c)
    for (int64_t i = 0; i < n; ++i) wa[c][i] = wa[c][i] + ta[c][i] * scale; /* opadd2cm */
  for (int64_t i = 0; i < n; ++i) w1[i] = vdiff[i] / vtrans[i];              /* invcol3 */
  for (int c = 0; c < 3; ++c)
    for (int64_t i = 0; i < n; ++i) wa[c][i] = wa[c][i] * w1[i];            /* opcolv */
  for (int64_t i = 0; i < n; ++i) {
    ta[0][i] = 1.0 / vtrans[i]; /* invers2 */
    ta[1][i] = 0.0;
  }
  ref_axhelm(ops, respr, pr, ta[0], ta[1]);
  for (int64_t i = 0; i < n; ++i) respr[i] = -respr[i]; /* chsign */
  for (int c = 0; c < 3; ++c)
    for (int64_t i = 0; i < n; ++i) ta[c][i] = bf[c][i] / vtrans[i] - wa[c][i];
  for (int c = 0; c < 3; ++c) {
    ref_dssum(ops, ta[c]); /* opdssum */
    for (int64_t i = 0; i < n; ++i) ta[c][i] = ta[c][i] * binv[i];
  }
  for (int c = 0; c < 3; ++c) ref_cdtp(nx1, nel, wa[c], ta[c], rst, jac, bm1, c + 1);
  for (int64_t i = 0; i < n; ++i) respr[i] = respr[i] + wa[0][i] + wa[1][i] + wa[2][i];
  for (int64_t i = 0; i < n; ++i) respr[i] = respr[i] + qtl[i] * bm1[i] * dtbd; /* admcol3 */
  if (fbc) /* face terms: velocity (types 1, 2) or symmetry (3) faces */
    for (int e = 0; e < nel; ++e)
      for (int f = 1; f <= 6; ++f) {
        const int t = fbc[6 * e + f - 1];
        if (t == 1 || t == 2) face_term(nx1, n, e, f, t, respr, vx, vy, vz, rst, w, dtbd);
        else if (t == 3) face_term(nx1, n, e, f, t, respr, ta[0], ta[1], ta[2], rst, w, dtbd);
      }
  if (null_space) { /* ortho: the mean over all points removed */
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s = s + respr[i];
    const double m = s / (double)n;
    for (int64_t i = 0; i < n; ++i) respr[i] = respr[i] - m;
  }
  (void)w2;
  (void)w3;
  free(buf);
}

/* conv1 (core/navier1.f:3276-3330): du = jacmi (vx (rx u_r + sx u_s + tx u_t)
 * + vy (ry u_r + ...) + vz (rz u_r + ...)), the convective term without
 * dealiasing (convop with ifdeal false, :3138) */
void ref_conv1(int nx1, int nel, double *du, const double *u, const double *vx, const double *vy,
               const double *vz, const double *rst, const double *jac) {
  const int nxyz = nx1 * nx1 * nx1;
  const int64_t n = (int64_t)nxyz * nel;
  double d[1024], dt[1024];
  double *ur = (double *)malloc(sizeof(double) * 3 * nxyz), *us = ur + nxyz, *ut = us + nxyz;
  dmat(nx1, d, dt, NULL);
  const double *rx = rst, *ry = rst + n, *rz = rst + 2 * n, *sx = rst + 3 * n, *sy = rst + 4 * n,
               *sz = rst + 5 * n, *tx = rst + 6 * n, *ty = rst + 7 * n, *tz = rst + 8 * n;
  for (int e = 0; e < nel; ++e) {
    const int64_t o = (int64_t)nxyz * e;
    ref_local_grad3(ur, us, ut, u + o, nx1 - 1, d, dt);
    for (int i = 0; i < nxyz; ++i) {
      const int64_t p = o + i;
      const double jacmi = 1.0 / jac[p];
      du[p] = jacmi * (vx[p] * (rx[p] * ur[i] + sx[p] * us[i] + tx[p] * ut[i]) +
                       vy[p] * (ry[p] * ur[i] + sy[p] * us[i] + ty[p] * ut[i]) +
                       vz[p] * (rz[p] * ur[i] + sz[p] * us[i] + tz[p] * ut[i]));
    }
  }
  free(ur);
}

/* advab (core/navier1.f:1516-1546): bf -= bm1 conv(v_c), per component */
void ref_advab(int nx1, int nel, double *bfx, double *bfy, double *bfz, const double *vx,
               const double *vy, const double *vz, const double *bm1, const double *rst,
               const double *jac) {
  const int64_t n = (int64_t)nx1 * nx1 * nx1 * nel;
  double *ta = (double *)malloc(sizeof(double) * n);
  double *bf[3] = {bfx, bfy, bfz};
  const double *v[3] = {vx, vy, vz};
  for (int c = 0; c < 3; ++c) {
    ref_conv1(nx1, nel, ta, v[c], vx, vy, vz, rst, jac);
    for (int64_t i = 0; i < n; ++i) bf[c][i] = bf[c][i] - bm1[i] * ta[i]; /* subcol3 */
  }
  free(ta);
}

/* ---- time-integration bookkeeping of the step (core/navier1.f, plan4.f) ---- */

/* makeabf (core/navier1.f:1597-1640, iflomach false), one component:
 * ta = ab1 abx1 + ab2 abx2; abx2 = abx1; abx1 = bf; bf = (ab0 bf + ta) vtrans */
void ref_makeabf(int64_t n, double *bf, double *abx1, double *abx2, const double *vtrans,
                 const double *ab) {
  for (int64_t i = 0; i < n; ++i) {
    const double ta = ab[1] * abx1[i] + ab[2] * abx2[i]; /* add3s2 */
    abx2[i] = abx1[i];
    abx1[i] = bf[i];
    bf[i] = ab[0] * bf[i] + ta; /* add2s1 */
    bf[i] = bf[i] * vtrans[i];  /* col2 */
  }
}

/* makebdf (core/navier1.f:1548-1595, fixed geometry, iflomach false), one
 * component: tb = v bm1 bd[1] + sum over lags l = 1..nbd-1 of vlag_l bm1
 * bd[l+1]; bf += tb (vtrans / dt).  vlag: nbd - 1 arrays of n. */
void ref_makebdf(int64_t n, double *bf, const double *v, const double *vlag, const double *bm1,
                 const double *vtrans, const double *bd, int nbd, double dt) {
  const double cnst = 1. / dt;
  for (int64_t i = 0; i < n; ++i) {
    const double h2 = vtrans[i] * cnst; /* cmult2 */
    double tb = v[i] * bm1[i] * bd[1]; /* opcolv3c */
    for (int l = 2; l <= nbd; ++l) tb = tb + vlag[(int64_t)(l - 2) * n + i] * bm1[i] * bd[l];
    bf[i] = bf[i] + tb * h2; /* opadd2col */
  }
}

/* sumab (core/plan4.f:525-540): v = ab0 vv + ab1 vvlag_1 (+ ab2 vvlag_2) */
void ref_sumab(int64_t n, double *v, const double *vv, const double *vvlag, const double *ab,
               int nab) {
  for (int64_t i = 0; i < n; ++i) {
    v[i] = ab[0] * vv[i] + ab[1] * vvlag[i]; /* add3s2 */
    if (nab == 3) v[i] = v[i] + ab[2] * vvlag[n + i]; /* add2s2 */
  }
}

/* ---- the dealiased convective term (core/convect.f) --------------------------- */

void ref_fd_weights(double xx, const double *x, int n, int m, double *c);

/* Gauss-Legendre points and weights (zwgl): roots of P_m by Newton from the
 * Chebyshev guesses, weights 2 / ((1 - x^2) P'_m(x)^2). */
static void gauss_points(int m, double *z, double *w) {
  for (int i = 0; i < m; ++i) {
    double x = -cos(3.14159265358979323846 * (i + 0.75) / (m + 0.5)), dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = x;
      for (int k = 1; k < m; ++k) {
        const double p2 = ((2 * k + 1) * x * p1 - k * p0) / (k + 1);
        p0 = p1;
        p1 = p2;
      }
      dp = m * (x * p1 - p0) / (x * x - 1.0);
      const double dx = p1 / dp;
      x -= dx;
      if (fabs(dx) < 1e-16) break;
    }
    z[i] = x;
    w[i] = 2.0 / ((1.0 - x * x) * dp * dp);
  }
}

/* v (nb^3) = [A (x) A (x) A] u (na^3), A nb x na column-major */
static void tensor3(double *v, int nb, const double *u, int na, const double *A, double *w1,
                    double *w2) {
  for (int k = 0; k < na; ++k) /* r */
    for (int j = 0; j < na; ++j)
      for (int i = 0; i < nb; ++i) {
        double s = 0.0;
        for (int l = 0; l < na; ++l) s += A[i + nb * l] * u[l + na * (j + na * k)];
        w1[i + nb * (j + na * k)] = s;
      }
  for (int k = 0; k < na; ++k) /* s */
    for (int j = 0; j < nb; ++j)
      for (int i = 0; i < nb; ++i) {
        double s = 0.0;
        for (int l = 0; l < na; ++l) s += A[j + nb * l] * w1[i + nb * (l + na * k)];
        w2[i + nb * (j + nb * k)] = s;
      }
  for (int k = 0; k < nb; ++k) /* t */
    for (int j = 0; j < nb; ++j)
      for (int i = 0; i < nb; ++i) {
        double s = 0.0;
        for (int l = 0; l < na; ++l) s += A[k + nb * l] * w2[i + nb * (j + nb * l)];
        v[i + nb * (j + nb * k)] = s;
      }
}

/* convop with dealiasing (param(99) = 4, core/navier1.f:3196-3204): conv =
 * convect_new(u; vx, vy, vz) / bm1 (core/convect.f:639-725, set_dealias_rx
 * core/convect2.f:120-175) on lxd Gauss points per direction. */
void ref_convect_new(int nx1, int nel, int lxd, double *conv, const double *u, const double *vx,
                     const double *vy, const double *vz, const double *rst, const double *bm1) {
  const int mx = nx1, md = lxd;
  const int64_t n1 = (int64_t)mx * mx * mx, nd = (int64_t)md * md * md, n = n1 * nel;
  double zg[32], wg[32], zd[32], wd[32], c[128];
  ref_zwgll(zg, wg, mx);
  gauss_points(md, zd, wd);
  double *J = (double *)malloc(sizeof(double) * md * mx), *Jt = (double *)malloc(sizeof(double) * md * mx);
  double *Dd = (double *)malloc(sizeof(double) * md * md);
  for (int i = 0; i < md; ++i) {
    ref_fd_weights(zd[i], zg, mx - 1, 0, c);
    for (int j = 0; j < mx; ++j) J[i + md * j] = c[j];
    ref_fd_weights(zd[i], zd, md - 1, 1, c);
    for (int j = 0; j < md; ++j) Dd[i + md * j] = c[j + md];
  }
  for (int i = 0; i < md; ++i)
    for (int j = 0; j < mx; ++j) Jt[j + mx * i] = J[i + md * j];
  double *buf = (double *)malloc(sizeof(double) * nd * 20);
  double *fx = buf, *fy = fx + nd, *fz = fy + nd, *uf = fz + nd, *ur = uf + nd, *us = ur + nd,
         *ut = us + nd, *w1 = ut + nd, *w2 = w1 + nd, *rxd = w2 + nd; /* rxd: 9 nd */
  double *out = rxd + 9 * nd;
  for (int e = 0; e < nel; ++e) {
    const int64_t o = n1 * e;
    for (int q = 0; q < 9; ++q) { /* set_dealias_rx */
      tensor3(rxd + q * nd, md, rst + (int64_t)q * n + o, mx, J, w1, w2);
      for (int k = 0; k < md; ++k)
        for (int j = 0; j < md; ++j)
          for (int i = 0; i < md; ++i)
            rxd[q * nd + i + md * (j + md * k)] *= wd[i] * wd[j] * wd[k];
    }
    tensor3(fx, md, vx + o, mx, J, w1, w2);
    tensor3(fy, md, vy + o, mx, J, w1, w2);
    tensor3(fz, md, vz + o, mx, J, w1, w2);
    tensor3(uf, md, u + o, mx, J, w1, w2);
    for (int k = 0; k < md; ++k) /* grad_rst on the Gauss grid */
      for (int j = 0; j < md; ++j)
        for (int i = 0; i < md; ++i) {
          double a = 0.0, b = 0.0, t = 0.0;
          for (int l = 0; l < md; ++l) {
            a += Dd[i + md * l] * uf[l + md * (j + md * k)];
            b += Dd[j + md * l] * uf[i + md * (l + md * k)];
            t += Dd[k + md * l] * uf[i + md * (j + md * l)];
          }
          const int64_t p = i + md * (j + md * k);
          ur[p] = a;
          us[p] = b;
          ut[p] = t;
        }
    for (int64_t p = 0; p < nd; ++p) {
      const double t1 = rxd[p] * fx[p] + rxd[nd + p] * fy[p] + rxd[2 * nd + p] * fz[p];
      const double t2 = rxd[3 * nd + p] * fx[p] + rxd[4 * nd + p] * fy[p] + rxd[5 * nd + p] * fz[p];
      const double t3 = rxd[6 * nd + p] * fx[p] + rxd[7 * nd + p] * fy[p] + rxd[8 * nd + p] * fz[p];
      uf[p] = t1 * ur[p] + t2 * us[p] + t3 * ut[p];
    }
    tensor3(out, mx, uf, md, Jt, w1, w2); /* project back: J^T */
    for (int64_t p = 0; p < n1; ++p) conv[o + p] = out[p] / bm1[o + p];
  }
  free(J);
  free(Jt);
  free(Dd);
  free(buf);
}

/* convop with the conservative form on the Gauss grid (param(99) = 5,
 * core/navier1.f:3205-3207 -> convect_cons, core/convect.f:729-800):
 * conv = J^T [sum_i (D_r (c_i u) rx_i + D_s (c_i u) sx_i + D_t (c_i u) tx_i)]
 * / bm1 with the Gauss-weighted fine metric terms. */
void ref_convect_cons(int nx1, int nel, int lxd, double *conv, const double *u,
                      const double *vx, const double *vy, const double *vz, const double *rst,
                      const double *bm1) {
  const int mx = nx1, md = lxd;
  const int64_t n1 = (int64_t)mx * mx * mx, nd = (int64_t)md * md * md, n = n1 * nel;
  double zg[32], wg[32], zd[32], wd[32], c[128];
  ref_zwgll(zg, wg, mx);
  gauss_points(md, zd, wd);
  double *J = (double *)malloc(sizeof(double) * md * mx), *Jt = (double *)malloc(sizeof(double) * md * mx);
  double *Dd = (double *)malloc(sizeof(double) * md * md);
  for (int i = 0; i < md; ++i) {
    ref_fd_weights(zd[i], zg, mx - 1, 0, c);
    for (int j = 0; j < mx; ++j) J[i + md * j] = c[j];
    ref_fd_weights(zd[i], zd, md - 1, 1, c);
    for (int j = 0; j < md; ++j) Dd[i + md * j] = c[j + md];
  }
  for (int i = 0; i < md; ++i)
    for (int j = 0; j < mx; ++j) Jt[j + mx * i] = J[i + md * j];
  double *buf = (double *)malloc(sizeof(double) * nd * 16);
  double *uf = buf, *cf = uf + nd, *cu = cf + nd, *w1 = cu + nd, *w2 = w1 + nd, *rxd = w2 + nd;
  double *out = rxd + 9 * nd;
  const double *cv[3] = {vx, vy, vz};
  for (int e = 0; e < nel; ++e) {
    const int64_t o = n1 * e;
    for (int q = 0; q < 9; ++q) {
      tensor3(rxd + q * nd, md, rst + (int64_t)q * n + o, mx, J, w1, w2);
      for (int k = 0; k < md; ++k)
        for (int j = 0; j < md; ++j)
          for (int i = 0; i < md; ++i)
            rxd[q * nd + i + md * (j + md * k)] *= wd[i] * wd[j] * wd[k];
    }
    tensor3(uf, md, u + o, mx, J, w1, w2);
    for (int64_t p = 0; p < nd; ++p) cu[p] = 0.0;
    for (int d = 0; d < 3; ++d) {
      tensor3(cf, md, cv[d] + o, mx, J, w1, w2);
      for (int64_t p = 0; p < nd; ++p) cf[p] = cf[p] * uf[p];
      for (int k = 0; k < md; ++k)
        for (int j = 0; j < md; ++j)
          for (int i = 0; i < md; ++i) {
            double a = 0.0, b = 0.0, t = 0.0;
            for (int l = 0; l < md; ++l) {
              a += Dd[i + md * l] * cf[l + md * (j + md * k)];
              b += Dd[j + md * l] * cf[i + md * (l + md * k)];
              t += Dd[k + md * l] * cf[i + md * (j + md * l)];
            }
            const int64_t p = i + md * (j + md * k);
            cu[p] = cu[p] + a * rxd[d * nd + p] + b * rxd[(d + 3) * nd + p] +
                    t * rxd[(d + 6) * nd + p];
          }
    }
    tensor3(out, mx, cu, md, Jt, w1, w2);
    for (int64_t p = 0; p < n1; ++p) conv[o + p] = out[p] / bm1[o + p];
  }
  free(J);
  free(Jt);
  free(Dd);
  free(buf);
}

/* conv2 (core/navier1.f:1288-1388, 3-D): dtfi = (D_r^T (w3 (rx vx + ry vy
 * + rz vz) fi) + D_s^T (...) + D_t^T (...)) / bm1, each col4 product
 * (m v) fi and the sums in the reference's order */
void ref_conv2(int nx1, int nel, double *dtfi, const double *fi, const double *vx,
               const double *vy, const double *vz, const double *rst, const double *bm1) {
  const int nxyz = nx1 * nx1 * nx1;
  const int64_t n = (int64_t)nxyz * nel;
  double d[1024], dt[1024];
  double *w3 = (double *)malloc(sizeof(double) * nxyz);
  double *ta = (double *)malloc(sizeof(double) * 4 * nxyz), *tb = ta + nxyz, *tc = tb + nxyz,
         *wk = tc + nxyz;
  dmat(nx1, d, dt, w3);
  for (int e = 0; e < nel; ++e) {
    const int64_t o = (int64_t)nxyz * e;
    double *t[3] = {ta, tb, tc};
    for (int q = 0; q < 3; ++q) { /* r, s, t */
      const double *mx = rst + (int64_t)(3 * q) * n, *my = rst + (int64_t)(3 * q + 1) * n,
                   *mz = rst + (int64_t)(3 * q + 2) * n;
      for (int i = 0; i < nxyz; ++i) {
        const int64_t p = o + i;
        double a = mx[p] * vx[p] * fi[p];
        a = a + my[p] * vy[p] * fi[p];
        a = a + mz[p] * vz[p] * fi[p];
        t[q][i] = a * w3[i];
      }
    }
    ref_local_grad3_t(dtfi + o, ta, tb, tc, nx1 - 1, d, dt, wk);
    for (int i = 0; i < nxyz; ++i) dtfi[o + i] = dtfi[o + i] / bm1[o + i];
  }
  free(w3);
  free(ta);
}

/* convopo with param(86) != 0 (core/navier1.f:1221-1286): the
 * skew-symmetric form, with cmask1 = 0 / cmask2 = 1 on the points of
 * outflow faces (cmask, :1390; ofc: 6 flags per element, preprocessor face
 * order) and 1 / 0 elsewhere. */
void ref_convopo(int nx1, int nel, double *conv, const double *fi, const double *vx,
                 const double *vy, const double *vz, const double *rst, const double *jac,
                 const double *bm1, const int *ofc) {
  const int nxyz = nx1 * nx1 * nx1, N = nx1 - 1;
  const int64_t n = (int64_t)nxyz * nel;
  double *c1 = (double *)malloc(sizeof(double) * 5 * n), *c2 = c1 + n, *mfi = c2 + n,
         *dm = mfi + n, *md = dm + n;
  for (int64_t i = 0; i < n; ++i) {
    c1[i] = 1.0;
    c2[i] = 0.0;
    conv[i] = 0.0;
  }
  for (int e = 0; e < nel; ++e)
    for (int f = 1; f <= 6; ++f) {
      if (!ofc[6 * e + f - 1]) continue;
      for (int k = 0; k < nx1; ++k)
        for (int j = 0; j < nx1; ++j)
          for (int i = 0; i < nx1; ++i) {
            const int on = (f == 1 && j == 0) || (f == 2 && i == N) || (f == 3 && j == N) ||
                           (f == 4 && i == 0) || (f == 5 && k == 0) || (f == 6 && k == N);
            if (!on) continue;
            const int64_t p = (int64_t)nxyz * e + i + nx1 * (j + nx1 * k);
            c1[p] = 0.0;
            c2[p] = 1.0;
          }
    }
  const double *v[3] = {vx, vy, vz};
  (void)v;
  for (int64_t i = 0; i < n; ++i) mfi[i] = fi[i] * c1[i];
  ref_conv1(nx1, nel, dm, mfi, vx, vy, vz, rst, jac);
  for (int64_t i = 0; i < n; ++i) {
    md[i] = dm[i] * c1[i];
    conv[i] = conv[i] + 0.5 * md[i];
    md[i] = dm[i] * c2[i];
    conv[i] = conv[i] + md[i];
  }
  ref_conv2(nx1, nel, dm, mfi, vx, vy, vz, rst, bm1);
  for (int64_t i = 0; i < n; ++i) {
    md[i] = dm[i] * c1[i];
    conv[i] = conv[i] + -0.5 * md[i];
  }
  for (int64_t i = 0; i < n; ++i) mfi[i] = fi[i] * c2[i];
  ref_conv1(nx1, nel, dm, mfi, vx, vy, vz, rst, jac);
  for (int64_t i = 0; i < n; ++i) {
    md[i] = dm[i] * c2[i];
    conv[i] = conv[i] + 0.5 * md[i];
  }
  ref_conv2(nx1, nel, dm, mfi, vx, vy, vz, rst, bm1);
  for (int64_t i = 0; i < n; ++i) {
    md[i] = dm[i] * c1[i];
    conv[i] = conv[i] + -1. * md[i];
    md[i] = dm[i] * c2[i];
    conv[i] = conv[i] + 0.5 * md[i];
  }
  free(c1);
}
