/*
 * nekref.c -- CPU oracle for the Nek5000 Helmholtz/Poisson solve path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker the parity tests compare the CUDA
 * library against, and the CPU baseline that bench.py times.  Parity
 * unpinned: no reference output exists to pin it (see nekref.h).  It is never
 * linked into, loaded by, or called from the product library.
 *
 * Each function restates one reference routine (file:line in the Nek5000
 * source tree) in the same loop order and the same left-to-right
 * accumulation order, in FP64, built with -ffp-contract=off.  The only
 * deliberate liberty is parallelism: with nthreads > 1, element loops run
 * under OpenMP (per-element work is independent, so results are unchanged),
 * and global sums are formed as per-thread partial sums over contiguous
 * element blocks, combined in thread order -- exactly what the reference does
 * on P MPI ranks with a contiguous element partition (local vlsc3/glsc3 sum,
 * then gop -> MPI_Allreduce, core/comm_mpi.f:216-259).  nthreads = 1 is the
 * serial single-rank reference order.
 */
#include "nekref.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

int ref_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* ========================================================================
 * Spectral library -- core/speclib.f
 * ====================================================================== */

/* GAMMAF (speclib.f:371-394): table lookup only, as in the reference. */
static double gammaf(double x) {
  const double pi = 4.0 * atan(1.0);
  double g = 1.0;
  if (x == -0.5) g = -2.0 * sqrt(pi);
  if (x == 0.5) g = sqrt(pi);
  if (x == 1.0) g = 1.0;
  if (x == 2.0) g = 1.0;
  if (x == 1.5) g = sqrt(pi) / 2.0;
  if (x == 2.5) g = 1.5 * sqrt(pi) / 2.0;
  if (x == 3.5) g = 0.5 * (2.5 * (1.5 * sqrt(pi)));
  if (x == 3.0) g = 2.0;
  if (x == 4.0) g = 6.0;
  if (x == 5.0) g = 24.0;
  if (x == 6.0) g = 120.0;
  return g;
}

/* PNORMJ (speclib.f:396-419) */
static double pnormj(int n, double alpha, double beta) {
  const double one = 1.0, two = 2.0;
  double dn = (double)n;
  double cnst = alpha + beta + one;
  double prod;
  if (n <= 1) {
    prod = gammaf(dn + alpha) * gammaf(dn + beta);
    prod = prod / (gammaf(dn) * gammaf(dn + alpha + beta));
    return prod * pow(two, cnst) / (two * dn + cnst);
  }
  prod = gammaf(alpha + one) * gammaf(beta + one);
  prod = prod / (two * (one + cnst) * gammaf(cnst + one));
  prod = prod * (one + alpha) * (two + alpha);
  prod = prod * (one + beta) * (two + beta);
  for (int i = 3; i <= n; ++i) {
    double dindx = (double)i;
    double frac = (dindx + alpha) * (dindx + beta) / (dindx * (dindx + alpha + beta));
    prod = prod * frac;
  }
  return prod * pow(two, cnst) / (two * dn + cnst);
}

/* JACOBF (speclib.f:479-518): Jacobi polynomial and derivative of degree n. */
static void jacobf(double *poly, double *pder, double *polym1, double *pderm1, double *polym2,
                   double *pderm2, int n, double alp, double bet, double x) {
  double apb = alp + bet;
  double p = 1.0, pd = 0.0;
  *poly = p;
  *pder = pd;
  if (n == 0) return;
  double polyl = p, pderl = pd;
  p = (alp - bet + (apb + 2.0) * x) / 2.0;
  pd = (apb + 2.0) / 2.0;
  *poly = p;
  *pder = pd;
  if (n == 1) return;
  double psave = 0.0, pdsave = 0.0;
  for (int k = 2; k <= n; ++k) {
    double dk = (double)k;
    double a1 = 2.0 * dk * (dk + apb) * (2.0 * dk + apb - 2.0);
    double a2 = (2.0 * dk + apb - 1.0) * (alp * alp - bet * bet);
    double b3 = (2.0 * dk + apb - 2.0);
    double a3 = b3 * (b3 + 1.0) * (b3 + 2.0);
    double a4 = 2.0 * (dk + alp - 1.0) * (dk + bet - 1.0) * (2.0 * dk + apb);
    double polyn = ((a2 + a3 * x) * p - a4 * polyl) / a1;
    double pdern = ((a2 + a3 * x) * pd - a4 * pderl + a3 * p) / a1;
    psave = polyl;
    pdsave = pderl;
    polyl = p;
    p = polyn;
    pderl = pd;
    pd = pdern;
  }
  *poly = p;
  *pder = pd;
  *polym1 = polyl;
  *pderm1 = pderl;
  *polym2 = psave;
  *pderm2 = pdsave;
}

/* JACG (speclib.f:421-477): Gauss points, Newton with deflation, then sort. */
static void jacg(double *xjac, int np, double alpha, double beta) {
  const int kstop = 10;
  const double eps = 1.0e-12;
  int n = np - 1;
  double one = 1.0;
  double dth = 4.0 * atan(one) / (2.0 * ((double)n) + 2.0);
  double xlast = 0.0;
  for (int j = 1; j <= np; ++j) {
    double x;
    if (j == 1) {
      x = cos((2.0 * (((double)j) - 1.0) + 1.0) * dth);
    } else {
      double x1 = cos((2.0 * (((double)j) - 1.0) + 1.0) * dth);
      double x2 = xlast;
      x = (x1 + x2) / 2.0;
    }
    for (int k = 1; k <= kstop; ++k) {
      double p, pd, pm1, pdm1, pm2, pdm2;
      jacobf(&p, &pd, &pm1, &pdm1, &pm2, &pdm2, np, alpha, beta, x);
      double recsum = 0.0;
      int jm = j - 1;
      for (int i = 1; i <= jm; ++i) recsum = recsum + 1.0 / (x - xjac[np - i]);
      double delx = -p / (pd - recsum * p);
      x = x + delx;
      if (fabs(delx) < eps) break;
    }
    xjac[np - j] = x;
    xlast = x;
  }
  for (int i = 1; i <= np; ++i) {
    double xmin = 2.0;
    int jmin = i;
    for (int j = i; j <= np; ++j) {
      if (xjac[j - 1] < xmin) {
        xmin = xjac[j - 1];
        jmin = j;
      }
    }
    if (jmin != i) {
      double swap = xjac[i - 1];
      xjac[i - 1] = xjac[jmin - 1];
      xjac[jmin - 1] = swap;
    }
  }
}

/* ZWGJD (speclib.f:155-206) */
static void zwgjd(double *z, double *w, int np, double alpha, double beta) {
  const double one = 1.0, two = 2.0;
  int n = np - 1;
  double apb = alpha + beta;
  if (np == 1) {
    z[0] = (beta - alpha) / (apb + two);
    w[0] = gammaf(alpha + one) * gammaf(beta + one) / gammaf(apb + two) * pow(two, apb + one);
    return;
  }
  jacg(z, np, alpha, beta);
  int np1 = n + 1, np2 = n + 2;
  double dnp1 = (double)np1, dnp2 = (double)np2;
  double fac1 = dnp1 + alpha + beta + one;
  double fac2 = fac1 + dnp1;
  double fac3 = fac2 + one;
  double fnorm = pnormj(np1, alpha, beta);
  double rcoef = (fnorm * fac2 * fac3) / (two * fac1 * dnp2);
  for (int i = 0; i < np; ++i) {
    double p, pd, pm1, pdm1, pm2, pdm2;
    jacobf(&p, &pd, &pm1, &pdm1, &pm2, &pdm2, np2, alpha, beta, z[i]);
    w[i] = -rcoef / (p * pdm1);
  }
}

/* ENDW1 / ENDW2 (speclib.f:278-370) */
static double endw(int n, double alpha, double beta, int which) {
  const double zero = 0.0, one = 1.0, two = 2.0, three = 3.0, four = 4.0;
  double apb = alpha + beta;
  if (n == 0) return zero;
  double f1, fint1, fint2, f2, f3 = 0.0;
  if (which == 1) {
    f1 = gammaf(alpha + two) * gammaf(beta + one) / gammaf(apb + three);
    f1 = f1 * (apb + two) * pow(two, apb + two) / two;
    if (n == 1) return f1;
    fint1 = gammaf(alpha + two) * gammaf(beta + one) / gammaf(apb + three);
    fint1 = fint1 * pow(two, apb + two);
    fint2 = gammaf(alpha + two) * gammaf(beta + two) / gammaf(apb + four);
    fint2 = fint2 * pow(two, apb + three);
    f2 = (-two * (beta + two) * fint1 + (apb + four) * fint2) * (apb + three) / four;
  } else {
    f1 = gammaf(alpha + one) * gammaf(beta + two) / gammaf(apb + three);
    f1 = f1 * (apb + two) * pow(two, apb + two) / two;
    if (n == 1) return f1;
    fint1 = gammaf(alpha + one) * gammaf(beta + two) / gammaf(apb + three);
    fint1 = fint1 * pow(two, apb + two);
    fint2 = gammaf(alpha + two) * gammaf(beta + two) / gammaf(apb + four);
    fint2 = fint2 * pow(two, apb + three);
    f2 = (two * (alpha + two) * fint1 - (apb + four) * fint2) * (apb + three) / four;
  }
  if (n == 2) return f2;
  for (int i = 3; i <= n; ++i) {
    double di = (double)(i - 1);
    double abn = alpha + beta + di;
    double abnn = abn + di;
    double a1 = -(two * (di + alpha) * (di + beta)) / (abn * abnn * (abnn + one));
    double a2 = (two * (alpha - beta)) / (abnn * (abnn + two));
    double a3 = (two * (abn + one)) / ((abnn + two) * (abnn + one));
    f3 = -(a2 * f2 + a1 * f1) / a3;
    f1 = f2;
    f2 = f3;
  }
  return f3;
}

/* ZWGLJD (speclib.f:238-276) */
static void zwgljd(double *z, double *w, int np, double alpha, double beta) {
  const double one = 1.0, two = 2.0;
  int n = np - 1, nm1 = n - 1;
  if (nm1 > 0) zwgjd(z + 1, w + 1, nm1, alpha + one, beta + one);
  z[0] = -one;
  z[np - 1] = one;
  for (int i = 2; i <= np - 1; ++i) w[i - 1] = w[i - 1] / (one - z[i - 1] * z[i - 1]);
  double p, pd, pm1, pdm1, pm2, pdm2;
  jacobf(&p, &pd, &pm1, &pdm1, &pm2, &pdm2, n, alpha, beta, z[0]);
  w[0] = endw(n, alpha, beta, 1) / (two * pd);
  jacobf(&p, &pd, &pm1, &pdm1, &pm2, &pdm2, n, alpha, beta, z[np - 1]);
  w[np - 1] = endw(n, alpha, beta, 2) / (two * pd);
}

/* ZWGLL (speclib.f:107-122) -> ZWGLJ (:207-236) -> ZWGLJD */
void ref_zwgll(double *z, double *w, int np) { zwgljd(z, w, np, 0.0, 0.0); }

/* PNLEG (speclib.f:875-905).  Like the Fortran, flushes |z| < 1e-25 to 0 in
 * the caller's storage. */
static double pnleg(double *z, int n) {
  if (fabs(*z) < 1.0e-25) *z = 0.0;
  double p1 = 1.0;
  if (n == 0) return p1;
  double p2 = *z, p3 = p2;
  for (int k = 1; k <= n - 1; ++k) {
    double fk = (double)k;
    p3 = ((2.0 * fk + 1.0) * (*z) * p2 - fk * p1) / (fk + 1.0);
    p1 = p2;
    p2 = p3;
  }
  return p3;
}

/* DGLL (speclib.f:811-838) */
void ref_dgll(double *d, double *dt, const double *zin, int nz) {
  double z[128];
  memcpy(z, zin, sizeof(double) * nz);
  int n = nz - 1;
  if (nz == 1) {
    d[0] = 0.0;
    return;
  }
  double fn = (double)n;
  double d0 = fn * (fn + 1.0) / 4.0;
  for (int i = 1; i <= nz; ++i) {
    for (int j = 1; j <= nz; ++j) {
      double v = 0.0;
      if (i != j) {
        double pi_ = pnleg(&z[i - 1], n);
        double pj_ = pnleg(&z[j - 1], n);
        v = pi_ / (pj_ * (z[i - 1] - z[j - 1]));
      }
      if (i == j && i == 1) v = -d0;
      if (i == j && i == nz) v = d0;
      d[(i - 1) + (j - 1) * nz] = v;
      dt[(j - 1) + (i - 1) * nz] = v;
    }
  }
}

/* ========================================================================
 * mxm (core/mxm_wrapper.f:1-87 -> mxm_std.f mxf<n2>): left-to-right sum
 * ====================================================================== */
void ref_mxm(const double *a, int n1, const double *b, int n2, double *c, int n3) {
  for (int j = 0; j < n3; ++j) {
    for (int i = 0; i < n1; ++i) {
      double s = a[i] * b[j * n2];
      for (int k = 1; k < n2; ++k) s = s + a[i + k * n1] * b[k + j * n2];
      c[i + j * n1] = s;
    }
  }
}

/* ========================================================================
 * Synthetic deformed box (harness input)
 * ====================================================================== */
void ref_box_mesh(int nx1, int kx, int ky, int kz, int periodic_y, int periodic_z, double amp,
                  const double *v3, double *xm1, double *ym1, double *zm1, int64_t *vertex) {
  double zg[128], wg[128];
  ref_zwgll(zg, wg, nx1);
  const double pi = 4.0 * atan(1.0);
  const int nxyz = nx1 * nx1 * nx1;
  const int64_t nvx = kx + 1;
  const int64_t nvy = periodic_y ? ky : ky + 1;
  const int64_t nvz = periodic_z ? kz : kz + 1;
  (void)nvz;
  const int nel = kx * ky * kz;
#pragma omp parallel for schedule(static)
  for (int e = 0; e < nel; ++e) {
    int ex = e % kx, ey = (e / kx) % ky, ez = e / (kx * ky);
    double xa = (double)ex / kx, xb = (double)(ex + 1) / kx;
    double ya = (double)ey / ky, yb = (double)(ey + 1) / ky;
    double za = (double)ez / kz, zb = (double)(ez + 1) / kz;
    for (int k = 0; k < 2; ++k)
      for (int j = 0; j < 2; ++j)
        for (int i = 0; i < 2; ++i) {
          int64_t vi = ex + i;
          int64_t vj = periodic_y ? (ey + j) % ky : ey + j;
          int64_t vk = periodic_z ? (ez + k) % kz : ez + k;
          vertex[8 * (int64_t)e + i + 2 * j + 4 * k] = 1 + vi + nvx * (vj + nvy * vk);
        }
    for (int iz = 0; iz < nx1; ++iz)
      for (int iy = 0; iy < nx1; ++iy)
        for (int ix = 0; ix < nx1; ++ix) {
          double hx1 = 0.5 * (1.0 + zg[ix]), hx0 = 0.5 * (1.0 - zg[ix]);
          double hy1 = 0.5 * (1.0 + zg[iy]), hy0 = 0.5 * (1.0 - zg[iy]);
          double hz1 = 0.5 * (1.0 + zg[iz]), hz0 = 0.5 * (1.0 - zg[iz]);
          double x = xa * hx0 + xb * hx1;
          double y = ya * hy0 + yb * hy1;
          double z = za * hz0 + zb * hz1;
          double s = amp * sin(pi * x) * sin(pi * y) * sin(pi * z);
          int64_t p = ix + nx1 * (iy + nx1 * iz) + (int64_t)nxyz * e;
          xm1[p] = x + s * v3[0];
          ym1[p] = y + s * v3[1];
          zm1[p] = z + s * v3[2];
        }
  }
}

/* ========================================================================
 * Geometry -- core/coef.f xyzrst (:879-926), glmapm1 (:555-631),
 * geodat1 (:633-784), genwz W3M1 (:263-267)
 * ====================================================================== */
static void geom_body(int nx1, int nel, const double *xm1, const double *ym1, const double *zm1,
                      double *g6, double *bm1, double *jacm1, double *rst);

void ref_geom(int nx1, int nel, const double *xm1, const double *ym1, const double *zm1,
              double *g6, double *bm1, double *jacm1) {
  geom_body(nx1, nel, xm1, ym1, zm1, g6, bm1, jacm1, NULL);
}

/* The same, with the metric terms rxm1..tzm1 (glmapm1's cofactors, nine
 * arrays of n in the order rx ry rz sx sy sz tx ty tz) and jacm1. */
void ref_geom_rst(int nx1, int nel, const double *xm1, const double *ym1, const double *zm1,
                  double *g6, double *bm1, double *jacm1, double *rst) {
  geom_body(nx1, nel, xm1, ym1, zm1, g6, bm1, jacm1, rst);
}

static void geom_body(int nx1, int nel, const double *xm1, const double *ym1, const double *zm1,
                      double *g6, double *bm1, double *jacm1, double *rst) {
  const int nxyz = nx1 * nx1 * nx1, nxy = nx1 * nx1;
  const int64_t n = (int64_t)nxyz * nel;
  double z[32], w[32], d[32 * 32], dt[32 * 32];
  ref_zwgll(z, w, nx1);
  ref_dgll(d, dt, z, nx1);
  double *w3 = (double *)malloc(sizeof(double) * nxyz);
  for (int iz = 0; iz < nx1; ++iz)
    for (int iy = 0; iy < nx1; ++iy)
      for (int ix = 0; ix < nx1; ++ix) w3[ix + nx1 * (iy + nx1 * iz)] = w[ix] * w[iy] * w[iz];
  double *g1 = g6, *g2 = g6 + n, *g3 = g6 + 2 * n, *g4 = g6 + 3 * n, *g5 = g6 + 4 * n,
         *g6_ = g6 + 5 * n;
#pragma omp parallel
  {
    double *buf = (double *)malloc(sizeof(double) * nxyz * 9);
    double *xr = buf, *yr = buf + nxyz, *zr = buf + 2 * nxyz, *xs = buf + 3 * nxyz,
           *ys = buf + 4 * nxyz, *zs = buf + 5 * nxyz, *xt = buf + 6 * nxyz, *yt = buf + 7 * nxyz,
           *zt = buf + 8 * nxyz;
#pragma omp for schedule(static)
    for (int e = 0; e < nel; ++e) {
      const int64_t o = (int64_t)nxyz * e;
      /* xyzrst */
      ref_mxm(d, nx1, xm1 + o, nx1, xr, nxy);
      ref_mxm(d, nx1, ym1 + o, nx1, yr, nxy);
      ref_mxm(d, nx1, zm1 + o, nx1, zr, nxy);
      for (int iz = 0; iz < nx1; ++iz) {
        ref_mxm(xm1 + o + iz * nxy, nx1, dt, nx1, xs + iz * nxy, nx1);
        ref_mxm(ym1 + o + iz * nxy, nx1, dt, nx1, ys + iz * nxy, nx1);
        ref_mxm(zm1 + o + iz * nxy, nx1, dt, nx1, zs + iz * nxy, nx1);
      }
      ref_mxm(xm1 + o, nxy, dt, nx1, xt, nx1);
      ref_mxm(ym1 + o, nxy, dt, nx1, yt, nx1);
      ref_mxm(zm1 + o, nxy, dt, nx1, zt, nx1);
      for (int i = 0; i < nxyz; ++i) {
        /* glmapm1: Jacobian by ADDCOL4/SUBCOL4, cofactors by ASCOL5 */
        double jac = 0.0;
        jac = jac + xr[i] * ys[i] * zt[i];
        jac = jac + xt[i] * yr[i] * zs[i];
        jac = jac + xs[i] * yt[i] * zr[i];
        jac = jac - xr[i] * yt[i] * zs[i];
        jac = jac - xs[i] * yr[i] * zt[i];
        jac = jac - xt[i] * ys[i] * zr[i];
        double rx = ys[i] * zt[i] - yt[i] * zs[i];
        double ry = xt[i] * zs[i] - xs[i] * zt[i];
        double rz = xs[i] * yt[i] - xt[i] * ys[i];
        double sx = yt[i] * zr[i] - yr[i] * zt[i];
        double sy = xr[i] * zt[i] - xt[i] * zr[i];
        double sz = xt[i] * yr[i] - xr[i] * yt[i];
        double tx = yr[i] * zs[i] - ys[i] * zr[i];
        double ty = xs[i] * zr[i] - xr[i] * zs[i];
        double tz = xr[i] * ys[i] - xs[i] * yr[i];
        /* geodat1: VDOT3, COL2 by WJ = 1/J, COL2 by W3M1; BM1 = J*W3M1 */
        double wj = 1.0 / jac;
        double a1 = rx * rx + ry * ry + rz * rz;
        double a2 = sx * sx + sy * sy + sz * sz;
        double a3 = tx * tx + ty * ty + tz * tz;
        double a4 = rx * sx + ry * sy + rz * sz;
        double a5 = rx * tx + ry * ty + rz * tz;
        double a6 = sx * tx + sy * ty + sz * tz;
        a1 = a1 * wj;
        a2 = a2 * wj;
        a3 = a3 * wj;
        a4 = a4 * wj;
        a5 = a5 * wj;
        a6 = a6 * wj;
        g1[o + i] = a1 * w3[i];
        g2[o + i] = a2 * w3[i];
        g3[o + i] = a3 * w3[i];
        g4[o + i] = a4 * w3[i];
        g5[o + i] = a5 * w3[i];
        g6_[o + i] = a6 * w3[i];
        bm1[o + i] = jac * w3[i];
        if (jacm1) jacm1[o + i] = jac;
        if (rst) {
          const double m9[9] = {rx, ry, rz, sx, sy, sz, tx, ty, tz};
          for (int q = 0; q < 9; ++q) rst[(int64_t)q * n + o + i] = m9[q];
        }
      }
    }
    free(buf);
  }
  free(w3);
}

/* ========================================================================
 * Global numbering -- core/navier8.f setvert3d (:2004-2360),
 * gbtuple_rank8 (:1934-2002) on one rank, i8rank_vecn (:1790-1830)
 * ====================================================================== */
typedef struct {
  int64_t k[3];
  int64_t pos;
} tup3;

static int nk_cmp;
static int cmp_tup(const void *a, const void *b) {
  const tup3 *x = (const tup3 *)a, *y = (const tup3 *)b;
  for (int i = 0; i < nk_cmp; ++i) {
    if (x->k[i] < y->k[i]) return -1;
    if (x->k[i] > y->k[i]) return 1;
  }
  return (x->pos < y->pos) ? -1 : (x->pos > y->pos);
}

/* rank (1-based) of each tuple among the sorted unique tuples */
static int64_t tuple_rank(tup3 *t, int64_t n, int nkey, int64_t *rank) {
  nk_cmp = nkey;
  qsort(t, n, sizeof(tup3), cmp_tup);
  int64_t nn = 0;
  for (int64_t i = 0; i < n; ++i) {
    int ne = (i == 0);
    if (i > 0)
      for (int q = 0; q < nkey; ++q)
        if (t[i].k[q] != t[i - 1].k[q]) ne = 1;
    if (ne) ++nn;
    rank[t[i].pos] = nn;
  }
  return nn;
}

static void sort4(int64_t *a) { /* ascending (i8sort of 4 corner ids) */
  for (int i = 1; i < 4; ++i) {
    int64_t v = a[i];
    int j = i - 1;
    while (j >= 0 && a[j] > v) {
      a[j + 1] = a[j];
      --j;
    }
    a[j + 1] = v;
  }
}

/* ICFACE (core/TOPOL:37-43), 3-D part, 0-based hypercube vertex index */
static const int icface[6][4] = {{0, 2, 4, 6}, {1, 3, 5, 7}, {0, 1, 4, 5},
                                 {2, 3, 6, 7}, {0, 1, 2, 3}, {4, 5, 6, 7}};

void ref_setvert3d(int64_t *glo_num, int64_t *ngv_out, int nx, int nel, const int64_t *vertex) {
  const int64_t nxyz = (int64_t)nx * nx * nx;
  /* glo_num(ile) uses 1-based ile; G(i) below is glo_num[i-1] */
#define G(ile) glo_num[(ile)-1]
  int64_t ngvv = 0;
  for (int64_t i = 0; i < 8 * (int64_t)nel; ++i)
    if (vertex[i] > ngvv) ngvv = vertex[i];
  for (int64_t i = 0; i < nxyz * nel; ++i) glo_num[i] = 0;
  for (int e = 0; e < nel; ++e)
    for (int k = 0; k < 2; ++k)
      for (int j = 0; j < 2; ++j)
        for (int i = 0; i < 2; ++i) {
          int64_t il = 1 + (int64_t)(nx - 1) * i + (int64_t)nx * (nx - 1) * j +
                       (int64_t)nx * nx * (nx - 1) * k;
          G(il + nxyz * e) = vertex[8 * (int64_t)e + i + 2 * j + 4 * k];
        }
  int64_t ngv = ngvv;
  if (nx == 2) {
    *ngv_out = ngv;
    return;
  }
  /* edges: pair index within the element = (r: j+2k), (s: 4+i+2k), (t: 8+i+2j) */
  const int64_t ne = 12 * (int64_t)nel;
  tup3 *et = (tup3 *)malloc(sizeof(tup3) * ne);
  int64_t *enm = (int64_t *)malloc(sizeof(int64_t) * ne);
  for (int e = 0; e < nel; ++e) {
    const int64_t *v = vertex + 8 * (int64_t)e;
    for (int c = 0; c < 4; ++c) {
      int64_t a0, a1;
      int b = c & 1, cc = c >> 1;
      /* r-edge (j=b,k=cc): endpoints vertex(0,j,k), vertex(1,j,k) */
      a0 = v[0 + 2 * b + 4 * cc];
      a1 = v[1 + 2 * b + 4 * cc];
      et[12 * (int64_t)e + c].k[0] = a0 < a1 ? a0 : a1;
      et[12 * (int64_t)e + c].k[1] = a0 < a1 ? a1 : a0;
      /* s-edge (i=b,k=cc) */
      a0 = v[b + 0 + 4 * cc];
      a1 = v[b + 2 + 4 * cc];
      et[12 * (int64_t)e + 4 + c].k[0] = a0 < a1 ? a0 : a1;
      et[12 * (int64_t)e + 4 + c].k[1] = a0 < a1 ? a1 : a0;
      /* t-edge (i=b,j=cc) */
      a0 = v[b + 2 * cc + 0];
      a1 = v[b + 2 * cc + 4];
      et[12 * (int64_t)e + 8 + c].k[0] = a0 < a1 ? a0 : a1;
      et[12 * (int64_t)e + 8 + c].k[1] = a0 < a1 ? a1 : a0;
    }
  }
  for (int64_t i = 0; i < ne; ++i) {
    et[i].k[2] = 0;
    et[i].pos = i;
  }
  int64_t n_unique_edges = tuple_rank(et, ne, 2, enm);
  free(et);
  const int64_t n_on_edge = nx - 2;
  const int64_t ngve = n_unique_edges * n_on_edge;
  for (int e = 0; e < nel; ++e) {
    int iedg = 0;
    const int64_t eo = nxyz * e;
    for (int k = 0; k < 2; ++k) /* edges 1-4 */
      for (int j = 0; j < 2; ++j) {
        int64_t igv = ngv + n_on_edge * (enm[12 * (int64_t)e + iedg] - 1);
        int64_t i0e = (int64_t)nx * (nx - 1) * j + (int64_t)nx * nx * (nx - 1) * k + eo;
        if (G(i0e + 1) < G(i0e + nx)) {
          for (int i = 2; i <= nx - 1; ++i) G(i0e + i) = igv + i - 1;
        } else {
          for (int i = 2; i <= nx - 1; ++i) G(i0e + i) = igv + 1 + n_on_edge - (i - 1);
        }
        ++iedg;
      }
    for (int k = 0; k < 2; ++k) /* edges 5-8 */
      for (int i = 0; i < 2; ++i) {
        int64_t igv = ngv + n_on_edge * (enm[12 * (int64_t)e + iedg] - 1);
        int64_t i0e = 1 + (int64_t)(nx - 1) * i + (int64_t)nx * nx * (nx - 1) * k + eo;
        if (G(i0e) < G(i0e + (int64_t)nx * (nx - 1))) {
          for (int j = 2; j <= nx - 1; ++j) G(i0e + (int64_t)(j - 1) * nx) = igv + j - 1;
        } else {
          for (int j = 2; j <= nx - 1; ++j)
            G(i0e + (int64_t)(j - 1) * nx) = igv + 1 + n_on_edge - (j - 1);
        }
        ++iedg;
      }
    for (int j = 0; j < 2; ++j) /* edges 9-12 */
      for (int i = 0; i < 2; ++i) {
        int64_t igv = ngv + n_on_edge * (enm[12 * (int64_t)e + iedg] - 1);
        int64_t i0e = 1 + (int64_t)(nx - 1) * i + (int64_t)nx * (nx - 1) * j + eo;
        if (G(i0e) < G(i0e + (int64_t)nx * nx * (nx - 1))) {
          for (int k = 2; k <= nx - 1; ++k) G(i0e + (int64_t)(k - 1) * nx * nx) = igv + k - 1;
        } else {
          for (int k = 2; k <= nx - 1; ++k)
            G(i0e + (int64_t)(k - 1) * nx * nx) = igv + 1 + n_on_edge - (k - 1);
        }
        ++iedg;
      }
  }
  free(enm);
  ngv = ngv + ngve;

  /* faces: the 3 smallest of the 4 corner ids, ranked */
  const int64_t nf = 6 * (int64_t)nel;
  tup3 *ft = (tup3 *)malloc(sizeof(tup3) * nf);
  int64_t *fnm = (int64_t *)malloc(sizeof(int64_t) * nf);
  for (int e = 0; e < nel; ++e)
    for (int f = 0; f < 6; ++f) {
      int64_t facet[4];
      for (int c = 0; c < 4; ++c) facet[c] = vertex[8 * (int64_t)e + icface[f][c]];
      sort4(facet);
      tup3 *t = &ft[6 * (int64_t)e + f];
      t->k[0] = facet[0];
      t->k[1] = facet[1];
      t->k[2] = facet[2];
      t->pos = 6 * (int64_t)e + f;
    }
  int64_t n_unique_faces = tuple_rank(ft, nf, 3, fnm);
  free(ft);
  /* SKPDAT (connect1.f:575-626) for nx=ny=nz */
  const int64_t NX = nx, NY = nx, NZ = nx;
  int64_t skp[6][6] = {
      {1, NX * (NY - 1) + 1, NX, 1, NY * (NZ - 1) + 1, NY},
      {1 + (NX - 1), NX * (NY - 1) + 1 + (NX - 1), NX, 1, NY * (NZ - 1) + 1, NY},
      {1, NX, 1, 1, NY * (NZ - 1) + 1, NY},
      {1 + NX * (NY - 1), NX + NX * (NY - 1), 1, 1, NY * (NZ - 1) + 1, NY},
      {1, NX, 1, 1, NY, 1},
      {1 + NX * NY * (NZ - 1), NX + NX * NY * (NZ - 1), 1, 1, NY, 1}};
  const int64_t n_on_face = (int64_t)(nx - 2) * (nx - 2);
  const int64_t nxx = (int64_t)nx * nx;
  for (int e = 0; e < nel; ++e)
    for (int f = 0; f < 6; ++f) {
      int64_t i0 = skp[f][0], i1 = skp[f][1], is = skp[f][2];
      int64_t j0 = skp[f][3], j1 = skp[f][4], js = skp[f][5];
      const int64_t eo = nxyz * e;
      int64_t gvf[4];
      gvf[0] = G(i0 + nx * (j0 - 1) + eo);
      gvf[1] = G(i1 + nx * (j0 - 1) + eo);
      gvf[2] = G(i0 + nx * (j1 - 1) + eo);
      gvf[3] = G(i1 + nx * (j1 - 1) + eo);
      int imin = 0;
      for (int q = 1; q < 4; ++q)
        if (gvf[q] < gvf[imin]) imin = q;
      int idir = 1, jdir = 1, ifij = 0;
      if (imin == 0) {
        idir = 1;
        jdir = 1;
        if (gvf[1] < gvf[2]) ifij = 1;
      } else if (imin == 1) {
        idir = -1;
        jdir = 1;
        if (gvf[0] < gvf[3]) ifij = 1;
      } else if (imin == 2) {
        idir = 1;
        jdir = -1;
        if (gvf[3] < gvf[0]) ifij = 1;
      } else {
        idir = -1;
        jdir = -1;
        if (gvf[2] < gvf[1]) ifij = 1;
      }
      if (idir < 0) {
        int64_t t = i0;
        i0 = i1;
        i1 = t;
        is = -is;
      }
      if (jdir < 0) {
        int64_t t = j0;
        j0 = j1;
        j1 = t;
        js = -js;
      }
      int64_t ig0 = ngv + n_on_face * (fnm[6 * (int64_t)e + f] - 1);
      int64_t k = 0, l = 0;
      int64_t ni = (i1 - i0 + is) / is, nj = (j1 - j0 + js) / js;
      if (ifij) {
        for (int64_t jj = 0; jj < nj; ++jj)
          for (int64_t ii = 0; ii < ni; ++ii) {
            int64_t i = i0 + ii * is, j = j0 + jj * js;
            ++k;
            if (k > nx && k < nxx - nx && k % nx != 1 && k % nx != 0) {
              ++l;
              G(i + nx * (j - 1) + eo) = l + ig0;
            }
          }
      } else {
        for (int64_t ii = 0; ii < ni; ++ii)
          for (int64_t jj = 0; jj < nj; ++jj) {
            int64_t i = i0 + ii * is, j = j0 + jj * js;
            ++k;
            if (k > nx && k < nxx - nx && k % nx != 1 && k % nx != 0) {
              ++l;
              G(i + nx * (j - 1) + eo) = l + ig0;
            }
          }
      }
    }
  free(fnm);
  ngv = ngv + n_unique_faces * n_on_face;
  /* interiors stay 0 (ifcenter = .false., dssum.f:16) */
  *ngv_out = ngv;
#undef G
}

/* ========================================================================
 * Gather-scatter -- gslib gs_setup / gs_op semantics as called from
 * core/dssum.f:20,79 (op table dssum.f:111-128): for every non-zero global
 * id shared by >= 2 local copies, combine the copies and write the result
 * back to each.  Combination order: ascending local index.
 * ====================================================================== */
struct ref_gs {
  int64_t nseg, nidx;
  int64_t *start; /* nseg+1 */
  int64_t *idx;   /* nidx, ascending within a segment */
  int64_t *id;    /* nseg, ascending */
};

typedef struct {
  int64_t id, i;
} idpair;
static int cmp_pair(const void *a, const void *b) {
  const idpair *x = (const idpair *)a, *y = (const idpair *)b;
  if (x->id != y->id) return x->id < y->id ? -1 : 1;
  return (x->i < y->i) ? -1 : (x->i > y->i);
}

ref_gs *ref_gs_setup(const int64_t *glo_num, int64_t n) {
  ref_gs *gs = (ref_gs *)calloc(1, sizeof(ref_gs));
  int64_t m = 0;
  for (int64_t i = 0; i < n; ++i) m += (glo_num[i] != 0);
  idpair *p = (idpair *)malloc(sizeof(idpair) * (m ? m : 1));
  m = 0;
  for (int64_t i = 0; i < n; ++i)
    if (glo_num[i] != 0) {
      p[m].id = glo_num[i];
      p[m].i = i;
      ++m;
    }
  qsort(p, m, sizeof(idpair), cmp_pair);
  int64_t nseg = 0, nidx = 0;
  for (int64_t a = 0; a < m;) {
    int64_t b = a + 1;
    while (b < m && p[b].id == p[a].id) ++b;
    if (b - a >= 2) {
      ++nseg;
      nidx += b - a;
    }
    a = b;
  }
  gs->nseg = nseg;
  gs->nidx = nidx;
  gs->start = (int64_t *)malloc(sizeof(int64_t) * (nseg + 1));
  gs->idx = (int64_t *)malloc(sizeof(int64_t) * (nidx ? nidx : 1));
  gs->id = (int64_t *)malloc(sizeof(int64_t) * (nseg ? nseg : 1));
  int64_t s = 0, q = 0;
  for (int64_t a = 0; a < m;) {
    int64_t b = a + 1;
    while (b < m && p[b].id == p[a].id) ++b;
    if (b - a >= 2) {
      gs->start[s] = q;
      gs->id[s] = p[a].id;
      for (int64_t c = a; c < b; ++c) gs->idx[q++] = p[c].i;
      ++s;
    }
    a = b;
  }
  gs->start[nseg] = q;
  free(p);
  return gs;
}

void ref_gs_free(ref_gs *gs) {
  if (!gs) return;
  free(gs->start);
  free(gs->idx);
  free(gs->id);
  free(gs);
}

int64_t ref_gs_nseg(const ref_gs *gs) { return gs->nseg; }
int64_t ref_gs_nidx(const ref_gs *gs) { return gs->nidx; }
void ref_gs_maps(const ref_gs *gs, int64_t *seg_start, int64_t *idx, int64_t *seg_id) {
  if (seg_start) memcpy(seg_start, gs->start, sizeof(int64_t) * (gs->nseg + 1));
  if (idx) memcpy(idx, gs->idx, sizeof(int64_t) * gs->nidx);
  if (seg_id) memcpy(seg_id, gs->id, sizeof(int64_t) * gs->nseg);
}

void ref_gs_op(const ref_gs *gs, double *u, int op) {
#pragma omp parallel for schedule(static)
  for (int64_t s = 0; s < gs->nseg; ++s) {
    int64_t a = gs->start[s], b = gs->start[s + 1];
    double t = u[gs->idx[a]];
    for (int64_t c = a + 1; c < b; ++c) {
      double v = u[gs->idx[c]];
      if (op == 0) t = t + v;
      else if (op == 1) t = t * v;
      else if (op == 2) t = (v > t) ? v : t;
      else t = (v < t) ? v : t;
    }
    for (int64_t c = a; c < b; ++c) u[gs->idx[c]] = t;
  }
}

/* ========================================================================
 * Operator state
 * ====================================================================== */
/* pointwise loops: independent per point, so threading leaves results unchanged */
#define PFOR _Pragma("omp parallel for schedule(static) num_threads(ops->nthreads)")

struct ref_ops {
  int nx1, nel, nthreads;
  int64_t n;
  const double *d, *dt, *g1, *g2, *g3, *g4, *g5, *g6, *bm1;
  ref_gs *gs;
  double vol;
};

const ref_gs *ref_ops_gs(const ref_ops *ops) { return ops->gs; }
int ref_ops_nx1(const ref_ops *ops) { return ops->nx1; }
int ref_ops_nel(const ref_ops *ops) { return ops->nel; }
int64_t ref_ops_n(const ref_ops *ops) { return ops->n; }

/* Global sum of a per-point expression, formed as contiguous element-block
 * partial sums in block order (the P-rank gop pattern).  EXPR(i) must be the
 * reference's per-point term; ACC is updated as ACC = ACC + term. */
#define GLOBAL_SUM(ops, result, TERM)                                              \
  do {                                                                             \
    int P_ = (ops)->nthreads;                                                      \
    if (P_ < 1) P_ = 1;                                                            \
    double part_[256];                                                             \
    if (P_ > 256) P_ = 256;                                                        \
    const int64_t nxyz_ = (int64_t)(ops)->nx1 * (ops)->nx1 * (ops)->nx1;           \
    _Pragma("omp parallel for num_threads(P_) schedule(static,1)")                 \
    for (int r_ = 0; r_ < P_; ++r_) {                                              \
      int64_t e0_ = (int64_t)(ops)->nel * r_ / P_, e1_ = (int64_t)(ops)->nel * (r_ + 1) / P_; \
      double acc_ = 0.0;                                                           \
      for (int64_t i = e0_ * nxyz_; i < e1_ * nxyz_; ++i) acc_ = acc_ + (TERM);    \
      part_[r_] = acc_;                                                            \
    }                                                                              \
    double tot_ = part_[0];                                                        \
    for (int r_ = 1; r_ < P_; ++r_) tot_ = tot_ + part_[r_];                       \
    (result) = tot_;                                                               \
  } while (0)

ref_ops *ref_ops_create(int nx1, int nel, const double *d, const double *dt, const double *g6,
                        const double *bm1, const int64_t *glo_num, int nthreads) {
  ref_ops *o = (ref_ops *)calloc(1, sizeof(ref_ops));
  o->nx1 = nx1;
  o->nel = nel;
  o->nthreads = nthreads < 1 ? 1 : nthreads;
  o->n = (int64_t)nx1 * nx1 * nx1 * nel;
  o->d = d;
  o->dt = dt;
  o->g1 = g6;
  o->g2 = g6 + o->n;
  o->g3 = g6 + 2 * o->n;
  o->g4 = g6 + 3 * o->n;
  o->g5 = g6 + 4 * o->n;
  o->g6 = g6 + 5 * o->n;
  o->bm1 = bm1;
  o->gs = ref_gs_setup(glo_num, o->n);
  double v;
  GLOBAL_SUM(o, v, bm1[i]); /* volvm1 = glsum(bm1), coef.f:1181 */
  o->vol = v;
  return o;
}

void ref_ops_free(ref_ops *o) {
  if (!o) return;
  ref_gs_free(o->gs);
  free(o);
}

void ref_dssum(const ref_ops *ops, double *u) { ref_gs_op(ops->gs, u, 0); }
void ref_dsop(const ref_ops *ops, double *u, int op) { ref_gs_op(ops->gs, u, op); }

double ref_glsc3(const ref_ops *ops, const double *a, const double *b, const double *m) {
  double s;
  GLOBAL_SUM(ops, s, a[i] * b[i] * m[i]); /* math.f:775-791 */
  return s;
}

/* ---- axhelm, 3-D deformed path (hmholtz.f:72-259; :191-217, :225) ------ */
void ref_axhelm(const ref_ops *ops, double *au, const double *u, const double *helm1,
                const double *helm2) {
  const int nx = ops->nx1, nxy = nx * nx, nyz = nx * nx, nxyz = nx * nx * nx;
  const int nel = ops->nel;
  const int64_t ntot = ops->n;
  const double *dxm1 = ops->d, *dxtm1 = ops->dt; /* dym1=dzm1=D, dytm1=dztm1=D^T */
#pragma omp parallel num_threads(ops->nthreads)
  {
    double *buf = (double *)malloc(sizeof(double) * nxyz * 6);
    double *dudr = buf, *duds = buf + nxyz, *dudt = buf + 2 * nxyz, *tmp1 = buf + 3 * nxyz,
           *tmp2 = buf + 4 * nxyz, *tmp3 = buf + 5 * nxyz;
    double *tm1 = dudr, *tm2 = duds, *tm3 = dudt; /* EQUIVALENCE (DUDR,TM1)... */
#pragma omp for schedule(static)
    for (int e = 0; e < nel; ++e) {
      const int64_t o = (int64_t)nxyz * e;
      const double *ue = u + o;
      ref_mxm(dxm1, nx, ue, nx, dudr, nyz);
      for (int iz = 0; iz < nx; ++iz) ref_mxm(ue + iz * nxy, nx, dxtm1, nx, duds + iz * nxy, nx);
      ref_mxm(ue, nxy, dxtm1, nx, dudt, nx);
      const double *g1 = ops->g1 + o, *g2 = ops->g2 + o, *g3 = ops->g3 + o, *g4 = ops->g4 + o,
                   *g5 = ops->g5 + o, *g6 = ops->g6 + o, *h1 = helm1 + o;
      for (int i = 0; i < nxyz; ++i) {
        double t1 = dudr[i] * g1[i];
        double t2 = duds[i] * g2[i];
        double t3 = dudt[i] * g3[i];
        t1 = t1 + duds[i] * g4[i];
        t1 = t1 + dudt[i] * g5[i];
        t2 = t2 + dudr[i] * g4[i];
        t2 = t2 + dudt[i] * g6[i];
        t3 = t3 + dudr[i] * g5[i];
        t3 = t3 + duds[i] * g6[i];
        tmp1[i] = t1 * h1[i];
        tmp2[i] = t2 * h1[i];
        tmp3[i] = t3 * h1[i];
      }
      ref_mxm(dxtm1, nx, tmp1, nx, tm1, nyz);
      for (int iz = 0; iz < nx; ++iz) ref_mxm(tmp2 + iz * nxy, nx, dxm1, nx, tm2 + iz * nxy, nx);
      ref_mxm(tmp3, nxy, dxm1, nx, tm3, nx);
      double *a = au + o;
      for (int i = 0; i < nxyz; ++i) {
        double s = 0.0;
        s = s + tm1[i];
        s = s + tm2[i];
        s = s + tm3[i];
        a[i] = s;
      }
    }
    free(buf);
  }
  /* ifh2 = vlamax(helm2) > 0 (setfast, hmholtz.f:302-304); addcol4 */
  double h2max = 0.0;
  for (int64_t i = 0; i < ntot; ++i) {
    double a = fabs(helm2[i]);
    if (a > h2max) h2max = a;
  }
  if (h2max > 0.0) {
#pragma omp parallel for num_threads(ops->nthreads) schedule(static)
    for (int64_t i = 0; i < ntot; ++i) au[i] = au[i] + helm2[i] * ops->bm1[i] * u[i];
  }
}

/* ---- setprec (hmholtz.f:380-524), 3-D deformed ------------------------- */
static void setprec_body(const ref_ops *ops, double *dpcm1, const double *helm1, const double *helm2,
                         int local) {
  const int nx = ops->nx1, nxyz = nx * nx * nx;
  const int64_t ntot = ops->n;
  const double *dxtm1 = ops->dt; /* dytm1 = dztm1 = dxtm1 */
#define DT(i, j) dxtm1[((i)-1) + ((j)-1) * nx]
#define IDX(ix, iy, iz) (((ix)-1) + nx * (((iy)-1) + nx * ((iz)-1)))
#pragma omp parallel for num_threads(ops->nthreads) schedule(static)
  for (int e = 0; e < ops->nel; ++e) {
    const int64_t o = (int64_t)nxyz * e;
    double *dp = dpcm1 + o;
    const double *g1 = ops->g1 + o, *g2 = ops->g2 + o, *g3 = ops->g3 + o, *g4 = ops->g4 + o,
                 *g5 = ops->g5 + o, *g6 = ops->g6 + o;
    for (int i = 0; i < nxyz; ++i) dp[i] = 0.0;
    for (int iq = 1; iq <= nx; ++iq)
      for (int iz = 1; iz <= nx; ++iz)
        for (int iy = 1; iy <= nx; ++iy)
          for (int ix = 1; ix <= nx; ++ix)
            dp[IDX(ix, iy, iz)] = dp[IDX(ix, iy, iz)] + g1[IDX(iq, iy, iz)] * (DT(ix, iq) * DT(ix, iq));
    for (int iq = 1; iq <= nx; ++iq)
      for (int iz = 1; iz <= nx; ++iz)
        for (int iy = 1; iy <= nx; ++iy)
          for (int ix = 1; ix <= nx; ++ix)
            dp[IDX(ix, iy, iz)] = dp[IDX(ix, iy, iz)] + g2[IDX(ix, iq, iz)] * (DT(iy, iq) * DT(iy, iq));
    for (int iq = 1; iq <= nx; ++iq)
      for (int iz = 1; iz <= nx; ++iz)
        for (int iy = 1; iy <= nx; ++iy)
          for (int ix = 1; ix <= nx; ++ix)
            dp[IDX(ix, iy, iz)] = dp[IDX(ix, iy, iz)] + g3[IDX(ix, iy, iq)] * (DT(iz, iq) * DT(iz, iq));
    /* cross terms on element-boundary index lines (deformed elements) */
    const int ends[2] = {1, nx};
    for (int a = 0; a < 2; ++a) /* DO 600 IY, IZ */
      for (int b = 0; b < 2; ++b) {
        int iy = ends[a], iz = ends[b];
        dp[IDX(1, iy, iz)] = dp[IDX(1, iy, iz)] + g4[IDX(1, iy, iz)] * DT(1, 1) * DT(iy, iy) +
                             g5[IDX(1, iy, iz)] * DT(1, 1) * DT(iz, iz);
        dp[IDX(nx, iy, iz)] = dp[IDX(nx, iy, iz)] + g4[IDX(nx, iy, iz)] * DT(nx, nx) * DT(iy, iy) +
                              g5[IDX(nx, iy, iz)] * DT(nx, nx) * DT(iz, iz);
      }
    for (int a = 0; a < 2; ++a) /* DO 700 IX, IZ */
      for (int b = 0; b < 2; ++b) {
        int ix = ends[a], iz = ends[b];
        dp[IDX(ix, 1, iz)] = dp[IDX(ix, 1, iz)] + g4[IDX(ix, 1, iz)] * DT(1, 1) * DT(ix, ix) +
                             g6[IDX(ix, 1, iz)] * DT(1, 1) * DT(iz, iz);
        dp[IDX(ix, nx, iz)] = dp[IDX(ix, nx, iz)] + g4[IDX(ix, nx, iz)] * DT(nx, nx) * DT(ix, ix) +
                              g6[IDX(ix, nx, iz)] * DT(nx, nx) * DT(iz, iz);
      }
    for (int a = 0; a < 2; ++a) /* DO 800 IX, IY */
      for (int b = 0; b < 2; ++b) {
        int ix = ends[a], iy = ends[b];
        dp[IDX(ix, iy, 1)] = dp[IDX(ix, iy, 1)] + g5[IDX(ix, iy, 1)] * DT(1, 1) * DT(ix, ix) +
                             g6[IDX(ix, iy, 1)] * DT(1, 1) * DT(iy, iy);
        dp[IDX(ix, iy, nx)] = dp[IDX(ix, iy, nx)] + g5[IDX(ix, iy, nx)] * DT(nx, nx) * DT(ix, ix) +
                              g6[IDX(ix, iy, nx)] * DT(nx, nx) * DT(iy, iy);
      }
  }
#undef DT
#undef IDX
  PFOR
  for (int64_t i = 0; i < ntot; ++i) dpcm1[i] = dpcm1[i] * helm1[i];                 /* COL2 */
  PFOR
  for (int64_t i = 0; i < ntot; ++i) dpcm1[i] = dpcm1[i] + helm2[i] * ops->bm1[i];  /* ADDCOL3 */
  if (local) return; /* the element-local diagonal alone */
  ref_dssum(ops, dpcm1);
  PFOR
  for (int64_t i = 0; i < ntot; ++i) dpcm1[i] = 1.0 / dpcm1[i];                     /* INVCOL1 */
}

void ref_setprec(const ref_ops *ops, double *dpcm1, const double *helm1, const double *helm2) {
  setprec_body(ops, dpcm1, helm1, helm2, 0);
}

/* setprec's element-local diagonal, before its dssum and reciprocal */
void ref_setprec_local(const ref_ops *ops, double *diag, const double *helm1,
                       const double *helm2) {
  setprec_body(ops, diag, helm1, helm2, 1);
}

/* ---- chktcg1 (hmholtz.f:527-609); EIGAA = 0 so ACONDNO = 10 ----------- */
void ref_chktcg1(const ref_ops *ops, double *tol, const double *res, const double *h1,
                 const double *h2, const double *mask, const double *mult, const double *binv) {
  const int64_t n = ops->n;
  double acondno = 10.0;
  double eps = 1.0e-13; /* FP64: 1+1e-9 != 1 */
  double vol = ops->vol;
  double *w1 = (double *)malloc(sizeof(double) * n);
  double *w2 = (double *)malloc(sizeof(double) * n);
  memcpy(w1, res, sizeof(double) * n);
  PFOR
  for (int64_t i = 0; i < n; ++i) w2[i] = binv[i] * w1[i];
  double rinit = sqrt(ref_glsc3(ops, w2, w1, mult) / vol);
  double rmin = eps * rinit;
  if (*tol < rmin) *tol = rmin;
  PFOR
  for (int64_t i = 0; i < n; ++i) w1[i] = 1.0;
  double bcneu1 = ref_glsc3(ops, w1, mask, mult);
  double bcneu2 = ref_glsc3(ops, w1, w1, mult);
  double bctest = fabs(bcneu1 - bcneu2);
  ref_axhelm(ops, w2, w1, h1, h2);
  PFOR
  for (int64_t i = 0; i < n; ++i) w2[i] = w2[i] * w2[i];
  PFOR
  for (int64_t i = 0; i < n; ++i) w2[i] = w2[i] * ops->bm1[i];
  double s;
  GLOBAL_SUM(ops, s, w2[i]);
  double bcrob = sqrt(s / vol);
  if (bctest < 0.1 && bcrob < eps * acondno) {
    double tolmin = rinit * eps * 10.0;
    if (*tol < tolmin) *tol = tolmin;
  }
  free(w1);
  free(w2);
}

/* ---- cggo (hmholtz.f:611-846), Jacobi preconditioner path -------------- */
int ref_cggo(const ref_ops *ops, double *x, const double *f, const double *h1, const double *h2,
             const double *mask, const double *mult, double tin, int maxit, int maxcg, int istep,
             const double *binv, double *rbn0_out, double *rbn2_out) {
  const int64_t n = ops->n;
  const int P = ops->nthreads;
  double vol = ops->vol;
  double tol = fabs(tin);
  int niter = maxit < maxcg ? maxit : maxcg;
  double *d = (double *)malloc(sizeof(double) * n);
  double *r = (double *)malloc(sizeof(double) * n);
  double *w = (double *)malloc(sizeof(double) * n);
  double *p = (double *)malloc(sizeof(double) * n);
  double *z = (double *)malloc(sizeof(double) * n);
  ref_setprec(ops, d, h1, h2);
  memcpy(r, f, sizeof(double) * n);
  PFOR
  for (int64_t i = 0; i < n; ++i) x[i] = 0.0;
  PFOR
  for (int64_t i = 0; i < n; ++i) p[i] = 0.0;
  double rbn0 = 0.0, rbn2 = 0.0;
  double fmax = 0.0;
  for (int64_t i = 0; i < n; ++i) fmax = fmax > fabs(f[i]) ? fmax : fabs(f[i]);
  if (fmax == 0.0) {
    *rbn0_out = 0.0;
    *rbn2_out = 0.0;
    free(d); free(r); free(w); free(p); free(z);
    return 0;
  }
  /* non-trivial null space: no Dirichlet point and h2 == 0 */
  double h2max = -99.0e20, skmin = 99.0e20;
  for (int64_t i = 0; i < n; ++i) {
    if (h2[i] > h2max) h2max = h2[i];
    if (mask[i] < skmin) skmin = mask[i];
  }
  int ifmcor = (skmin > 0.0 && h2max == 0.0);
  double smean = 0.0;
  if (ifmcor) {
    double sb, sr;
    GLOBAL_SUM(ops, sb, ops->bm1[i]);
    smean = -1.0 / sb;
    GLOBAL_SUM(ops, sr, r[i] * mult[i]);
    double rmean = smean * sr;
    memcpy(x, ops->bm1, sizeof(double) * n);
    ref_dssum(ops, x);
    PFOR
    for (int64_t i = 0; i < n; ++i) r[i] = r[i] + rmean * x[i];
    PFOR
    for (int64_t i = 0; i < n; ++i) x[i] = 0.0;
  }
  double rtz1 = 1.0, rtz2, rho = 0.0;
  int iter;
  (void)P;
  for (iter = 1; iter <= niter; ++iter) {
    PFOR
    for (int64_t i = 0; i < n; ++i) z[i] = r[i] * d[i]; /* col3 */
    if (ifmcor) {
      double sz;
      GLOBAL_SUM(ops, sz, z[i] * ops->bm1[i]);
      double rmean = smean * sz;
      PFOR
      for (int64_t i = 0; i < n; ++i) z[i] = z[i] + rmean;
    }
    rtz2 = rtz1;
    double s1, s2;
    GLOBAL_SUM(ops, s1, z[i] * r[i] * mult[i]);          /* vlsc3 */
    GLOBAL_SUM(ops, s2, mult[i] * binv[i] * r[i] * r[i]); /* vlsc32 */
    rtz1 = s1;
    rbn2 = sqrt(s2 / vol);
    if (iter == 1) rbn0 = rbn2;
    if (tin < 0) tol = fabs(tin) * rbn0;
    if (rbn2 <= tol && (iter > 1 || istep <= 5)) {
      niter = iter - 1;
      goto done;
    }
    double beta = rtz1 / rtz2;
    if (iter == 1) beta = 0.0;
    PFOR
    for (int64_t i = 0; i < n; ++i) p[i] = beta * p[i] + z[i]; /* add2s1 */
    ref_axhelm(ops, w, p, h1, h2);
    ref_dssum(ops, w);
    PFOR
    for (int64_t i = 0; i < n; ++i) w[i] = w[i] * mask[i];
    rho = ref_glsc3(ops, w, p, mult);
    double alpha = rtz1 / rho;
    double alphm = -alpha;
    PFOR
    for (int64_t i = 0; i < n; ++i) x[i] = x[i] + alpha * p[i]; /* add2s2 */
    PFOR
    for (int64_t i = 0; i < n; ++i) r[i] = r[i] + alphm * w[i];
  }
  niter = iter - 1;
done:
  *rbn0_out = rbn0;
  *rbn2_out = rbn2;
  free(d); free(r); free(w); free(p); free(z);
  return niter;
}

/* ---- hmholtz (hmholtz.f:2-69) ------------------------------------------ */
int ref_hmholtz(const ref_ops *ops, double *u, double *rhs, const double *h1, const double *h2,
                const double *mask, const double *mult, double tli, int maxit, int maxcg,
                int istep, const double *binv, double *rbn0, double *rbn2) {
  const int64_t n = ops->n;
  double tol = fabs(tli);
  ref_dssum(ops, rhs);
  PFOR
  for (int64_t i = 0; i < n; ++i) rhs[i] = rhs[i] * mask[i];
  ref_chktcg1(ops, &tol, rhs, h1, h2, mask, mult, binv);
  if (tli < 0) tol = tli;
  return ref_cggo(ops, u, rhs, h1, h2, mask, mult, tol, maxit, maxcg, istep, binv, rbn0, rbn2);
}

/* ---- local_grad3 (navier5.f:428-445) / local_grad3_t (navier1.f:4669-4692) */
void ref_local_grad3(double *ur, double *us, double *ut, const double *u, int N, const double *d,
                     const double *dt) {
  int m1 = N + 1, m2 = m1 * m1;
  ref_mxm(d, m1, u, m1, ur, m2);
  for (int k = 0; k <= N; ++k) ref_mxm(u + k * m2, m1, dt, m1, us + k * m2, m1);
  ref_mxm(u, m2, dt, m1, ut, m1);
}

void ref_local_grad3_t(double *u, const double *ur, const double *us, const double *ut, int N,
                       const double *d, const double *dt, double *w) {
  int m1 = N + 1, m2 = m1 * m1, m3 = m2 * m1;
  ref_mxm(dt, m1, ur, m1, u, m2);
  for (int k = 0; k <= N; ++k) ref_mxm(us + k * m2, m1, d, m1, w + k * m2, m1);
  for (int i = 0; i < m3; ++i) u[i] = u[i] + w[i];
  ref_mxm(ut, m2, d, m1, w, m1);
  for (int i = 0; i < m3; ++i) u[i] = u[i] + w[i];
}

/* ======================================================================== */
/* Residual projection onto previous solutions (navier4.f:562-1188).        */
/* ======================================================================== */
struct ref_proj {
  int mmx, m;
  int64_t n;
  double *xx, *bb;           /* X(n,mmx), B(n,mmx) = A*X                      */
  double *xbar, *bbar;       /* best fit in X and A*xbar                      */
  double *h1old, *h2old;     /* h1 / h2 the basis was built with (zero-filled) */
};

ref_proj *ref_proj_create(const ref_ops *ops, int mmx) {
  ref_proj *p = (ref_proj *)calloc(1, sizeof(ref_proj));
  const int64_t n = ops->n;
  p->mmx = mmx;
  p->n = n;
  p->xx = (double *)calloc((size_t)n * mmx, sizeof(double));
  p->bb = (double *)calloc((size_t)n * mmx, sizeof(double));
  p->xbar = (double *)calloc(n, sizeof(double));
  p->bbar = (double *)calloc(n, sizeof(double));
  p->h1old = (double *)calloc(n, sizeof(double));
  p->h2old = (double *)calloc(n, sizeof(double));
  return p;
}

void ref_proj_free(ref_proj *p) {
  if (!p) return;
  free(p->xx); free(p->bb); free(p->xbar); free(p->bbar); free(p->h1old); free(p->h2old);
  free(p);
}

int ref_proj_m(const ref_proj *p) { return p->m; }
const double *ref_proj_x(const ref_proj *p, int k) { return p->xx + (size_t)k * p->n; }
const double *ref_proj_b(const ref_proj *p, int k) { return p->bb + (size_t)k * p->n; }

/* proj_matvec (navier4.f:827): b = mask * dssum(A x), imsh = 1, isd = 1 */
static void proj_matvec(const ref_ops *ops, double *b, const double *x, const double *h1,
                        const double *h2, const double *msk) {
  const int64_t n = ops->n;
  ref_axhelm(ops, b, x, h1, h2);
  ref_dssum(ops, b);
  PFOR
  for (int64_t i = 0; i < n; ++i) b[i] = b[i] * msk[i];
}

/* vlsc3 summed over ranks (gop): sum x*w*y */
static double gdot3(const ref_ops *ops, const double *x, const double *w, const double *y) {
  double s;
  GLOBAL_SUM(ops, s, x[i] * w[i] * y[i]);
  return s;
}

/* 0.5*(vlsc3(a,w,b) + vlsc3(c,w,d)) per rank, then gop over ranks
 * (proj_ortho :865-876, proj_ortho_full_cgs2 :1078-1086) */
static double gdot3_sym(const ref_ops *ops, const double *a, const double *w, const double *b,
                        const double *c, const double *d) {
  int P_ = ops->nthreads < 1 ? 1 : ops->nthreads;
  if (P_ > 256) P_ = 256;
  double part_[256];
  const int64_t nxyz_ = (int64_t)ops->nx1 * ops->nx1 * ops->nx1;
  _Pragma("omp parallel for num_threads(P_) schedule(static,1)")
  for (int r_ = 0; r_ < P_; ++r_) {
    int64_t e0_ = (int64_t)ops->nel * r_ / P_, e1_ = (int64_t)ops->nel * (r_ + 1) / P_;
    double s1 = 0.0, s2 = 0.0;
    for (int64_t i = e0_ * nxyz_; i < e1_ * nxyz_; ++i) s1 = s1 + a[i] * w[i] * b[i];
    for (int64_t i = e0_ * nxyz_; i < e1_ * nxyz_; ++i) s2 = s2 + c[i] * w[i] * d[i];
    part_[r_] = 0.5 * (s1 + s2);
  }
  double tot_ = part_[0];
  for (int r_ = 1; r_ < P_; ++r_) tot_ = tot_ + part_[r_];
  return tot_;
}

/* add2s2 (math.f:689): a = a + c1*b */
static void add2s2(const ref_ops *ops, double *a, const double *b, double c1) {
  const int64_t n = ops->n;
  PFOR
  for (int64_t i = 0; i < n; ++i) a[i] = a[i] + c1 * b[i];
}

static void cmult(const ref_ops *ops, double *a, double c) {
  const int64_t n = ops->n;
  PFOR
  for (int64_t i = 0; i < n; ++i) a[i] = a[i] * c;
}

/* hypot (navier4.f:1330-1342, Nek's own, not libm's) */
static double nek_hypot(double a, double b) {
  double c = fabs(a), d = fabs(b);
  double x = c > d ? c : d;
  double ix = 1.0 / x;
  double t = c < d ? c : d;
  t = ix * t;
  return x * sqrt(1.0 + t * t);
}

/* givens_rotation (navier4.f:1308) */
static void givens_rotation(double a, double b, double *c, double *s, double *r) {
  if (b != 0.0) {
    double h = nek_hypot(a, b);
    double d = 1.0 / h;
    *c = fabs(a) * d;
    *s = copysign(d, a) * b;
    *r = copysign(1.0, a) * h;
  } else {
    *c = 1.0;
    *s = 0.0;
    *r = a;
  }
}

/* proj_ortho_full_cgs2 (navier4.f:1060-1127) */
static void proj_ortho_full_cgs2(const ref_ops *ops, ref_proj *p, const double *w) {
  const int64_t n = ops->n;
  int m = p->m;
  if (m <= 0) return;
  double tol = 1.0e-7;
  double alpha[64];
  int flag[64];
  for (int it = 0; it < 2; ++it) {
    for (int k = m; k >= 1; --k) {
      double *xk = p->xx + (size_t)(k - 1) * n, *bk = p->bb + (size_t)(k - 1) * n;
      for (int j = m; j >= k; --j) {
        const double *xj = p->xx + (size_t)(j - 1) * n, *bj = p->bb + (size_t)(j - 1) * n;
        alpha[j - 1] = gdot3_sym(ops, xj, w, bk, bj, xk);
      }
      for (int j = m; j >= k + 1; --j) {
        add2s2(ops, xk, p->xx + (size_t)(j - 1) * n, -alpha[j - 1]);
        add2s2(ops, bk, p->bb + (size_t)(j - 1) * n, -alpha[j - 1]);
      }
      double normp = sqrt(alpha[k - 1]);
      double normk = sqrt(gdot3(ops, xk, w, bk));
      if (normk > tol * normp) {
        double scl1 = 1.0 / normk;
        cmult(ops, xk, scl1);
        cmult(ops, bk, scl1);
        flag[k - 1] = 1;
      } else {
        flag[k - 1] = 0;
      }
    }
  }
  int k = 0;
  for (int j = 1; j <= m; ++j) {
    if (flag[j - 1] == 1) {
      k = k + 1;
      if (k < j) {
        memcpy(p->xx + (size_t)(k - 1) * n, p->xx + (size_t)(j - 1) * n, sizeof(double) * n);
        memcpy(p->bb + (size_t)(k - 1) * n, p->bb + (size_t)(j - 1) * n, sizeof(double) * n);
      }
    }
  }
  p->m = k;
}

/* project1 (navier4.f:636-733) + project1_a (:735-825); b <- b - B*alpha */
static void project1(const ref_ops *ops, ref_proj *p, double *b, const double *h1,
                     const double *h2, const double *msk, const double *w) {
  const int64_t n = ops->n;
  int m = p->m;
  if (m <= 0) return;
  /* iproj_chk (:788-820): matrix changed if h1/h2 differ from the old ones */
  double dh1 = 0.0, dh2 = 0.0;
  for (int64_t i = 0; i < n; ++i) {
    double a1 = fabs(h1[i] - p->h1old[i]), a2 = fabs(h2[i] - p->h2old[i]);
    dh1 = dh1 > a1 ? dh1 : a1;
    dh2 = dh2 > a2 ? dh2 : a2;
  }
  double dh = dh1 > dh2 ? dh1 : dh2;
  if (dh > 0.0) {
    memcpy(p->h1old, h1, sizeof(double) * n);
    memcpy(p->h2old, h2, sizeof(double) * n);
    for (int j = 0; j < m; ++j)
      proj_matvec(ops, p->bb + (size_t)j * n, p->xx + (size_t)j * n, h1, h2, msk);
    proj_ortho_full_cgs2(ops, p, w);
    m = p->m;
  }
  double alpha[64];
  /* first round of CGS */
  for (int k = 0; k < m; ++k) alpha[k] = gdot3(ops, p->xx + (size_t)k * n, w, b);
  PFOR
  for (int64_t i = 0; i < n; ++i) p->xbar[i] = alpha[0] * p->xx[i]; /* cmult2 */
  PFOR
  for (int64_t i = 0; i < n; ++i) p->bbar[i] = alpha[0] * p->bb[i];
  add2s2(ops, b, p->bb, -alpha[0]);
  for (int k = 1; k < m; ++k) {
    add2s2(ops, p->xbar, p->xx + (size_t)k * n, alpha[k]);
    add2s2(ops, p->bbar, p->bb + (size_t)k * n, alpha[k]);
    add2s2(ops, b, p->bb + (size_t)k * n, -alpha[k]);
  }
  /* second round */
  for (int k = 0; k < m; ++k) alpha[k] = gdot3(ops, p->xx + (size_t)k * n, w, b);
  for (int k = 0; k < m; ++k) {
    add2s2(ops, p->xbar, p->xx + (size_t)k * n, alpha[k]);
    add2s2(ops, p->bbar, p->bb + (size_t)k * n, alpha[k]);
    add2s2(ops, b, p->bb + (size_t)k * n, -alpha[k]);
  }
}

/* proj_ortho (navier4.f:852-957): O(nm) update after appending x_m, b_m */
static void proj_ortho(const ref_ops *ops, ref_proj *p, const double *w) {
  const int64_t n = ops->n;
  int m = p->m;
  if (m <= 0) return;
  double alpha[64], beta[64];
  double *xm = p->xx + (size_t)(m - 1) * n, *bm = p->bb + (size_t)(m - 1) * n;
  for (int k = 0; k < m; ++k) {
    const double *xk = p->xx + (size_t)k * n, *bk = p->bb + (size_t)k * n;
    alpha[k] = gdot3_sym(ops, xk, w, bm, bk, xm);
  }
  double nrm = sqrt(alpha[m - 1]);
  for (int k = 0; k < m - 1; ++k) {
    add2s2(ops, xm, p->xx + (size_t)k * n, -alpha[k]);
    add2s2(ops, bm, p->bb + (size_t)k * n, -alpha[k]);
  }
  for (int k = 0; k < m - 1; ++k) {
    const double *xk = p->xx + (size_t)k * n, *bk = p->bb + (size_t)k * n;
    beta[k] = gdot3_sym(ops, xk, w, bm, bk, xm);
  }
  for (int k = 0; k < m - 1; ++k) {
    add2s2(ops, xm, p->xx + (size_t)k * n, -beta[k]);
    add2s2(ops, bm, p->bb + (size_t)k * n, -beta[k]);
    alpha[k] = alpha[k] + beta[k];
  }
  alpha[m - 1] = sqrt(gdot3(ops, xm, w, bm));
  double tol = 1.0e-7;
  if (alpha[m - 1] > tol * nrm) {
    double scl1 = 1.0 / alpha[m - 1];
    cmult(ops, xm, scl1);
    cmult(ops, bm, scl1);
    for (int k = m; k >= 2; --k) {
      int h = k - 1;
      double c, s;
      givens_rotation(alpha[h - 1], alpha[k - 1], &c, &s, &nrm);
      alpha[h - 1] = nrm;
      double *xh = p->xx + (size_t)(h - 1) * n, *xk = p->xx + (size_t)(k - 1) * n;
      double *bh = p->bb + (size_t)(h - 1) * n, *bk = p->bb + (size_t)(k - 1) * n;
      PFOR
      for (int64_t i = 0; i < n; ++i) {
        double scl1_ = c * xh[i] + s * xk[i];
        xk[i] = -s * xh[i] + c * xk[i];
        xh[i] = scl1_;
        double scl2_ = c * bh[i] + s * bk[i];
        bk[i] = -s * bh[i] + c * bk[i];
        bh[i] = scl2_;
      }
    }
  } else {
    p->m = m - 1;
  }
}

/* project2 (navier4.f:1129-1154) + project2_a (:1156-1187) */
static void project2(const ref_ops *ops, ref_proj *p, double *x, const double *h1,
                     const double *h2, const double *msk, const double *w) {
  const int64_t n = ops->n;
  if (p->m > 0) {
    PFOR
    for (int64_t i = 0; i < n; ++i) x[i] = x[i] + p->xbar[i]; /* add2 */
  }
  p->m = p->m + 1 < p->mmx ? p->m + 1 : p->mmx;
  double *xm = p->xx + (size_t)(p->m - 1) * n, *bm = p->bb + (size_t)(p->m - 1) * n;
  memcpy(xm, x, sizeof(double) * n);
  proj_matvec(ops, bm, xm, h1, h2, msk);
  proj_ortho(ops, p, w);
}

/* hsolve with projection (navier4.f:562-634, the ifstdh = .false. branch) and
 * hmhzpf (:513-560, param(22) = 0, not 'PRES'): r <- dssum(r*vmk), project,
 * chktcg1 + cggo, un-project and update the space. */
int ref_hsolve(const ref_ops *ops, ref_proj *p, double *u, double *r, const double *h1,
               const double *h2, const double *vmk, const double *vml, double tli, int maxit,
               int maxcg, int istep, const double *binv, double *rbn0, double *rbn2) {
  const int64_t n = ops->n;
  PFOR
  for (int64_t i = 0; i < n; ++i) r[i] = r[i] * vmk[i]; /* col2 */
  ref_dssum(ops, r);
  project1(ops, p, r, h1, h2, vmk, vml);
  double tol = tli;
  ref_chktcg1(ops, &tol, r, h1, h2, vmk, vml, binv);
  int niter = ref_cggo(ops, u, r, h1, h2, vmk, vml, tol, maxit, maxcg, istep, binv, rbn0, rbn2);
  project2(ops, p, u, h1, h2, vmk, vml);
  return niter;
}

/* ========================================================================
 * hmh_gmres -- core/gmres.f:304-560 (see nekref.h), preconditioner M = diag
 * ====================================================================== */
static void gm_ax(const ref_ops *ops, double *w, const double *x, const double *h1,
                  const double *h2, const double *mask) {
  ref_axhelm(ops, w, x, h1, h2); /* ax, gmres.f:284-302 */
  ref_dssum(ops, w);
  for (int64_t i = 0; i < ops->n; ++i) w[i] = w[i] * mask[i];
}

static void gm_ortho(const ref_ops *ops, double *z, int null_space) {
  if (!null_space) return;
  double sum; /* glsum / ntotg, cadd (navier1.f:242-245) */
  GLOBAL_SUM(ops, sum, z[i]);
  const double rlam = sum / (double)ops->n;
  for (int64_t i = 0; i < ops->n; ++i) z[i] = z[i] + (-rlam);
}

static int gmres_body(const ref_ops *ops, const ref_h1mg *mg, double *res, const double *h1,
                      const double *h2, const double *wt, const double *mask, double tol,
                      int maxit, int m, int null_space, double *div0_out, double *rnorm_out) {
  const int64_t n = ops->n;
  if (m < 1) m = 1;
  double *d = (double *)malloc(sizeof(double) * n);
  double *r = (double *)malloc(sizeof(double) * n);
  double *w = (double *)malloc(sizeof(double) * n);
  double *x = (double *)calloc((size_t)n, sizeof(double));
  double *V = (double *)malloc(sizeof(double) * n * m);
  double *Z = (double *)malloc(sizeof(double) * n * m);
  double *H = (double *)calloc((size_t)(m + 1) * (m + 1), sizeof(double)); /* H[i + (m+1) j] */
  double *c = (double *)calloc((size_t)m + 1, sizeof(double));
  double *sn = (double *)calloc((size_t)m + 1, sizeof(double));
  double *gam = (double *)calloc((size_t)m + 2, sizeof(double));
  ref_setprec(ops, d, h1, h2);
  const double norm_fac = 1.0 / sqrt(ops->vol);
  double tolpss = fabs(tol), div0 = 0.0, rnorm = 0.0;
  int iter = 0, iconv = 0;
#define HM(i, j) H[(i) + (size_t)(m + 1) * (j)]
  while (!iconv) {
    if (iter == 0) {
      for (int64_t i = 0; i < n; ++i) r[i] = 1.0 * res[i]; /* col3(r, ml, res) */
    } else {
      gm_ax(ops, w, x, h1, h2, mask);
      for (int64_t i = 0; i < n; ++i) r[i] = res[i] + (-1.0) * w[i]; /* add2s2(r, w, -1) */
    }
    gam[0] = sqrt(ref_glsc3(ops, r, r, wt));
    if (iter == 0) {
      div0 = gam[0] * norm_fac;
      if (tol < 0) tolpss = fabs(tol) * div0;
    }
    rnorm = 0.0;
    if (gam[0] == 0.0) break; /* lucky convergence */
    double temp = 1.0 / gam[0];
    for (int64_t i = 0; i < n; ++i) V[i] = r[i] * temp;
    int j;
    int restart = 0;
    for (j = 0; j < m; ++j) {
      ++iter;
      double *zj = Z + (size_t)n * j, *vj = V + (size_t)n * j;
      if (mg) { /* h1mg_solve(z_j, w = mu v_j); w is masked in place, then overwritten */
        for (int64_t i = 0; i < n; ++i) w[i] = 1.0 * vj[i];
        ref_h1mg_solve(mg, zj, w);
      } else {
        for (int64_t i = 0; i < n; ++i) zj[i] = d[i] * (1.0 * vj[i]); /* M (mu v_j) */
      }
      gm_ortho(ops, zj, null_space);
      gm_ax(ops, w, zj, h1, h2, mask);
      for (int iv = 0; iv <= j; ++iv) { /* h_ij = vlsc3(w, v_i, wt) */
        const double *vi = V + (size_t)n * iv;
        double hs;
        GLOBAL_SUM(ops, hs, w[i] * vi[i] * wt[i]);
        HM(iv, j) = hs;
      }
      for (int i = 0; i <= j; ++i) {
        const double *vi = V + (size_t)n * i;
        const double a = -HM(i, j);
        for (int64_t q = 0; q < n; ++q) w[q] = w[q] + a * vi[q];
      }
      for (int i = 0; i < j; ++i) { /* Givens rotations on the new column */
        const double t = HM(i, j);
        HM(i, j) = c[i] * t + sn[i] * HM(i + 1, j);
        HM(i + 1, j) = -sn[i] * t + c[i] * HM(i + 1, j);
      }
      const double alpha = sqrt(ref_glsc3(ops, w, w, wt));
      rnorm = 0.0;
      if (alpha == 0.0) {
        iconv = 1;
        break;
      }
      const double l = sqrt(HM(j, j) * HM(j, j) + alpha * alpha);
      temp = 1.0 / l;
      c[j] = HM(j, j) * temp;
      sn[j] = alpha * temp;
      HM(j, j) = l;
      gam[j + 1] = -sn[j] * gam[j];
      gam[j] = c[j] * gam[j];
      rnorm = fabs(gam[j + 1]) * norm_fac;
      if (iter + 1 > maxit || rnorm < tolpss) {
        iconv = 1;
        break;
      }
      if (j == m - 1) {
        restart = 1;
        break;
      }
      temp = 1.0 / alpha;
      double *vn = V + (size_t)n * (j + 1);
      for (int64_t i = 0; i < n; ++i) vn[i] = w[i] * temp;
    }
    (void)restart;
    /* back substitution c = H^-1 gamma, then x += sum c_i z_i */
    const int jj = j < m ? j : m - 1;
    for (int k = jj; k >= 0; --k) {
      double t = gam[k];
      for (int i = jj; i > k; --i) t = t - HM(k, i) * c[i];
      c[k] = t / HM(k, k);
    }
    for (int i = 0; i <= jj; ++i) {
      const double *zi = Z + (size_t)n * i;
      for (int64_t q = 0; q < n; ++q) x[q] = x[q] + c[i] * zi[q];
    }
  }
#undef HM
  for (int64_t i = 0; i < n; ++i) res[i] = x[i];
  gm_ortho(ops, res, null_space);
  if (div0_out) *div0_out = div0;
  if (rnorm_out) *rnorm_out = rnorm;
  free(d);
  free(r);
  free(w);
  free(x);
  free(V);
  free(Z);
  free(H);
  free(c);
  free(sn);
  free(gam);
  return iter;
}

int ref_gmres(const ref_ops *ops, double *res, const double *h1, const double *h2,
              const double *wt, const double *mask, double tol, int maxit, int m, int null_space,
              double *div0_out, double *rnorm_out) {
  return gmres_body(ops, NULL, res, h1, h2, wt, mask, tol, maxit, m, null_space, div0_out,
                    rnorm_out);
}

int ref_gmres_h1mg(const ref_ops *ops, const ref_h1mg *mg, double *res, const double *h1,
                   const double *h2, const double *wt, const double *mask, double tol, int maxit,
                   int m, int null_space, double *div0_out, double *rnorm_out) {
  return gmres_body(ops, mg, res, h1, h2, wt, mask, tol, maxit, m, null_space, div0_out,
                    rnorm_out);
}

/* ========================================================================
 * hmh_flex_cg -- core/hmholtz.f:2164-2289 (see nekref.h), M = diag
 * ====================================================================== */
static int flex_body(const ref_ops *ops, const ref_h1mg *mg, double *res, const double *h1,
                     const double *h2, const double *wt, const double *mask, double tol,
                     int maxit, int null_space, double *div0_out, double *rnorm_out) {
  const int64_t n = ops->n;
  double *d = (double *)malloc(sizeof(double) * n);
  double *r = (double *)malloc(sizeof(double) * n);
  double *r1 = (double *)calloc((size_t)n, sizeof(double));
  double *p = (double *)calloc((size_t)n, sizeof(double));
  double *z = (double *)malloc(sizeof(double) * n);
  double *w = (double *)malloc(sizeof(double) * n);
  ref_setprec(ops, d, h1, h2);
  for (int64_t i = 0; i < n; ++i) {
    r[i] = res[i];
    res[i] = 0.0;
  }
  double rho1 = 1.0, t;
  GLOBAL_SUM(ops, t, r[i] * wt[i] * r[i]); /* glsc3(r, wt, r) */
  const double div0 = sqrt(t / ops->vol);
  const double tolpss = tol < 0 ? fabs(tol) * div0 : fabs(tol);
  double rnorm = div0;
  int iter = 0;
  /* a zero right-hand side is solved by x = 0 after no iteration (the
     reference's loop would form 0/0 there) */
  for (int k = 1; k <= maxit && div0 != 0.0; ++k) {
    if (mg) /* h1mg_solve(z, r): r is masked in place */
      ref_h1mg_solve(mg, z, r);
    else
      for (int64_t i = 0; i < n; ++i) z[i] = d[i] * r[i]; /* z = M r */
    for (int64_t i = 0; i < n; ++i) r1[i] = r1[i] - r[i]; /* sub2 */
    const double rho0 = rho1;
    GLOBAL_SUM(ops, rho1, z[i] * wt[i] * r[i]);
    double rho2;
    GLOBAL_SUM(ops, rho2, z[i] * wt[i] * r1[i]);
    rho2 = -rho2;
    const double beta = rho2 / rho0;
    for (int64_t i = 0; i < n; ++i) r1[i] = r[i];
    for (int64_t i = 0; i < n; ++i) p[i] = beta * p[i] + z[i]; /* add2s1 */
    gm_ax(ops, w, p, h1, h2, mask);
    double den;
    GLOBAL_SUM(ops, den, w[i] * wt[i] * p[i]);
    const double alpha = rho1 / den;
    for (int64_t i = 0; i < n; ++i) {
      res[i] = res[i] + alpha * p[i];
      r[i] = r[i] - alpha * w[i];
    }
    double rn;
    GLOBAL_SUM(ops, rn, r[i] * r[i] * wt[i]);
    rnorm = sqrt(rn / ops->vol);
    ++iter;
    if (rnorm < tolpss) break;
  }
  gm_ortho(ops, res, null_space);
  if (div0_out) *div0_out = div0;
  if (rnorm_out) *rnorm_out = rnorm;
  free(d);
  free(r);
  free(r1);
  free(p);
  free(z);
  free(w);
  return iter;
}

int ref_flex_cg(const ref_ops *ops, double *res, const double *h1, const double *h2,
                const double *wt, const double *mask, double tol, int maxit, int null_space,
                double *div0_out, double *rnorm_out) {
  return flex_body(ops, NULL, res, h1, h2, wt, mask, tol, maxit, null_space, div0_out, rnorm_out);
}

int ref_flex_cg_h1mg(const ref_ops *ops, const ref_h1mg *mg, double *res, const double *h1,
                     const double *h2, const double *wt, const double *mask, double tol,
                     int maxit, int null_space, double *div0_out, double *rnorm_out) {
  return flex_body(ops, mg, res, h1, h2, wt, mask, tol, maxit, null_space, div0_out, rnorm_out);
}
