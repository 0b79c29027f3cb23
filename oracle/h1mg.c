/*
 * h1mg.c -- CPU restatement of the pressure solve's preconditioner (TEST
 * INFRASTRUCTURE ONLY: the oracle the device path is checked against; never
 * linked into the product).
 *
 * h1mg_solve (core/hsmg.f:1855-1949) with if_hybrid = .false., the setting
 * hmh_gmres and hmh_flex_cg use (core/gmres.f:332, core/hmholtz.f:2194): an
 * additive multilevel Schwarz method.  Levels (h1mg_setup_mg_nx :2272-2338)
 * are polynomial orders 1, min(3, ...) and N; on every level above the
 * coarsest, overlapping Schwarz with fast-diagonalisation local solves on
 * elements extended by one layer of the neighbours' points
 * (h1mg_schwarz_part1 :440-494, hsmg_do_fast :897-930); restriction by J^T
 * with 1/multiplicity weights (h1mg_rstr :2216-2232); the coarsest level
 * (trilinear, one unknown per vertex) solved exactly with the Galerkin matrix
 * b_i^T A_e b_j of the fine operator (get_local_crs_galerkin,
 * core/navier8.f:1648-1687; crs_setup / crs_solve, core/crs_xxt.c:863-975);
 * corrections interpolated up (hsmg_intp :205-212) and averaged (dsavg,
 * core/ic.f:1871).
 *
 * Where this differs from the reference:
 *   - the 1-D generalised eigenproblems (generalev, core/hmholtz.f:1369,
 *     LAPACK dsygv) are solved here by cyclic Jacobi rotations on
 *     B^-1/2 A B^-1/2 (B is diagonal); S diag(1/lambda) S^T is the same
 *     operator to rounding, but not bit for bit;
 *   - the coarse system is factored densely (Cholesky) instead of by XXT's
 *     nested-dissection X X^T.  On one rank XXT solves the same system; with
 *     a null space it pins the last local unknown and removes the mean
 *     (crs_xxt.c:940-957); here the pinned unknown is the one with the
 *     largest vertex id, which is XXT's last local unknown when its local
 *     order is by id (not checked against the reference: parity unpinned).
 * Face types (get_fast_bc, core/fast3d.f:802-870) are given per element in
 * the order r-, r+, s-, s+, t-, t+: 0 = shared with a neighbour (also
 * periodic), 1 = Dirichlet ('O', outflow), 2 = Neumann (wall, inflow).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "nekref.h"

void ref_zwgll(double *z, double *w, int np);
void ref_mxm(const double *a, int n1, const double *b, int n2, double *c, int n3);

#define MGMAX 4

typedef struct {
  int nx;                /* points per direction: order + 1 */
  int64_t n;             /* nx^3 nel */
  ref_gs *gs, *gse;      /* level and extended ((nx+2)^3) numberings */
  double *mask;          /* 0 on Dirichlet points, else 1 */
  double *rwt;           /* restriction weights: 1/multiplicity */
  double *swt;           /* Schwarz weights (levels above the coarsest) */
  double *S;             /* per element, direction: S then S^T, nl x nl each */
  double *dinv;          /* per element: nl^3 inverse eigenvalue sums */
  double z[16], w[16];   /* GLL points and weights */
  double ah[256];        /* 1-D stiffness (semhat a) */
  double jh[256], jht[256]; /* interpolation from the next coarser level */
} mglev;

struct ref_h1mg {
  const ref_ops *ops;
  int nel, lmax, null_space;
  mglev lev[MGMAX];      /* lev[0] = level 1 (order 1) */
  int64_t nc;            /* coarse unknowns */
  int64_t *cid;          /* per level-1 point: coarse unknown or -1 */
  double *L;             /* Cholesky factor of the coarse matrix, nc x nc */
  int64_t nsolve;        /* unknowns in the factor (nc, or nc - 1 pinned) */
  double *vmult;         /* fine 1/multiplicity (dsavg) */
  double *ext0, *ext1, *ext2; /* scratch: extended arrays (finest) */
  double *len;           /* per element: left r s t, middle r s t, right r s t */
};

/* ---- Fornberg weights ---------------------------------------------------- */
/* c[j + (n+1) k]: the weight of x[j] in the k-th derivative at xx, k <= m,
 * from the n+1 nodes x[0..n] (B. Fornberg, "Calculation of weights in finite
 * difference formulas", SIAM Review 40 (1998) 685-691), the recursion
 * fd_weights_full (core/fast3d.f:1294) evaluates. */
void ref_fd_weights(double xx, const double *x, int n, int m, double *c) {
  const int ld = n + 1;
  for (int k = 0; k <= m; ++k)
    for (int j = 0; j <= n; ++j) c[j + ld * k] = 0.0;
  double c1 = 1.0, c4 = x[0] - xx;
  c[0] = 1.0;
  for (int i = 1; i <= n; ++i) {
    const int mn = i < m ? i : m;
    double c2 = 1.0;
    const double c5 = c4;
    c4 = x[i] - xx;
    for (int j = 0; j < i; ++j) {
      const double c3 = x[i] - x[j];
      c2 = c2 * c3;
      if (j == i - 1) {
        for (int k = mn; k >= 1; --k)
          c[i + ld * k] = c1 * ((double)k * c[i - 1 + ld * (k - 1)] - c5 * c[i - 1 + ld * k]) / c2;
        c[i] = -c1 * c5 * c[i - 1] / c2;
      }
      for (int k = mn; k >= 1; --k)
        c[j + ld * k] = (c4 * c[j + ld * k] - (double)k * c[j + ld * (k - 1)]) / c3;
      c[j] = c4 * c[j] / c3;
    }
    c1 = c2;
  }
}

/* ---- level orders (h1mg_setup_mg_nx, 3-D) -------------------------------- */
int ref_h1mg_levels(int lx1, int *order) {
  static const int mgn2[10] = {1, 2, 2, 2, 2, 3, 3, 5, 5, 5};
  int lmax = lx1 == 4 ? 2 : 3;
  int mglx2 = 2 * (lx1 / 4) + 1; /* lx2 = lx1 on the PN-PN pressure */
  if (lx1 == 5) mglx2 = 3;
  if (lx1 <= 10) mglx2 = mgn2[(lx1 < 10 ? lx1 : 10) - 1];
  if (lx1 == 8) mglx2 = 3;
  if (mglx2 > 3) mglx2 = 3;
  order[0] = 1;
  order[1] = mglx2;
  order[2] = mglx2 + 1;
  order[lmax - 1] = lx1 - 1;
  return lmax;
}

/* ---- symmetric eigenproblem (cyclic Jacobi) -------------------------------- */
/* a (n x n, column-major, symmetric) is destroyed; lam ascending, V columns
 * the orthonormal eigenvectors in the same order. */
static void jacobi_eig(double *a, int n, double *lam, double *V) {
  double *v = (double *)malloc(sizeof(double) * n * n);
  for (int i = 0; i < n * n; ++i) v[i] = 0.0;
  for (int i = 0; i < n; ++i) v[i + n * i] = 1.0;
#define A_(i, j) a[(i) + n * (j)]
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        tot += A_(i, j) * A_(i, j);
        if (i != j) off += A_(i, j) * A_(i, j);
      }
    if (off <= 1e-32 * tot) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A_(p, q);
        if (apq == 0.0) continue;
        const double theta = (A_(q, q) - A_(p, p)) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) { /* columns p, q */
          const double akp = A_(k, p), akq = A_(k, q);
          A_(k, p) = c * akp - s * akq;
          A_(k, q) = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) { /* rows p, q */
          const double apk = A_(p, k), aqk = A_(q, k);
          A_(p, k) = c * apk - s * aqk;
          A_(q, k) = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = v[k + n * p], vkq = v[k + n * q];
          v[k + n * p] = c * vkp - s * vkq;
          v[k + n * q] = s * vkp + c * vkq;
        }
      }
  }
  int *ord = (int *)malloc(sizeof(int) * n);
  for (int i = 0; i < n; ++i) ord[i] = i;
  for (int i = 1; i < n; ++i) { /* insertion sort by eigenvalue */
    const int t = ord[i];
    int j = i - 1;
    while (j >= 0 && A_(ord[j], ord[j]) > A_(t, t)) {
      ord[j + 1] = ord[j];
      --j;
    }
    ord[j + 1] = t;
  }
  for (int i = 0; i < n; ++i) {
    lam[i] = A_(ord[i], ord[i]);
    for (int k = 0; k < n; ++k) V[k + n * i] = v[k + n * ord[i]];
  }
#undef A_
  free(ord);
  free(v);
}

/* ---- 1-D fast-diagonalisation operators (hsmg_setup_fast1d :783-881) ------ */
/* s: nl x nl eigenvectors (column j = vector j), then their transpose, with
 * the rows of excluded points zeroed; lam ascending.  n = order, nl = n + 3;
 * ah: (n+1)^2 stiffness, bh: n+1 weights. */
static void fast1d(double *s, double *lam, int lbc, int rbc, double ll, double lm, double lr,
                   const double *ah, const double *bh, int n) {
  const int nl = n + 3, na = n + 1;
  double *a = (double *)calloc((size_t)nl * nl, sizeof(double));
  double *b = (double *)calloc((size_t)nl, sizeof(double)); /* diagonal */
#define A_(i, j) a[(i) + nl * (j)]
#define AH(i, j) ah[(i) + na * (j)]
  const int i0 = lbc == 1 ? 1 : 0, i1 = rbc == 1 ? n - 1 : n;
  double fac = 2.0 / lm;
  A_(1, 1) = 1.0;
  A_(n + 1, n + 1) = 1.0;
  for (int j = i0; j <= i1; ++j)
    for (int i = i0; i <= i1; ++i) A_(i + 1, j + 1) = fac * AH(i, j);
  if (lbc == 0) {
    fac = 2.0 / ll;
    A_(0, 0) = fac * AH(n - 1, n - 1);
    A_(1, 0) = fac * AH(n, n - 1);
    A_(0, 1) = fac * AH(n - 1, n);
    A_(1, 1) = A_(1, 1) + fac * AH(n, n);
  } else {
    A_(0, 0) = 1.0;
  }
  if (rbc == 0) {
    fac = 2.0 / lr;
    A_(n + 1, n + 1) = A_(n + 1, n + 1) + fac * AH(0, 0);
    A_(n + 2, n + 1) = fac * AH(1, 0);
    A_(n + 1, n + 2) = fac * AH(0, 1);
    A_(n + 2, n + 2) = fac * AH(1, 1);
  } else {
    A_(n + 2, n + 2) = 1.0;
  }
  fac = 0.5 * lm; /* hsmg_setup_fast1d_b */
  b[1] = 1.0;
  b[n + 1] = 1.0;
  for (int i = i0; i <= i1; ++i) b[i + 1] = fac * bh[i];
  if (lbc == 0) {
    fac = 0.5 * ll;
    b[0] = fac * bh[n - 1];
    b[1] = b[1] + fac * bh[n];
  } else {
    b[0] = 1.0;
  }
  if (rbc == 0) {
    fac = 0.5 * lr;
    b[n + 1] = b[n + 1] + fac * bh[0];
    b[n + 2] = fac * bh[1];
  } else {
    b[n + 2] = 1.0;
  }
  /* A x = lam B x with B diagonal: C = B^-1/2 A B^-1/2, S = B^-1/2 V */
  double *c = (double *)malloc(sizeof(double) * nl * nl), *v = (double *)malloc(sizeof(double) * nl * nl);
  for (int j = 0; j < nl; ++j)
    for (int i = 0; i < nl; ++i) c[i + nl * j] = A_(i, j) / sqrt(b[i] * b[j]);
  jacobi_eig(c, nl, lam, v);
  for (int j = 0; j < nl; ++j)
    for (int i = 0; i < nl; ++i) s[i + nl * j] = v[i + nl * j] / sqrt(b[i]);
  for (int j = 0; j < nl; ++j) { /* row_zero: excluded points */
    if (lbc > 0) s[0 + nl * j] = 0.0;
    if (lbc == 1) s[1 + nl * j] = 0.0;
    if (rbc > 0) s[nl - 1 + nl * j] = 0.0;
    if (rbc == 1) s[nl - 2 + nl * j] = 0.0;
  }
  double *st = s + nl * nl;
  for (int j = 0; j < nl; ++j)
    for (int i = 0; i < nl; ++i) st[j + nl * i] = s[i + nl * j];
#undef A_
#undef AH
  free(a);
  free(b);
  free(c);
  free(v);
}

/* ---- element widths (swap_lengths, core/fast3d.f:1542-1617) --------------- */
/* lm[3 e + d]: harmonic-mean distance between the element's two faces normal
 * to direction d over the interior points (plane_space :306-423; its weights
 * are w(j) for interior point j, i.e. the GLL weight one index lower);
 * ll/lr: the same width of the neighbour across the left/right face (0 on the
 * boundary), taken from a dssum of the widths on the face interiors. */
static void swap_lengths(const ref_ops *ops, const double *x, const double *y, const double *z,
                         const double *w, double *ll, double *lm, double *lr) {
  const int nx1 = ref_ops_nx1(ops), nel = ref_ops_nel(ops), m = nx1 - 2, n2 = nx1 - 1;
  const int64_t nxyz = (int64_t)nx1 * nx1 * nx1;
#define P(i, j, k) ((i) + nx1 * ((j) + nx1 * (k)))
  for (int e = 0; e < nel; ++e) {
    const double *xe = x + e * nxyz, *ye = y + e * nxyz, *ze = z + e * nxyz;
    for (int d = 0; d < 3; ++d) {
      double l2 = 0.0, wsum = 0.0;
      for (int b = 1; b <= m; ++b)
        for (int a = 1; a <= m; ++a) {
          const double weight = w[a - 1] * w[b - 1];
          int p1, p2;
          if (d == 0) {
            p1 = P(0, a, b);
            p2 = P(n2, a, b);
          } else if (d == 1) {
            p1 = P(a, 0, b);
            p2 = P(a, n2, b);
          } else {
            p1 = P(a, b, 0);
            p2 = P(a, b, n2);
          }
          const double dx = xe[p2] - xe[p1], dy = ye[p2] - ye[p1], dz = ze[p2] - ze[p1];
          l2 = l2 + weight / (dx * dx + dy * dy + dz * dz);
          wsum = wsum + weight;
        }
      l2 = l2 / wsum;
      lm[3 * e + d] = 1.0 / sqrt(l2);
    }
  }
  double *l = (double *)calloc((size_t)(nxyz * nel), sizeof(double));
  for (int e = 0; e < nel; ++e) {
    double *le = l + e * nxyz;
    for (int j = 1; j <= m; ++j)
      for (int k = 1; k <= m; ++k) {
        le[P(0, k, j)] = lm[3 * e];
        le[P(n2, k, j)] = lm[3 * e];
        le[P(k, 0, j)] = lm[3 * e + 1];
        le[P(k, n2, j)] = lm[3 * e + 1];
        le[P(k, j, 0)] = lm[3 * e + 2];
        le[P(k, j, n2)] = lm[3 * e + 2];
      }
  }
  ref_dssum(ops, l);
  for (int e = 0; e < nel; ++e) {
    const double *le = l + e * nxyz;
    ll[3 * e] = le[P(0, 1, 1)] - lm[3 * e];
    lr[3 * e] = le[P(n2, 1, 1)] - lm[3 * e];
    ll[3 * e + 1] = le[P(1, 0, 1)] - lm[3 * e + 1];
    lr[3 * e + 1] = le[P(1, n2, 1)] - lm[3 * e + 1];
    ll[3 * e + 2] = le[P(1, 1, 0)] - lm[3 * e + 2];
    lr[3 * e + 2] = le[P(1, 1, n2)] - lm[3 * e + 2];
  }
#undef P
  free(l);
}

/* ---- extended-element arrays ---------------------------------------------- */
/* hsmg_extrude (:368-423): on the face regions (the nl-2 by nl-2 middle of
 * each face) of every element, arr1[layer l1 from the face] = f1 arr1[...] +
 * f2 arr2[layer l2 from the face]; faces r, s, t in turn. */
static void extrude(double *a1, int l1, double f1, const double *a2, int l2, double f2, int nl,
                    int nel) {
  const int64_t nn = (int64_t)nl * nl * nl;
#define X(i, j, k) ((i) + nl * ((j) + nl * (k)))
  for (int e = 0; e < nel; ++e) {
    double *u = a1 + e * nn;
    const double *v = a2 + e * nn;
    for (int k = 1; k <= nl - 2; ++k)
      for (int j = 1; j <= nl - 2; ++j) {
        u[X(l1, j, k)] = f1 * u[X(l1, j, k)] + f2 * v[X(l2, j, k)];
        u[X(nl - 1 - l1, j, k)] = f1 * u[X(nl - 1 - l1, j, k)] + f2 * v[X(nl - 1 - l2, j, k)];
      }
    for (int k = 1; k <= nl - 2; ++k)
      for (int i = 1; i <= nl - 2; ++i) {
        u[X(i, l1, k)] = f1 * u[X(i, l1, k)] + f2 * v[X(i, l2, k)];
        u[X(i, nl - 1 - l1, k)] = f1 * u[X(i, nl - 1 - l1, k)] + f2 * v[X(i, nl - 1 - l2, k)];
      }
    for (int j = 1; j <= nl - 2; ++j)
      for (int i = 1; i <= nl - 2; ++i) {
        u[X(i, j, l1)] = f1 * u[X(i, j, l1)] + f2 * v[X(i, j, l2)];
        u[X(i, j, nl - 1 - l1)] = f1 * u[X(i, j, nl - 1 - l1)] + f2 * v[X(i, j, nl - 1 - l2)];
      }
  }
}

static void to_ext(double *a, const double *b, int nx, int nel) { /* hsmg_schwarz_toext3d */
  const int nl = nx + 2;
  const int64_t nn = (int64_t)nl * nl * nl, nb = (int64_t)nx * nx * nx;
  memset(a, 0, sizeof(double) * nn * nel);
  for (int e = 0; e < nel; ++e)
    for (int k = 0; k < nx; ++k)
      for (int j = 0; j < nx; ++j)
        for (int i = 0; i < nx; ++i)
          a[e * nn + X(i + 1, j + 1, k + 1)] = b[e * nb + i + nx * (j + nx * k)];
}

static void to_reg(double *b, const double *a, int nx, int nel) { /* hsmg_schwarz_toreg3d */
  const int nl = nx + 2;
  const int64_t nn = (int64_t)nl * nl * nl, nb = (int64_t)nx * nx * nx;
  for (int e = 0; e < nel; ++e)
    for (int k = 0; k < nx; ++k)
      for (int j = 0; j < nx; ++j)
        for (int i = 0; i < nx; ++i)
          b[e * nb + i + nx * (j + nx * k)] = a[e * nn + X(i + 1, j + 1, k + 1)];
}
#undef X

/* v = [C (x) B (x) A] u on one element (hsmg_tnsr3d_el :309-324): A nv x nu,
 * Bt = B^T and Ct = C^T nu x nv. */
static void tnsr3d_el(double *v, int nv, const double *u, int nu, const double *A,
                      const double *Bt, const double *Ct, double *work, double *work2) {
  ref_mxm(A, nv, u, nu, work, nu * nu);
  for (int i = 0; i < nu; ++i) ref_mxm(work + nv * nu * i, nv, Bt, nu, work2 + nv * nv * i, nv);
  ref_mxm(work2, nv * nv, Ct, nu, v, nv);
}

/* ---- setup ---------------------------------------------------------------- */
static int cmp_i64(const void *a, const void *b) {
  const int64_t x = *(const int64_t *)a, y = *(const int64_t *)b;
  return x < y ? -1 : x > y;
}

/* zero the points of face f (r-, r+, s-, s+, t-, t+) of an nx^3 element */
static void face_zero(double *u, int nx, int f) {
  for (int b = 0; b < nx; ++b)
    for (int a = 0; a < nx; ++a) {
      const int fix = (f & 1) ? nx - 1 : 0;
      int p;
      if (f < 2) p = fix + nx * (a + nx * b);
      else if (f < 4) p = a + nx * (fix + nx * b);
      else p = a + nx * (b + nx * fix);
      u[p] = 0.0;
    }
}

/* Cholesky A = L L^T (lower, column-major, n x n, in place); 0 or -1. */
static int chol(double *A, int64_t n) {
  for (int64_t j = 0; j < n; ++j) {
    double d = A[j + n * j];
    for (int64_t k = 0; k < j; ++k) d -= A[j + n * k] * A[j + n * k];
    if (!(d > 0.0)) return -1;
    d = sqrt(d);
    A[j + n * j] = d;
    for (int64_t i = j + 1; i < n; ++i) {
      double s = A[i + n * j];
      for (int64_t k = 0; k < j; ++k) s -= A[i + n * k] * A[j + n * k];
      A[i + n * j] = s / d;
    }
  }
  return 0;
}

ref_h1mg *ref_h1mg_create(const ref_ops *ops, const double *x, const double *y, const double *z,
                          const int *fbc, const int64_t *vertex, int null_space) {
  const int nx1 = ref_ops_nx1(ops), nel = ref_ops_nel(ops);
  if (nx1 < 3 || nx1 > 14) return NULL;
  ref_h1mg *mg = (ref_h1mg *)calloc(1, sizeof(ref_h1mg));
  mg->ops = ops;
  mg->nel = nel;
  mg->null_space = null_space;
  int order[MGMAX];
  mg->lmax = ref_h1mg_levels(nx1, order);
  /* vertex ids ranked 1..nv (setvert3d numbers edges and faces after them) */
  const int64_t nvt = 8 * (int64_t)nel;
  int64_t *srt = (int64_t *)malloc(sizeof(int64_t) * nvt), *vr = (int64_t *)malloc(sizeof(int64_t) * nvt);
  memcpy(srt, vertex, sizeof(int64_t) * nvt);
  qsort(srt, (size_t)nvt, sizeof(int64_t), cmp_i64);
  int64_t nu = 0;
  for (int64_t i = 0; i < nvt; ++i)
    if (i == 0 || srt[i] != srt[i - 1]) srt[nu++] = srt[i];
  for (int64_t i = 0; i < nvt; ++i) {
    const int64_t *p = (const int64_t *)bsearch(&vertex[i], srt, (size_t)nu, sizeof(int64_t), cmp_i64);
    vr[i] = (p - srt) + 1;
  }
  free(srt);
  double *lw = (double *)malloc(sizeof(double) * 9 * nel);
  double *wf = (double *)malloc(sizeof(double) * nx1), *zf = (double *)malloc(sizeof(double) * nx1);
  ref_zwgll(zf, wf, nx1);
  swap_lengths(ops, x, y, z, wf, lw, lw + 3 * nel, lw + 6 * nel);
  const double *lenl = lw, *lenm = lw + 3 * nel, *lenr = lw + 6 * nel;
  for (int l = 0; l < mg->lmax; ++l) {
    mglev *L = &mg->lev[l];
    const int N = order[l], nx = N + 1, nl = nx + 2;
    L->nx = nx;
    L->n = (int64_t)nx * nx * nx * nel;
    ref_zwgll(L->z, L->w, nx);
    /* semhat: D from the Fornberg weights, a = D^T diag(w) D */
    double c[64], D[256];
    for (int i = 0; i <= N; ++i) {
      ref_fd_weights(L->z[i], L->z, N, 1, c);
      for (int j = 0; j <= N; ++j) D[i + nx * j] = c[j + nx];
    }
    for (int j = 0; j <= N; ++j)
      for (int i = 0; i <= N; ++i) {
        double a = 0.0;
        for (int k = 0; k <= N; ++k) a = a + D[k + nx * i] * L->w[k] * D[k + nx * j];
        L->ah[i + nx * j] = a;
      }
    if (l > 0) { /* jh: values at this level's points from the coarser level's */
      const mglev *C = &mg->lev[l - 1];
      const int nc = C->nx;
      for (int i = 0; i < nx; ++i) {
        ref_fd_weights(L->z[i], C->z, nc - 1, 1, c);
        for (int j = 0; j < nc; ++j) L->jh[i + nx * j] = c[j];
      }
      for (int i = 0; i < nx; ++i)
        for (int j = 0; j < nc; ++j) L->jht[j + nc * i] = L->jh[i + nx * j];
    }
    /* numberings (setupds: set_vert on the level and on the extended grid) */
    int64_t *glo = (int64_t *)malloc(sizeof(int64_t) * (int64_t)nl * nl * nl * nel), ngv;
    ref_setvert3d(glo, &ngv, nx, nel, vr);
    L->gs = ref_gs_setup(glo, L->n);
    if (l == 0) { /* coarse unknowns: the unmasked level-1 ids */
      mg->cid = (int64_t *)malloc(sizeof(int64_t) * L->n);
      memcpy(mg->cid, glo, sizeof(int64_t) * L->n);
    }
    ref_setvert3d(glo, &ngv, nl, nel, vr);
    L->gse = ref_gs_setup(glo, (int64_t)nl * nl * nl * nel);
    free(glo);
    /* mask (h1mg_setup_mask :2426-2508): Dirichlet faces, then dsprod */
    L->mask = (double *)malloc(sizeof(double) * L->n);
    for (int64_t i = 0; i < L->n; ++i) L->mask[i] = 1.0;
    const int64_t nxyz = (int64_t)nx * nx * nx;
    for (int e = 0; e < nel; ++e)
      for (int f = 0; f < 6; ++f)
        if (fbc[6 * e + f] == 1) face_zero(L->mask + e * nxyz, nx, f);
    ref_gs_op(L->gs, L->mask, 1);
    /* restriction weights (hsmg_setup_rstr_wt :987-1067) */
    L->rwt = (double *)malloc(sizeof(double) * L->n);
    for (int64_t i = 0; i < L->n; ++i) L->rwt[i] = 1.0;
    ref_gs_op(L->gs, L->rwt, 0);
    for (int64_t i = 0; i < L->n; ++i) L->rwt[i] = 1.0 / L->rwt[i];
    if (l == 0) continue;
    /* fast diagonalisation (hsmg_setup_fast :701-781) */
    const int64_t nn = (int64_t)nl * nl * nl;
    L->S = (double *)malloc(sizeof(double) * 6 * nl * nl * nel);
    L->dinv = (double *)malloc(sizeof(double) * nn * nel);
    double lam[3][32];
    for (int e = 0; e < nel; ++e) {
      for (int d = 0; d < 3; ++d)
        fast1d(L->S + ((int64_t)e * 3 + d) * 2 * nl * nl, lam[d], fbc[6 * e + 2 * d],
               fbc[6 * e + 2 * d + 1], lenl[3 * e + d], lenm[3 * e + d], lenr[3 * e + d], L->ah,
               L->w, N);
      double mx[3];
      for (int d = 0; d < 3; ++d) { /* vlmax(lam(2), nl-2) */
        mx[d] = lam[d][1];
        for (int i = 2; i <= nl - 2; ++i)
          if (lam[d][i] > mx[d]) mx[d] = lam[d][i];
      }
      const double eps = 1.e-5 * (mx[0] + mx[1] + mx[2]);
      double *de = L->dinv + e * nn;
      int64_t il = 0;
      for (int k = 0; k < nl; ++k)
        for (int j = 0; j < nl; ++j)
          for (int i = 0; i < nl; ++i) {
            const double diag = lam[0][i] + lam[1][j] + lam[2][k];
            de[il++] = diag > eps ? 1.0 / diag : 0.0;
          }
    }
    /* Schwarz weights (h1mg_setup_schwarz_wt_1 :3048-3104) */
    double *A = (double *)calloc((size_t)(nn * nel), sizeof(double));
    double *B = (double *)malloc(sizeof(double) * nn * nel);
    for (int64_t i = 0; i < nn * nel; ++i) B[i] = 1.0;
    extrude(A, 0, 0.0, B, 0, 1.0, nl, nel);
    ref_gs_op(L->gse, B, 0);
    extrude(B, 0, 1.0, A, 0, -1.0, nl, nel);
    extrude(B, 2, 1.0, B, 0, 1.0, nl, nel);
    L->swt = (double *)malloc(sizeof(double) * L->n);
    to_reg(L->swt, B, nx, nel);
    ref_gs_op(L->gs, L->swt, 0);
    for (int64_t i = 0; i < L->n; ++i) L->swt[i] = 1.0 / L->swt[i];
    free(A);
    free(B);
  }
  free(vr);
  mg->len = (double *)malloc(sizeof(double) * 9 * nel);
  for (int e = 0; e < nel; ++e)
    for (int d = 0; d < 3; ++d) {
      mg->len[9 * e + d] = lenl[3 * e + d];
      mg->len[9 * e + 3 + d] = lenm[3 * e + d];
      mg->len[9 * e + 6 + d] = lenr[3 * e + d];
    }
  free(lw);
  /* coarse unknowns and the Galerkin matrix (set_up_h1_crs, core/navier8.f:83-238) */
  {
    const mglev *C = &mg->lev[0];
    const int64_t n1 = C->n;
    int64_t *ids = (int64_t *)malloc(sizeof(int64_t) * n1);
    int64_t m = 0;
    for (int64_t i = 0; i < n1; ++i)
      if (C->mask[i] >= 0.1) ids[m++] = mg->cid[i];
    qsort(ids, (size_t)m, sizeof(int64_t), cmp_i64);
    int64_t nc = 0;
    for (int64_t i = 0; i < m; ++i)
      if (i == 0 || ids[i] != ids[i - 1]) ids[nc++] = ids[i];
    for (int64_t i = 0; i < n1; ++i) {
      if (C->mask[i] < 0.1) {
        mg->cid[i] = -1;
        continue;
      }
      const int64_t *p = (const int64_t *)bsearch(&mg->cid[i], ids, (size_t)nc, sizeof(int64_t), cmp_i64);
      mg->cid[i] = p - ids;
    }
    free(ids);
    mg->nc = nc;
    const int64_t nxyz = (int64_t)nx1 * nx1 * nx1, n = ref_ops_n(ops);
    double *b = (double *)malloc(sizeof(double) * 8 * nxyz); /* gen_crs_basis */
    for (int j = 0; j < 8; ++j)
      for (int r = 0; r < nx1; ++r)
        for (int q = 0; q < nx1; ++q)
          for (int p = 0; p < nx1; ++p) {
            const double zr = (j & 1) ? 0.5 * (1 + zf[p]) : 0.5 * (1 - zf[p]);
            const double zs = (j & 2) ? 0.5 * (1 + zf[q]) : 0.5 * (1 - zf[q]);
            const double zt = (j & 4) ? 0.5 * (1 + zf[r]) : 0.5 * (1 - zf[r]);
            b[j * nxyz + p + nx1 * (q + nx1 * r)] = zr * zs * zt;
          }
    double *w1 = (double *)malloc(sizeof(double) * n), *w2 = (double *)malloc(sizeof(double) * n);
    double *h1 = (double *)malloc(sizeof(double) * n), *h2 = (double *)calloc((size_t)n, sizeof(double));
    for (int64_t i = 0; i < n; ++i) h1[i] = 1.0;
    double *Ac = (double *)calloc((size_t)(nc * nc), sizeof(double));
    for (int j = 0; j < 8; ++j) {
      for (int e = 0; e < nel; ++e) memcpy(w1 + e * nxyz, b + j * nxyz, sizeof(double) * nxyz);
      ref_axhelm(ops, w2, w1, h1, h2);
      for (int e = 0; e < nel; ++e)
        for (int i = 0; i < 8; ++i) {
          double a = 0.0; /* vlsc2 */
          for (int64_t p = 0; p < nxyz; ++p) a = a + b[i * nxyz + p] * w2[e * nxyz + p];
          const int64_t ci = mg->cid[8 * e + i], cj = mg->cid[8 * e + j];
          if (ci >= 0 && cj >= 0) Ac[ci + nc * cj] += a;
        }
    }
    free(b);
    free(w1);
    free(w2);
    free(h1);
    free(h2);
    const int64_t ns = (null_space && nc > 0) ? nc - 1 : nc;
    mg->nsolve = ns;
    mg->L = (double *)malloc(sizeof(double) * (ns > 0 ? ns * ns : 1));
    for (int64_t j = 0; j < ns; ++j)
      for (int64_t i = 0; i < ns; ++i) mg->L[i + ns * j] = Ac[i + nc * j];
    free(Ac);
    if (chol(mg->L, ns)) {
      ref_h1mg_free(mg);
      free(wf);
      free(zf);
      return NULL;
    }
  }
  free(wf);
  free(zf);
  const int64_t nfine = ref_ops_n(ops);
  mg->vmult = (double *)malloc(sizeof(double) * nfine);
  for (int64_t i = 0; i < nfine; ++i) mg->vmult[i] = 1.0;
  ref_dssum(ops, mg->vmult);
  for (int64_t i = 0; i < nfine; ++i) mg->vmult[i] = 1.0 / mg->vmult[i];
  const int nlf = nx1 + 2;
  const int64_t ne = (int64_t)nlf * nlf * nlf * nel;
  mg->ext0 = (double *)malloc(sizeof(double) * ne);
  mg->ext1 = (double *)malloc(sizeof(double) * ne);
  mg->ext2 = (double *)malloc(sizeof(double) * ne);
  return mg;
}

void ref_h1mg_free(ref_h1mg *mg) {
  if (!mg) return;
  for (int l = 0; l < MGMAX; ++l) {
    mglev *L = &mg->lev[l];
    if (L->gs) ref_gs_free(L->gs);
    if (L->gse) ref_gs_free(L->gse);
    free(L->mask);
    free(L->rwt);
    free(L->swt);
    free(L->S);
    free(L->dinv);
  }
  free(mg->cid);
  free(mg->len);
  free(mg->L);
  free(mg->vmult);
  free(mg->ext0);
  free(mg->ext1);
  free(mg->ext2);
  free(mg);
}

/* ---- apply ---------------------------------------------------------------- */
/* e = W sigma (Schwarz on level l) r; r is masked in place (h1mg_schwarz
 * :425-438, h1mg_schwarz_part1 :440-494). */
static void schwarz(const ref_h1mg *mg, int l, double *e, double *r) {
  const mglev *L = &mg->lev[l];
  const int nx = L->nx, nl = nx + 2, nel = mg->nel;
  const int64_t nn = (int64_t)nl * nl * nl;
  double *A = mg->ext0, *E = mg->ext1;
  for (int64_t i = 0; i < L->n; ++i)
    if (L->mask[i] == 0.0) r[i] = 0.0;
  to_ext(A, r, nx, nel);
  /* exchange: the border layers take the neighbours' first interior layers */
  extrude(A, 0, 0.0, A, 2, 1.0, nl, nel);
  ref_gs_op(L->gse, A, 0);
  extrude(A, 0, 1.0, A, 2, -1.0, nl, nel);
  /* local solves: E = S diag(1/lambda) S^T A, element by element */
  double work[4096], work2[4096];
  for (int el = 0; el < nel; ++el) {
    const double *S = L->S + (int64_t)el * 6 * nl * nl; /* [d][S, S^T] */
    const double *Sr = S, *SrT = S + nl * nl, *Ss = S + 2 * nl * nl, *SsT = S + 3 * nl * nl;
    const double *St = S + 4 * nl * nl, *StT = S + 5 * nl * nl;
    double *ae = A + el * nn, *ee = E + el * nn;
    tnsr3d_el(ee, nl, ae, nl, SrT, Ss, St, work, work2);
    const double *de = L->dinv + el * nn;
    for (int64_t i = 0; i < nn; ++i) ae[i] = de[i] * ee[i];
    tnsr3d_el(ee, nl, ae, nl, Sr, SsT, StT, work, work2);
  }
  /* sum the overlap: each element's border solution goes back to the
     neighbour's first interior layer */
  extrude(A, 0, 0.0, E, 0, 1.0, nl, nel);
  ref_gs_op(L->gse, E, 0);
  extrude(E, 0, 1.0, A, 0, -1.0, nl, nel);
  extrude(E, 2, 1.0, E, 0, 1.0, nl, nel);
  to_reg(e, E, nx, nel);
  ref_gs_op(L->gs, e, 0);
  for (int64_t i = 0; i < L->n; ++i) {
    if (L->mask[i] == 0.0) e[i] = 0.0;
    e[i] = e[i] * L->swt[i]; /* hsmg_schwarz_wt */
    e[i] = e[i] * 1.0;       /* sigma */
  }
}

/* v (level l) = [J (x) J (x) J] u (level l-1), hsmg_intp / hsmg_tnsr3d */
static void intp(const ref_h1mg *mg, int l, double *v, const double *u) {
  const mglev *F = &mg->lev[l], *C = &mg->lev[l - 1];
  const int nf = F->nx, nc = C->nx;
  const int64_t n3f = (int64_t)nf * nf * nf, n3c = (int64_t)nc * nc * nc;
  double work[4096], work2[4096];
  for (int e = 0; e < mg->nel; ++e)
    tnsr3d_el(v + e * n3f, nf, u + e * n3c, nc, F->jh, F->jht, F->jht, work, work2);
}

/* u (level l-1) = [J^T (x) J^T (x) J^T] (rwt r) (level l) (h1mg_rstr);
 * r is weighted in place as the reference does */
static void rstr(const ref_h1mg *mg, int l, double *u, double *r, int dssum) {
  const mglev *F = &mg->lev[l], *C = &mg->lev[l - 1];
  const int nf = F->nx, nc = C->nx;
  const int64_t n3f = (int64_t)nf * nf * nf, n3c = (int64_t)nc * nc * nc;
  for (int64_t i = 0; i < F->n; ++i) r[i] = r[i] * F->rwt[i];
  double work[4096], work2[4096];
  for (int e = 0; e < mg->nel; ++e)
    tnsr3d_el(u + e * n3c, nc, r + e * n3f, nf, F->jht, F->jh, F->jh, work, work2);
  if (dssum) ref_gs_op(C->gs, u, 0);
}

/* e = A_c^-1 r on the coarse level (crs_solve, core/crs_xxt.c:918-962):
 * r element-local (summed into the unknowns here), e element-local */
static void coarse_solve(const ref_h1mg *mg, double *e, const double *r) {
  const int64_t nc = mg->nc, ns = mg->nsolve, n1 = mg->lev[0].n;
  double *v = (double *)calloc((size_t)(nc > 0 ? nc : 1), sizeof(double));
  for (int64_t i = 0; i < n1; ++i)
    if (mg->cid[i] >= 0) v[mg->cid[i]] += r[i];
  const double *L = mg->L;
  for (int64_t i = 0; i < ns; ++i) { /* L y = v */
    double s = v[i];
    for (int64_t k = 0; k < i; ++k) s -= L[i + ns * k] * v[k];
    v[i] = s / L[i + ns * i];
  }
  for (int64_t i = ns - 1; i >= 0; --i) { /* L^T x = y */
    double s = v[i];
    for (int64_t k = i + 1; k < ns; ++k) s -= L[k + ns * i] * v[k];
    v[i] = s / L[i + ns * i];
  }
  if (mg->null_space && nc > 0) {
    v[nc - 1] = 0.0;
    double s = 0.0;
    const double sw = 1.0 / (double)nc;
    for (int64_t i = 0; i < nc; ++i) s += sw * v[i];
    for (int64_t i = 0; i < nc; ++i) v[i] -= s;
  }
  for (int64_t i = 0; i < n1; ++i) e[i] = mg->cid[i] >= 0 ? v[mg->cid[i]] : 0.0;
  free(v);
}

void ref_h1mg_solve(const ref_h1mg *mg, double *z, double *rhs) {
  const int lmax = mg->lmax;
  const mglev *Lf = &mg->lev[lmax - 1];
  double *e[MGMAX] = {0}, *r[MGMAX] = {0};
  for (int l = 0; l < lmax - 1; ++l) {
    e[l] = (double *)calloc((size_t)mg->lev[l].n, sizeof(double));
    r[l] = (double *)calloc((size_t)mg->lev[l].n, sizeof(double));
  }
  double *rf = (double *)malloc(sizeof(double) * Lf->n);
  schwarz(mg, lmax - 1, z, rhs);
  memcpy(rf, rhs, sizeof(double) * Lf->n);
  double *rcur = rf;
  for (int l = lmax - 2; l >= 1; --l) { /* downward leg */
    rstr(mg, l + 1, r[l], rcur, 1);
    schwarz(mg, l, e[l], r[l]);
    rcur = r[l];
  }
  rstr(mg, 1, r[0], rcur, 0);
  for (int64_t i = 0; i < mg->lev[0].n; ++i)
    if (mg->lev[0].mask[i] == 0.0) r[0][i] = 0.0;
  coarse_solve(mg, e[0], r[0]);
  for (int64_t i = 0; i < mg->lev[0].n; ++i)
    if (mg->lev[0].mask[i] == 0.0) e[0][i] = 0.0;
  for (int l = 1; l < lmax - 1; ++l) { /* unwind, no smoothing */
    double *w = (double *)malloc(sizeof(double) * mg->lev[l].n);
    intp(mg, l, w, e[l - 1]);
    for (int64_t i = 0; i < mg->lev[l].n; ++i) e[l][i] = e[l][i] + w[i];
    free(w);
  }
  double *w = (double *)malloc(sizeof(double) * Lf->n);
  intp(mg, lmax - 1, w, e[lmax - 2]);
  for (int64_t i = 0; i < Lf->n; ++i) z[i] = z[i] + w[i];
  free(w);
  ref_dssum(mg->ops, z); /* dsavg */
  for (int64_t i = 0; i < Lf->n; ++i) z[i] = z[i] * mg->vmult[i];
  for (int l = 0; l < lmax - 1; ++l) {
    free(e[l]);
    free(r[l]);
  }
  free(rf);
}

/* Level data for tests: order (polynomial) and sizes; pointers into the
 * setup for level l (0 = coarsest). */
int ref_h1mg_nlev(const ref_h1mg *mg) { return mg->lmax; }
int ref_h1mg_nx(const ref_h1mg *mg, int l) { return mg->lev[l].nx; }
int64_t ref_h1mg_ncoarse(const ref_h1mg *mg) { return mg->nc; }
void ref_h1mg_level(const ref_h1mg *mg, int l, double *mask, double *rwt, double *swt) {
  const mglev *L = &mg->lev[l];
  if (mask) memcpy(mask, L->mask, sizeof(double) * L->n);
  if (rwt) memcpy(rwt, L->rwt, sizeof(double) * L->n);
  if (swt && L->swt) memcpy(swt, L->swt, sizeof(double) * L->n);
}
/* the Schwarz solve of one level alone (tests) */
void ref_h1mg_schwarz(const ref_h1mg *mg, int l, double *e, double *r) { schwarz(mg, l, e, r); }
void ref_h1mg_coarse(const ref_h1mg *mg, double *e, const double *r) { coarse_solve(mg, e, r); }

/* One 1-D fast-diagonalisation operator of order n (tests): s (column j =
 * vector j, excluded rows zeroed) and lam ascending, nl = n + 3. */
void ref_fdm1d(int n, int lbc, int rbc, double ll, double lm, double lr, double *s, double *lam) {
  const int nx = n + 1;
  double z[16], w[16], c[64], D[256], ah[256];
  ref_zwgll(z, w, nx);
  for (int i = 0; i <= n; ++i) {
    ref_fd_weights(z[i], z, n, 1, c);
    for (int j = 0; j <= n; ++j) D[i + nx * j] = c[j + nx];
  }
  for (int j = 0; j <= n; ++j)
    for (int i = 0; i <= n; ++i) {
      double a = 0.0;
      for (int k = 0; k <= n; ++k) a = a + D[k + nx * i] * w[k] * D[k + nx * j];
      ah[i + nx * j] = a;
    }
  double *tmp = (double *)malloc(sizeof(double) * 2 * (n + 3) * (n + 3));
  fast1d(tmp, lam, lbc, rbc, ll, lm, lr, ah, w, n);
  memcpy(s, tmp, sizeof(double) * (n + 3) * (n + 3));
  free(tmp);
}

void ref_h1mg_lengths(const ref_h1mg *mg, double *out) {
  memcpy(out, mg->len, sizeof(double) * 9 * mg->nel);
}
