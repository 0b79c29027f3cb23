/*
 * nekref.h -- CPU oracle for the Nek5000 Helmholtz/Poisson solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a C restatement of the reference
 * Fortran (Nek5000 core/ *.f files) in the same loop and accumulation order, used
 * by the test-suite as the parity checker and by bench.py as the timed CPU
 * baseline.  The product library (nek5000_gb300/csrc) never links, loads or
 * calls it.
 *
 * Parity unpinned: the reference Fortran cannot be compiled or run here and
 * ships no function-level golden vectors, so this restatement is pinned by
 * known-answer tests (quadrature and differentiation exactness, operator
 * symmetry and null space, spectral convergence) rather than by reference
 * outputs.
 *
 * Array conventions follow the Fortran: every field is (lx1,ly1,lz1,nel)
 * column-major (x fastest, element slowest), 0-based here.  D(i,j) is stored
 * d[i + j*nx].  All arithmetic is FP64, compiled with -ffp-contract=off so no
 * multiply-add is fused (gfortran's default for these loops).
 */
#ifndef NEKREF_H
#define NEKREF_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- spectral library (core/speclib.f) ---------------------------------- */
void ref_zwgll(double *z, double *w, int np);                          /* ZWGLL  speclib.f:107 */
void ref_dgll(double *d, double *dt, const double *z, int nz);         /* DGLL   speclib.f:811 */

/* ---- synthetic deformed box (harness input, not on the solve path) ------- */
/* kx*ky*kz hex elements on the unit cube, element e = ex + kx*(ey + ky*ez).
 * GLL nodes by the trilinear map, then x -> x + amp*sin(pi x)sin(pi y)sin(pi z)*v.
 * vertex(8,nel): hypercube-ordered lattice ids, wrapped in y/z when periodic. */
void ref_box_mesh(int nx1, int kx, int ky, int kz, int periodic_y, int periodic_z,
                  double amp, const double *v3, double *xm1, double *ym1, double *zm1,
                  int64_t *vertex);

/* ---- geometry (core/coef.f xyzrst/glmapm1/geodat1) ----------------------- */
/* g6 holds G1..G6 as six consecutive arrays of n = nx1^3*nel. */
void ref_geom(int nx1, int nel, const double *xm1, const double *ym1, const double *zm1,
              double *g6, double *bm1, double *jacm1);

/* ---- global numbering (core/navier8.f setvert3d) ------------------------- */
void ref_setvert3d(int64_t *glo_num, int64_t *ngv, int nx, int nel, const int64_t *vertex);

/* ---- gather-scatter (gslib gs_setup/gs_op semantics) --------------------- */
typedef struct ref_gs ref_gs;
ref_gs *ref_gs_setup(const int64_t *glo_num, int64_t n);
void ref_gs_free(ref_gs *gs);
/* op: 0 '+', 1 '*', 2 'M' (max), 3 'm' (min) */
void ref_gs_op(const ref_gs *gs, double *u, int op);
/* number of shared groups / total members in them; fills CSR maps when non-null */
int64_t ref_gs_nseg(const ref_gs *gs);
int64_t ref_gs_nidx(const ref_gs *gs);
void ref_gs_maps(const ref_gs *gs, int64_t *seg_start, int64_t *idx, int64_t *seg_id);

/* ---- operator state ------------------------------------------------------ */
typedef struct ref_ops ref_ops;
/* Pointers are borrowed (caller keeps them alive).  d/dt: D and D^T. */
ref_ops *ref_ops_create(int nx1, int nel, const double *d, const double *dt,
                        const double *g6, const double *bm1, const int64_t *glo_num,
                        int nthreads);
void ref_ops_free(ref_ops *ops);
const ref_gs *ref_ops_gs(const ref_ops *ops);

void ref_axhelm(const ref_ops *ops, double *au, const double *u, const double *h1,
                const double *h2);                                   /* hmholtz.f:72  */
void ref_dssum(const ref_ops *ops, double *u);                       /* dssum.f:33    */
void ref_dsop(const ref_ops *ops, double *u, int op);                 /* dssum.f:100   */
void ref_setprec(const ref_ops *ops, double *d, const double *h1, const double *h2); /* :380 */
void ref_setprec_local(const ref_ops *ops, double *d, const double *h1, const double *h2);
double ref_glsc3(const ref_ops *ops, const double *a, const double *b, const double *m);
void ref_chktcg1(const ref_ops *ops, double *tol, const double *res, const double *h1,
                 const double *h2, const double *mask, const double *mult,
                 const double *binv);                                /* hmholtz.f:527 */
/* cggo (hmholtz.f:611).  maxcg = the reference's 900 cap (pass a large value
 * to lift it).  istep feeds the "take at least one iteration" rule.
 * Returns niter; rbn0/rbn2 out. */
int ref_cggo(const ref_ops *ops, double *x, const double *f, const double *h1,
             const double *h2, const double *mask, const double *mult, double tin,
             int maxit, int maxcg, int istep, const double *binv, double *rbn0,
             double *rbn2);
/* hmholtz (hmholtz.f:2): dssum+mask the rhs (in place), chktcg1, cggo. */
int ref_hmholtz(const ref_ops *ops, double *u, double *rhs, const double *h1,
                const double *h2, const double *mask, const double *mult, double tli,
                int maxit, int maxcg, int istep, const double *binv, double *rbn0,
                double *rbn2);

/* ---- residual projection onto previous solutions (navier4.f:562-1188) --- */
/* One projection space (X, B = A X, xbar, bbar, h1old, h2old; the
 * reference's approx / napprox arrays) of at most mmx vectors
 * ((mxprev-4)/2 = 8 in the reference's default SIZE). */
typedef struct ref_proj ref_proj;
ref_proj *ref_proj_create(const ref_ops *ops, int mmx);
void ref_proj_free(ref_proj *p);
int ref_proj_m(const ref_proj *p);
const double *ref_proj_x(const ref_proj *p, int k);
const double *ref_proj_b(const ref_proj *p, int k);
/* hsolve with projection (navier4.f:562, ifstdh = .false.): r is masked and
 * dssum'ed in place, projected (project1), solved by hmhzpf (chktcg1 +
 * cggo, tolerance tli as chktcg1 leaves it), u un-projected and appended to
 * the space (project2).  Returns cggo's niter. */
int ref_hsolve(const ref_ops *ops, ref_proj *p, double *u, double *r, const double *h1,
               const double *h2, const double *vmk, const double *vml, double tli, int maxit,
               int maxcg, int istep, const double *binv, double *rbn0, double *rbn2);

/* hmh_gmres (gmres.f:304-560): right-preconditioned restarted GMRES on
 * ax() = dssum(axhelm(x)) * mask (gmres.f:284-302), weights wt (vmult),
 * restart length m (lgmres), classical Gram-Schmidt (the 1st pass of
 * :430-446), Givens rotations, back substitution; ml = mu = 1
 * (uzawa_gmres_split :252-271); ortho() (navier1.f:223-256) removes the mean
 * of z_j and of the result when null_space is set.  The preconditioner is
 * M w = d w with d = setprec's Jacobi diagonal: a stand-in for the
 * reference's Schwarz-multigrid / FDM + coarse-grid preconditioner, which
 * this restatement does not have.  res: in the right-hand side, out the
 * solution.  tol: absolute on rnorm = |gamma| / sqrt(volvm1) (tol < 0:
 * relative to the initial one).  Returns the iteration count; *div0 and
 * *rnorm the first and last residual norms. */
int ref_gmres(const ref_ops *ops, double *res, const double *h1, const double *h2,
              const double *wt, const double *mask, double tol, int maxit, int m, int null_space,
              double *div0, double *rnorm);

/* hmh_flex_cg (hmholtz.f:2164-2289): the pressure solve's flexible
 * (Polak-Ribiere) preconditioned CG, param(42) = 2, on the same ax() and
 * weights as ref_gmres, with the same Jacobi stand-in for the reference's
 * multigrid preconditioner; ortho() on the result when null_space is set.
 * res: in the right-hand side, out the solution.  tol as ref_gmres.
 * Returns the iteration count. */
int ref_flex_cg(const ref_ops *ops, double *res, const double *h1, const double *h2,
                const double *wt, const double *mask, double tol, int maxit, int null_space,
                double *div0, double *rnorm);

/* local_grad3 (navier5.f:428) / local_grad3_t (navier1.f:4669), one element */
void ref_local_grad3(double *ur, double *us, double *ut, const double *u, int N,
                     const double *d, const double *dt);
void ref_local_grad3_t(double *u, const double *ur, const double *us, const double *ut,
                       int N, const double *d, const double *dt, double *w);

/* mxm (mxm_wrapper.f:1 -> mxf<n2>): c(n1,n3) = a(n1,n2) b(n2,n3) */
void ref_mxm(const double *a, int n1, const double *b, int n2, double *c, int n3);

/* threads actually used by the OpenMP loops (1 without OpenMP) */
int ref_max_threads(void);

/* ---- the pressure preconditioner h1mg_solve (h1mg.c; core/hsmg.f) ------- */
typedef struct ref_h1mg ref_h1mg;
/* x, y, z: fine GLL coordinates; fbc: 6 face types per element (r-, r+, s-,
 * s+, t-, t+; 0 shared, 1 Dirichlet, 2 Neumann); vertex: 8 vertex ids per
 * element (tensor corner order).  NULL when lx1 < 3 or the coarse matrix is
 * not positive definite. */
ref_h1mg *ref_h1mg_create(const ref_ops *ops, const double *x, const double *y, const double *z,
                          const int *fbc, const int64_t *vertex, int null_space);
void ref_h1mg_free(ref_h1mg *mg);
int ref_h1mg_levels(int lx1, int *order);
/* z = M rhs (h1mg_solve, if_hybrid = .false.); rhs is masked in place */
void ref_h1mg_solve(const ref_h1mg *mg, double *z, double *rhs);
int ref_h1mg_nlev(const ref_h1mg *mg);
int ref_h1mg_nx(const ref_h1mg *mg, int l);
int64_t ref_h1mg_ncoarse(const ref_h1mg *mg);
void ref_h1mg_level(const ref_h1mg *mg, int l, double *mask, double *rwt, double *swt);
void ref_h1mg_schwarz(const ref_h1mg *mg, int l, double *e, double *r);
void ref_h1mg_coarse(const ref_h1mg *mg, double *e, const double *r);
void ref_h1mg_lengths(const ref_h1mg *mg, double *out);
void ref_fdm1d(int n, int lbc, int rbc, double ll, double lm, double lr, double *s, double *lam);
/* hmh_gmres / hmh_flex_cg preconditioned by h1mg_solve */
int ref_gmres_h1mg(const ref_ops *ops, const ref_h1mg *mg, double *res, const double *h1,
                   const double *h2, const double *wt, const double *mask, double tol, int maxit,
                   int m, int null_space, double *div0_out, double *rnorm_out);
int ref_flex_cg_h1mg(const ref_ops *ops, const ref_h1mg *mg, double *res, const double *h1,
                     const double *h2, const double *wt, const double *mask, double tol,
                     int maxit, int null_space, double *div0_out, double *rnorm_out);

/* ---- gradient-type operators of the splitting step (gradops.c) --------- */
void ref_geom_rst(int nx1, int nel, const double *xm1, const double *ym1, const double *zm1,
                  double *g6, double *bm1, double *jacm1, double *rst);
void ref_wgradm1(int nx1, int nel, double *ux, double *uy, double *uz, const double *u,
                 const double *rst);
void ref_cdtp(int nx1, int nel, double *dtx, const double *x, const double *rst,
              const double *jac, const double *bm1, int isd);
void ref_dudxyz(int nx1, int nel, double *du, const double *u, const double *rst,
                const double *jac, int isd);
void ref_op_curl(const ref_ops *ops, double *w1, double *w2, double *w3, const double *u1,
                 const double *u2, const double *u3, int ifavg, const double *rst,
                 const double *jac, const double *bm1, const double *binv);

void ref_cresvsp(const ref_ops *ops, double *r1, double *r2, double *r3, const double *vx,
                 const double *vy, const double *vz, const double *h1, const double *h2,
                 const double *vdiff, const double *qtl, const double *pr, const double *bfx,
                 const double *bfy, const double *bfz, const double *rst);
void ref_cresvsp_weak(const ref_ops *ops, double *r1, double *r2, double *r3, const double *vx,
                      const double *vy, const double *vz, const double *h1, const double *h2,
                      const double *vdiff, const double *qtl, const double *pr,
                      const double *bfx, const double *bfy, const double *bfz,
                      const double *rst, const double *jac, const double *bm1, int stress);
void ref_axsf(const ref_ops *ops, double *au, double *av, double *aw, const double *u,
              const double *v, const double *w, const double *h1, const double *h2,
              const double *rst, const double *jac, const double *bm1);
int ref_hmhzsf(const ref_ops *ops, double *u1, double *u2, double *u3, double *r1, double *r2,
               double *r3, const double *h1, const double *h2, const double *m1,
               const double *m2, const double *m3, const double *mult, const double *binv,
               const double *rst, const double *jac, const double *bm1, double vol, double tin,
               double *rbn0, double *rbn2);
void ref_crespsp(const ref_ops *ops, double *respr, const double *vxe, const double *vye,
                 const double *vze, const double *pr, const double *qtl, const double *vdiff,
                 const double *vtrans, const double *bfx, const double *bfy, const double *bfz,
                 const double *bm1, const double *binv, double dtbd, int null_space,
                 const double *rst, const double *jac, const double *vx, const double *vy,
                 const double *vz, const int *fbc, const double *w);

void ref_conv1(int nx1, int nel, double *du, const double *u, const double *vx, const double *vy,
               const double *vz, const double *rst, const double *jac);
void ref_advab(int nx1, int nel, double *bfx, double *bfy, double *bfz, const double *vx,
               const double *vy, const double *vz, const double *bm1, const double *rst,
               const double *jac);

void ref_makeabf(int64_t n, double *bf, double *abx1, double *abx2, const double *vtrans,
                 const double *ab);
void ref_makebdf(int64_t n, double *bf, const double *v, const double *vlag, const double *bm1,
                 const double *vtrans, const double *bd, int nbd, double dt);
void ref_sumab(int64_t n, double *v, const double *vv, const double *vvlag, const double *ab,
               int nab);

void ref_convect_new(int nx1, int nel, int lxd, double *conv, const double *u, const double *vx,
                     const double *vy, const double *vz, const double *rst, const double *bm1);

void ref_convect_cons(int nx1, int nel, int lxd, double *conv, const double *u,
                      const double *vx, const double *vy, const double *vz, const double *rst,
                      const double *bm1);

void ref_conv2(int nx1, int nel, double *dtfi, const double *fi, const double *vx,
               const double *vy, const double *vz, const double *rst, const double *bm1);
void ref_convopo(int nx1, int nel, double *conv, const double *fi, const double *vx,
                 const double *vy, const double *vz, const double *rst, const double *jac,
                 const double *bm1, const int *ofc);

/* sizes of an operator state */
int ref_ops_nx1(const ref_ops *ops);
int ref_ops_nel(const ref_ops *ops);
int64_t ref_ops_n(const ref_ops *ops);

#ifdef __cplusplus
}
#endif
#endif
