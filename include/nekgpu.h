/*
 * nekgpu.h -- C ABI of the GB300 Helmholtz/Poisson solve path for Nek5000.
 *
 * Drop-in replacements for the reference's matrix-free Helmholtz operator
 * (axhelm), direct-stiffness sum (dssum -> gslib gs_op), Jacobi
 * preconditioner (setprec) and Jacobi-PCG solver (cggo / hmholtz).  Every
 * entry point takes its arguments by pointer, exactly as Fortran passes them,
 * so a Fortran caller binds them with ISO_C_BINDING `bind(C)` interfaces and
 * no name mangling; arrays are the reference's element-major layout
 * (lx1,ly1,lz1,nel), x fastest.  The caller keeps ownership of every array it
 * passes; the library copies what it needs.
 *
 * Status: every function returns 0 (NEKGPU_OK) or a negative NEKGPU_E* code;
 * nekgpu_last_error() gives the message.  Nothing calls exit() and no device
 * code traps.  A handle owns one CUDA stream on one device and is not
 * thread-safe; separate handles may be used concurrently.
 *
 * Unless a name ends in _dev, array arguments are HOST pointers and the call
 * moves them to and from the device inside the call.  The _dev variants take
 * device pointers (cudaMalloc'ed, or torch tensors' data_ptr) and copy
 * nothing; they run on the handle's stream and return when the work is
 * complete.
 *
 * Ordering with the caller's own GPU work: the handle's stream is created
 * non-blocking, so every call first makes it wait for all work already
 * queued on the legacy default stream (stream 0: torch's default stream,
 * cudaMemcpy, kernels launched without a stream), and every call waits for
 * the handle's stream before it returns.  Inputs written by such work are
 * therefore complete when the call's kernels read them, and outputs may be
 * read from any stream once the call has returned.  Work the caller queued
 * on a non-blocking stream of its own must be finished (or synchronized
 * with stream 0) before the call.
 */
#ifndef NEKGPU_H
#define NEKGPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NEKGPU_OK 0
#define NEKGPU_EINVAL (-1)    /* bad argument: N, nel, null pointer, size   */
#define NEKGPU_EHANDLE (-2)   /* unknown or finalized handle                */
#define NEKGPU_ECUDA (-3)     /* CUDA runtime error                         */
#define NEKGPU_ENOMEM (-4)    /* device allocation failed                   */
#define NEKGPU_ENOTCONV (-5)  /* PCG stopped at maxit without converging    */
#define NEKGPU_ENOSETUP (-6)  /* mesh / geometry not set up on the handle   */
#define NEKGPU_ENAN (-7)      /* non-finite value met in the solve          */

/* Largest polynomial order served (lx1 = N+1 <= NEKGPU_MAX_LX1). */
#define NEKGPU_MAX_LX1 12

/* Options for nekgpu_set_option */
#define NEKGPU_OPT_EXACT 1   /* 1: FP64 products and sums rounded one by one in the
                                reference's order (bit-faithful operator); 0: fused
                                multiply-adds (default)                           */
#define NEKGPU_OPT_TIMING 2  /* 1: time the solve and its operator kernels with
                                CUDA events (nekgpu_last_timing)                  */
#define NEKGPU_OPT_CHUNK 3   /* PCG iterations launched between host convergence
                                checks (default 16)                               */
#define NEKGPU_OPT_ISTEP 4   /* time-step index the reference's cggo sees; with
                                istep <= 5 the first iteration may already stop
                                (core/hmholtz.f:778)                              */
#define NEKGPU_OPT_TMA 5     /* 1 (default): stage element blocks with bulk async
                                copies where lx1 is even; 0: plain loads         */
#define NEKGPU_OPT_GRAPH 6   /* 1 (default): replay each chunk of PCG iterations
                                as one captured CUDA graph; 0: direct launches   */
#define NEKGPU_OPT_AUTOTUNE 8  /* 1 (default): on the first solve of a mesh in
                                a precision, time the operator's launch shapes
                                and keep the fastest (nekgpu_autotune); 0: the
                                built-in shapes.  Setting it forgets the picks. */
#define NEKGPU_OPT_SPLIT 9    /* mixed solve, residual-replacement mode: 1
                                keep the FP32 inner PCG's vectors once per
                                global node on element boundaries and once per
                                element inside (two kernels per iteration; even
                                lx1 >= 4 with the TMA operator); 0 (default)
                                the element-local form of the FP64 solver    */
#define NEKGPU_OPT_DF 10     /* 1: the FP64 operator (fused multiply-add form)
                                forms its tensor contractions in double-float
                                arithmetic -- pairs of FP32 values, 48
                                significant bits, compensated products and
                                sums -- on the FP32 pipe; FP64 in and out, the
                                mass term and the PCG's vector algebra in FP64.
                                0 (default): FP64 contractions            */
#define NEKGPU_OPT_FACE_ORDER 11  /* mixed solve, residual-replacement mode: 1
                                store each element's points of the FP32 inner
                                vectors face by face (face interiors, edges,
                                vertices, then the element interior), so that
                                the direct-stiffness sum reads and writes whole
                                memory sectors; 0 (default) the reference's
                                x-fastest order.  Results agree to FP32
                                rounding.                                    */
#define NEKGPU_OPT_COARSE 12  /* coarse solve of the pressure preconditioner
                                set up by the next nekgpu_h1mg_setup: 0
                                (default) the sparse X X^T factor (the
                                reference's param(40) = 0, crs_xxt); 1 algebraic
                                multigrid (param(40) = 1, crs_amg; see
                                nekgpu_crs_amg_setup)                        */
#define NEKGPU_OPT_MIXED_MODE 7  /* mixed solve: 1 (default) one FP32 PCG whose
                                residual is replaced by the FP64 one each time
                                it drops by inner_tol, search direction kept;
                                0 a fresh FP32 PCG per outer step               */

/* ---- life cycle ---------------------------------------------------------- */
/* Create a handle on CUDA device *device.  Replaces the per-rank setup the
 * reference does once in nek_init (core/drive1.f:2-178). */
int nekgpu_init(const int *device, int64_t *handle);
int nekgpu_finalize(int64_t *handle);
/* Copy the last error message (NUL-terminated, truncated to *buflen). */
int nekgpu_last_error(const int64_t *handle, char *buf, const int *buflen);

/* Set a handle option (NEKGPU_OPT_*). */
int nekgpu_set_option(const int64_t *handle, const int *key, const int *value);

/* ---- mesh data ----------------------------------------------------------- */
/* Upload the operator data the reference keeps in COMMON blocks and build the
 * gather-scatter maps:
 *   dxm1(lx1,lx1)            -- /DXYZ/ (core/DXYZ, genwz core/coef.f:1-355)
 *   g1..g6(lx1^3*nel)        -- /GMFACT/ g1m1..g6m1 (core/GEOM, geodat1 core/coef.f:633-784)
 *   bm1(lx1^3*nel)           -- /MASS/ bm1 (core/MASS)
 *   glo_num(lx1^3*nel)       -- global ids from set_vert (core/navier8.f:3-33);
 *                               0 = not shared (element interior)
 * Replaces setupds -> fgslib_gs_setup (core/dssum.f:1-31) plus the geometry
 * COMMON-block setup.  Any earlier mesh on the handle is released. */
int nekgpu_setup(const int64_t *handle, const int *lx1, const int *nel, const double *dxm1,
                 const double *g1, const double *g2, const double *g3, const double *g4,
                 const double *g5, const double *g6, const double *bm1, const int64_t *glo_num);

/* The pressure solve's Krylov method: hmh_gmres (core/gmres.f:304-560),
 * right-preconditioned restarted GMRES with restart length *kmax (the
 * reference's lgmres, 30; at most NEKGPU_GMRES_MAX) on
 * A x = mask * dssum(axhelm(x, h1, h2)) (gmres.f:284-302), inner products
 * weighted by wt (vmult), classical Gram-Schmidt, Givens rotations.  res
 * (device array): in the right-hand side, out the solution.  Stops when
 * rnorm = |gamma| / sqrt(volvm1) < *tol (absolute; *tol < 0: relative to the
 * initial rnorm, as param(21) < 0) or after *maxit iterations (status
 * NEKGPU_ENOTCONV above the tolerance).  *null_space != 0 removes the mean
 * of every preconditioned vector and of the solution (ortho,
 * core/navier1.f:223-256), for a pure-Neumann pressure (ifvcor).  The
 * preconditioner is the Jacobi diagonal (setprec), standing in for the
 * reference's Schwarz-multigrid / FDM + coarse-grid one: iteration counts are
 * this method's; the solution is the same system's to the tolerance.
 * Outputs: iterations, initial and final rnorm. */
#define NEKGPU_GMRES_MAX 50
int nekgpu_hmh_gmres_dev(const int64_t *handle, double *res, const double *h1, const double *h2,
                         const double *wt, const double *mask, const double *tol,
                         const int *maxit, const int *kmax, const int *null_space, int *niter,
                         double *div0, double *rnorm);
/* The pressure solve's other Krylov method, hmh_flex_cg (core/hmholtz.f:
 * 2164-2289, param(42) = 2): flexible (Polak-Ribiere) preconditioned CG on
 * the same operator, weights, stopping test, null-space handling and Jacobi
 * stand-in preconditioner as nekgpu_hmh_gmres_dev.  A zero right-hand side
 * returns x = 0 after no iteration. */
int nekgpu_hmh_flex_cg_dev(const int64_t *handle, double *res, const double *h1,
                           const double *h2, const double *wt, const double *mask,
                           const double *tol, const int *maxit, const int *null_space,
                           int *niter, double *div0, double *rnorm);
int nekgpu_hmh_flex_cg(const int64_t *handle, double *res, const double *h1, const double *h2,
                       const double *wt, const double *mask, const double *tol, const int *maxit,
                       const int *null_space, int *niter, double *div0, double *rnorm);
/* The pressure preconditioner h1mg_solve (core/hsmg.f:1855-1949, with
 * if_hybrid = .false. as hmh_gmres and hmh_flex_cg call it; setup h1mg_setup
 * :2234-2270 and set_up_h1_crs, core/navier8.f:83-238): additive multilevel
 * overlapping Schwarz on polynomial orders N, min(3, ...) and 1, with
 * fast-diagonalisation local solves on elements extended by one layer and
 * a Galerkin coarse solve on the vertices (exact: A^-1 = X X^T with X sparse
 * in nested-dissection order, as crs_xxt factors it).  Host arrays: x, y, z the GLL coordinates
 * (xm1, ym1, zm1), glo_num the numbering given to nekgpu_setup, and either
 * fbc (6 face types per element, r-, r+, s-, s+, t-, t+: 0 interior or
 * periodic, 1 Dirichlet ('O'), 2 Neumann (wall); get_fast_bc,
 * core/fast3d.f:802) or, with fbc null, the pressure mask they are read
 * from (nekmesh_face_types).  *null_space != 0 when the pressure has a null
 * space (no outflow): the coarse solve pins one vertex and removes the mean.
 * Once set up, nekgpu_hmh_gmres(_dev) and nekgpu_hmh_flex_cg(_dev) use it
 * instead of the Jacobi diagonal; nekgpu_h1mg_free returns to Jacobi; a new
 * mesh drops it.  3 <= lx1 <= 12. */
int nekgpu_h1mg_setup(const int64_t *handle, const double *x, const double *y, const double *z,
                      const double *mask, const int64_t *glo_num, const int *fbc,
                      const int *null_space);
int nekgpu_h1mg_free(const int64_t *handle);
/* z = M rhs on device arrays; rhs is masked in place, as h1mg_solve leaves it. */
int nekgpu_h1mg_apply_dev(const int64_t *handle, double *z, double *rhs);

/* The coarse solve of the reference's crs_amg interface on a handle:
 * crs_amg_setup (core/crs_amg.c:531: n unknowns, nz matrix entries in
 * coordinate form ai, aj, av -- zero-based, duplicates summed -- and the
 * null-space flag) and crs_amg_solve (:186: x = one AMG V-cycle applied to
 * b, device arrays of n; with the null space the last unknown is pinned to 0
 * during the cycle and the mean of x is removed afterwards, as crs_solve
 * does).  The hierarchy is built on the host by the setup nekmesh_amg_setup
 * describes (the reference reads it from files its setup tool writes). */
int nekgpu_crs_amg_setup(const int64_t *handle, const int64_t *n, const int64_t *nz,
                         const int *ai, const int *aj, const double *av, const int *null_space);
int nekgpu_crs_amg_solve_dev(const int64_t *handle, double *x, const double *b);
/* ---- gradient-type operators of the splitting step (plan4) --------------
 * On device arrays of the handle's n points, in the reference's arithmetic
 * order (bit-identical to its unfused FP64 evaluation).  They need the metric
 * terms rxm1..tzm1 and jacm1, which the library keeps when the geometry comes
 * from coordinates (nekgpu_setup_xyz, nekgpu_geom_update_dev); NEKGPU_ENOSETUP
 * otherwise.  isd = 1, 2, 3 selects x, y, z.
 *   wgradm1  u_x,y,z = w3m1 (u_r r_x + u_s s_x + u_t t_x), ...
 *            (opgrad for PN-PN, core/navier1.f:4170)
 *   dudxyz   du = (u_r r_isd + u_s s_isd + u_t t_isd) / jacm1 (:1156)
 *   cdtp     dtx = D^T (bm1 x / jacm1 times r_isd, s_isd, t_isd) (:330)
 *   op_curl  w = curl u from dudxyz; with *ifavg != 0 averaged as
 *            w = binv dssum(bm1 w) (core/plan4.f:368-430) */
int nekgpu_wgradm1_dev(const int64_t *handle, double *ux, double *uy, double *uz,
                       const double *u);
int nekgpu_dudxyz_dev(const int64_t *handle, double *du, const double *u, const int *isd);
int nekgpu_cdtp_dev(const int64_t *handle, double *dtx, const double *x, const int *isd);
int nekgpu_op_curl_dev(const int64_t *handle, double *w1, double *w2, double *w3,
                       const double *u1, const double *u2, const double *u3, const int *ifavg,
                       const double *binv);
/* The convective term with dealiasing (convop with param(99) = 4,
 * core/navier1.f:3196 -> convect_new, core/convect.f:639): after
 * nekgpu_dealias_setup(lxd) (lx1 <= lxd <= 18, typically 3 lx1 / 2) the
 * field and velocity are interpolated to lxd Gauss points per direction,
 * the product formed there with the Gauss-weighted metric terms, projected
 * back and divided by bm1.  nekgpu_convop_dev is convop: dealiased once set
 * up, conv1 otherwise; nekgpu_advab_dev follows the same choice.  Agrees
 * with the reference to rounding (not bit for bit).  A moved geometry
 * (nekgpu_geom_update_dev) rebuilds the fine metric terms. */
int nekgpu_dealias_setup(const int64_t *handle, const int *lxd);
int nekgpu_convop_dev(const int64_t *handle, double *conv, const double *u, const double *vx,
                      const double *vy, const double *vz);
/* conv2 (core/navier1.f:1288): dtfi = D^T (w3 (rst v) fi) / bm1, the
 * transposed (weak) convective operator; and the skew-symmetric form
 * (convopo with param(86) != 0, :1221): conv1 and conv2 of fi masked by
 * cmask (:1390), whose ofc flags (host, 6 per element, preprocessor face
 * order; null for none) mark the outflow ('O', 'o') faces.  Bit-identical to
 * the reference's unfused FP64 arithmetic. */
int nekgpu_conv2_dev(const int64_t *handle, double *dtfi, const double *fi, const double *vx,
                     const double *vy, const double *vz);
int nekgpu_convopo_dev(const int64_t *handle, double *conv, const double *fi, const double *vx,
                       const double *vy, const double *vz, const int *ofc);
/* The conservative form on the same Gauss grid (convop with param(99) = 5,
 * convect_cons, core/convect.f:729): conv = div(v u) in weak form / bm1;
 * needs nekgpu_dealias_setup. */
int nekgpu_convect_cons_dev(const int64_t *handle, double *conv, const double *u,
                            const double *vx, const double *vy, const double *vz);
/* The convective term without dealiasing (conv1, core/navier1.f:3276; what
 * convop uses when dealiasing is off): du = (v . grad) u, and advab
 * (:1516): bf_c -= bm1 (v . grad) v_c for the three components. */
int nekgpu_conv1_dev(const int64_t *handle, double *du, const double *u, const double *vx,
                     const double *vy, const double *vz);
int nekgpu_advab_dev(const int64_t *handle, double *bfx, double *bfy, double *bfz,
                     const double *vx, const double *vy, const double *vz);

/* The splitting step's explicit right-hand sides (plan4, core/plan4.f), on
 * device arrays, PN-PN without the stress formulation.  Same setup needs as
 * the operators above; with NEKGPU_OPT_EXACT set they are the reference's
 * unfused FP64 values bit for bit.
 *   cresvsp  (:264-306) r = -A(h1, h2) v - opgrad(pr - vdiff qtl / 3) + bf
 *   crespsp  (:99-260)  the pressure right-hand side (curl curl of the
 *            extrapolated velocity, opgrad qtl, A(1/vtrans, 0) pr, the
 *            forcing, qtl bm1 bd(1)/dt, the face terms; the mean removed when
 *            *null_space).  fbc (host, 6 per element in the preprocessor
 *            face order of cbc; may be null for none): 0 no face term, 1
 *            'V', 'v', 'MV', 'mv' (the current velocity vx, vy, vz through
 *            the face, times bd(1)/dt), 2 'shl' (the same, unscaled), 3
 *            'SYM'. */
int nekgpu_cresvsp_dev(const int64_t *handle, double *r1, double *r2, double *r3,
                       const double *vx, const double *vy, const double *vz, const double *h1,
                       const double *h2, const double *vdiff, const double *qtl,
                       const double *pr, const double *bfx, const double *bfy,
                       const double *bfz);
/* cresvsp_weak (core/plan4.f:308-361), the velocity residual of plan4's
 * stress-formulation branch (:84-86, ifstrs and not ifaxis):
 *   r = -A(h1, h2) v - (opgrad(scale vdiff qtl) - cdtp(pr)) + bf
 * per component, the pressure through its weak gradient (cdtp per
 * direction with the mesh's mass and metric terms), scale = 2/3 when
 * *stress, else -1/3.  Same setup needs and exact-mode behaviour as
 * nekgpu_cresvsp_dev.  The traction boundary terms that the reference adds
 * before it (bcneutr) and the coupled stress operator the velocity solve
 * then uses (ophinv with ifstrs) are not part of this library. */
int nekgpu_cresvsp_weak_dev(const int64_t *handle, double *r1, double *r2, double *r3,
                            const double *vx, const double *vy, const double *vz,
                            const double *h1, const double *h2, const double *vdiff,
                            const double *qtl, const double *pr, const double *bfx,
                            const double *bfy, const double *bfz, const int *stress);
/* The stress formulation's coupled velocity operator and solve (device
 * arrays; FP64, products and sums rounded in the reference's order; the
 * geometry must come from coordinates, nekgpu_setup_xyz):
 *   axhmsf  core/subs1.f:1240-1315 for a fluid (matmod = 0) in 3-D, its
 *           default path axsf_e_3d (:2031-2116):
 *           au_i = sum_j D^T (h1 w3 / J) (du_i/dx_j + du_j/dx_i) + h2 B u_i
 *   hmhzsf  core/subs1.f:1093-1147 without the projection onto previous
 *           solutions (param(94) = 0): r masked by m1, m2, m3 (the volume
 *           masks of rmask) and dssum'ed in place, u = 0, chktcgs's
 *           tolerance floor, then cggosf (:2-165): Jacobi-PCG on the coupled
 *           system, preconditioned by the sum of the three setprec
 *           diagonals, at most 200 iterations (the reference fixes that cap;
 *           NEKGPU_ENOTCONV when reached).  *tol: absolute tolerance on
 *           sqrt(sum binv mult |r|^2 / vol).  The face, edge and corner
 *           masks of qmask (symmetry and other mixed conditions) are not
 *           applied. */
int nekgpu_axhmsf_dev(const int64_t *handle, double *au1, double *au2, double *au3,
                      const double *u1, const double *u2, const double *u3, const double *h1,
                      const double *h2);
int nekgpu_hmhzsf_dev(const int64_t *handle, double *u1, double *u2, double *u3, double *r1,
                      double *r2, double *r3, const double *h1, const double *h2,
                      const double *m1, const double *m2, const double *m3, const double *mult,
                      const double *binv, const double *tol, int *niter, double *rbn0,
                      double *rbn2);
int nekgpu_crespsp_dev(const int64_t *handle, double *respr, const double *vxe,
                       const double *vye, const double *vze, const double *pr,
                       const double *qtl, const double *vdiff, const double *vtrans,
                       const double *bfx, const double *bfy, const double *bfz,
                       const double *binv, const double *dtbd, const int *null_space,
                       const double *vx, const double *vy, const double *vz, const int *fbc);

/* The step's time-integration bookkeeping, one velocity component per call
 * (fixed geometry, constant-density flow):
 *   makeabf (core/navier1.f:1597) extrapolated forcing: ta = ab1 abx1 +
 *           ab2 abx2; abx2 = abx1; abx1 = bf; bf = (ab0 bf + ta) vtrans
 *           (ab: the 3 coefficients of setab3)
 *   makebdf (:1548) bf += (v bm1 bd(2) + sum over the lags of vlag bm1
 *           bd(l+1)) vtrans / dt; bd: nbd + 1 coefficients (1 <= nbd <= 3);
 *           vlag: nbd - 1 lagged fields of n, back to back
 *   sumab   (core/plan4.f:525) v = ab0 vv + ab1 vvlag_1 (+ ab2 vvlag_2 when
 *           nab = 3); vvlag: the lagged fields back to back */
int nekgpu_makeabf_dev(const int64_t *handle, double *bf, double *abx1, double *abx2,
                       const double *vtrans, const double *ab);
int nekgpu_makebdf_dev(const int64_t *handle, double *bf, const double *v, const double *vlag,
                       const double *vtrans, const double *bd, const int *nbd,
                       const double *dt);
int nekgpu_sumab_dev(const int64_t *handle, double *v, const double *vv, const double *vvlag,
                     const double *ab, const int *nab);

/* ---- a solve split over element shards ----------------------------------
 * The reference splits the mesh over MPI ranks; each rank's solve runs its
 * local operator and gather-scatter, exchanges the sums at the points it
 * shares with other ranks (inside gs_op), and adds its local dot products
 * over the ranks (gop, core/comm_mpi.f:216).  These device entry points are
 * the local pieces a caller's loop needs between its own exchanges (MPI,
 * NCCL or torch.distributed); all arrays are the handle's n local points.
 *   col2   a = a b           (core/math.f:563)
 *   col3   a = b c           (core/math.f:597)
 *   add2s1 a = c1 a + b      (core/math.f:677)
 *   add2s2 a = a + c2 b      (core/math.f:689)
 *   vlsc3  *out = local sum of a b c        (core/navier4.f:323)
 *   vlsc32 *out = local sum of b c a^2      (core/hmholtz.f:848)
 *   invcol1 a = 1/a          (core/math.f:61)
 *   vlmax  *out = local max |a| (*mode 0), max a (1) or min a (2) */
int nekgpu_col2_dev(const int64_t *handle, double *a, const double *b);
int nekgpu_col3_dev(const int64_t *handle, double *a, const double *b, const double *c);
int nekgpu_add2s1_dev(const int64_t *handle, double *a, const double *b, const double *c1);
int nekgpu_add2s2_dev(const int64_t *handle, double *a, const double *b, const double *c2);
int nekgpu_vlsc3_dev(const int64_t *handle, const double *a, const double *b, const double *c,
                     double *out);
int nekgpu_vlsc32_dev(const int64_t *handle, const double *a, const double *b, const double *c,
                      double *out);
int nekgpu_invcol1_dev(const int64_t *handle, double *a);
int nekgpu_vlmax_dev(const int64_t *handle, const double *a, const int *mode, double *out);
/* setprec's element-local diagonal (core/hmholtz.f:380-524 before its dssum
 * and reciprocal): a shard sums it locally (nekgpu_dssum_dev), across its
 * interfaces, then inverts. */
int nekgpu_setprec_local_dev(const int64_t *handle, double *diag, const double *h1,
                             const double *h2);
/* Interface points shared with other shards: point k has the local copies
 * pos[start[k] .. start[k+1]-1] (host arrays, start has nk+1 entries).
 * gather: buf[k] = u at point k's first copy (after the local dssum all
 * copies agree); scatter: every copy of point k = buf[k]. */
int nekgpu_iface_setup(const int64_t *handle, const int64_t *nk, const int64_t *start,
                       const int64_t *pos);
int nekgpu_iface_gather_dev(const int64_t *handle, double *buf, const double *u);
int nekgpu_iface_scatter_dev(const int64_t *handle, double *u, const double *buf);

/* The same on host arrays (copied in and out inside the call). */
int nekgpu_hmh_gmres(const int64_t *handle, double *res, const double *h1, const double *h2,
                     const double *wt, const double *mask, const double *tol, const int *maxit,
                     const int *kmax, const int *null_space, int *niter, double *div0,
                     double *rnorm);

/* As nekgpu_setup, with the geometric factors and the mass computed on the
 * device from the GLL coordinates xm1, ym1, zm1 (host arrays, lx1^3 nel
 * each) and the GLL weights wxm1 (lx1): xyzrst (core/coef.f:879-926), glmapm1
 * (:555-631) and geodat1 (:633-784), with W3M1 = w(i) w(j) w(k); products,
 * sums and 1/J rounded one by one in the reference's order, so G1..G6 and
 * bm1 are the reference's bit for bit.  NEKGPU_EINVAL when a Jacobian is not
 * positive. */
int nekgpu_setup_xyz(const int64_t *handle, const int *lx1, const int *nel, const double *dxm1,
                     const double *wxm1, const double *xm1, const double *ym1, const double *zm1,
                     const int64_t *glo_num);
/* A moved mesh (same numbering): G1..G6, bm1 and volvm1 recomputed from new
 * device coordinates, as the reference's geom_reset does each step of a
 * moving-boundary run (geom_reset, core/ic.f:1824, -> geom1, core/coef.f:360).
 * On NEKGPU_EINVAL (a Jacobian not positive) the refused geometry is left in
 * place: pass valid coordinates before the next solve. */
int nekgpu_geom_update_dev(const int64_t *handle, const double *wxm1, const double *xm1,
                           const double *ym1, const double *zm1);
/* The geometry in use, copied to host arrays (lx1^3 nel each; any may be
 * null). */
int nekgpu_geometry(const int64_t *handle, double *g1, double *g2, double *g3, double *g4,
                    double *g5, double *g6, double *bm1);
/* Number of shared groups and of local copies in them (gs_setup's maps);
 * with non-null outputs, copies the CSR maps: seg_start[nseg+1], idx[nidx]
 * (0-based local indices, ascending inside a group, groups by ascending id). */
int nekgpu_gs_maps(const int64_t *handle, int64_t *nseg, int64_t *nidx, int64_t *seg_start,
                   int64_t *idx);

/* ---- operator ------------------------------------------------------------ */
/* au = h1 * A u + h2 * B u  (core/hmholtz.f:72-259, 3-D deformed path).
 * imesh / isd are accepted for signature parity (imesh selects nelv/nelt in
 * the reference; one element count is served here; isd only matters for the
 * axisymmetric branch, which is not served). */
int nekgpu_axhelm(const int64_t *handle, double *au, const double *u, const double *h1,
                  const double *h2, const int *imesh, const int *isd);
int nekgpu_axhelm_dev(const int64_t *handle, double *au, const double *u, const double *h1,
                      const double *h2, const int *imesh, const int *isd);

/* u <- dssum(u): sum of all local copies of every shared node, written back
 * to each copy (core/dssum.f:33-98 -> fgslib_gs_op(gsh,u,1,1,0)). */
int nekgpu_dssum(const int64_t *handle, double *u);
int nekgpu_dssum_dev(const int64_t *handle, double *u);
/* gs_op with op '+', '*', 'M' (max) or 'm' (min)  (core/dssum.f:100-160 dsop) */
int nekgpu_dsop_dev(const int64_t *handle, double *u, const char *op);

/* d = 1 / dssum(diag approx of h1*A + h2*B)  (core/hmholtz.f:380-524) */
int nekgpu_setprec(const int64_t *handle, double *d, const double *h1, const double *h2,
                   const int *imsh, const int *isd);
int nekgpu_setprec_dev(const int64_t *handle, double *d, const double *h1, const double *h2,
                       const int *imsh, const int *isd);

/* ---- Jacobi-PCG ---------------------------------------------------------- */
/* cggo (core/hmholtz.f:611-846): x solves H x = f with H = h1 A + h2 B,
 * Jacobi preconditioner, masked by mask, dot products weighted by mult,
 * residual norm sqrt(sum r^2 mult binv / vol).  tin < 0 means relative
 * tolerance |tin| * (iteration-1 norm).  The reference's hard cap of 900
 * iterations (maxcg) is applied when *maxcg is NULL; pass a pointer to lift
 * it.  Outputs: *niter, *rbn0 (first norm), *rbn2 (last norm).  Returns
 * NEKGPU_ENOTCONV (with x = the last iterate) when the cap is reached. */
int nekgpu_cggo(const int64_t *handle, double *x, const double *f, const double *h1,
                const double *h2, const double *mask, const double *mult, const int *imsh,
                const double *tin, const int *maxit, const int *isd, const double *binv,
                const int *maxcg, int *niter, double *rbn0, double *rbn2);
int nekgpu_cggo_dev(const int64_t *handle, double *x, const double *f, const double *h1,
                    const double *h2, const double *mask, const double *mult, const int *imsh,
                    const double *tin, const int *maxit, const int *isd, const double *binv,
                    const int *maxcg, int *niter, double *rbn0, double *rbn2);

/* hmholtz (core/hmholtz.f:2-69): rhs <- mask * dssum(rhs) (in place, as the
 * reference does), tolerance guard chktcg1 (:527-609), then cggo. */
int nekgpu_hmholtz(const int64_t *handle, double *u, double *rhs, const double *h1,
                   const double *h2, const double *mask, const double *mult, const int *imsh,
                   const double *tli, const int *maxit, const int *isd, const double *binv,
                   const int *maxcg, int *niter, double *rbn0, double *rbn2);
int nekgpu_hmholtz_dev(const int64_t *handle, double *u, double *rhs, const double *h1,
                       const double *h2, const double *mask, const double *mult,
                       const int *imsh, const double *tli, const int *maxit, const int *isd,
                       const double *binv, const int *maxcg, int *niter, double *rbn0,
                       double *rbn2);

/* Allocation-free operator.  No counterpart in the reference: it exists for
 * callers that cannot let a library allocate device memory -- a code that
 * has given all device memory to its own pool allocator, one that runs under
 * a hard memory budget, or a time-step loop that must not pay for the
 * device-wide synchronisation cudaMalloc brings.  Same arguments and result
 * as nekgpu_axhelm_dev (device arrays); it keeps the partial results of its
 * h1/h2 scan in one fixed array of NEKGPU_NOALLOC_MAX_POINTS / 2048 * 4
 * doubles (64 KiB) that every GPU loading this library holds until the
 * process exits, and makes no device allocation itself.  Meshes of more than
 * NEKGPU_NOALLOC_MAX_POINTS local points are rejected with NEKGPU_EINVAL.
 * Like every call here it waits for its own kernels before it returns.  The
 * first call on a device also looks up that array's device address (with
 * the device current); make that first call before any stream capture.
 * Calls share the array: calls that overlap on the GPU (from several threads
 * or handles at once) race on it; each call writes every slot it reads, so
 * nothing needs clearing between calls.  With NEKGPU_OPT_TIMING on it
 * records the scan and the operator together, as nekgpu_axhelm_dev does. */
#define NEKGPU_NOALLOC_MAX_POINTS 4194304
int nekgpu_axhelm_dev_noalloc(const int64_t *handle, double *au, const double *u,
                              const double *h1, const double *h2, const int *imesh,
                              const int *isd);

/* ---- mixed precision --------------------------------------------------- */
/* Same system and FP64 stopping rule as cggo, solved by FP64 defect
 * correction around an FP32 Jacobi-PCG (G, D, fields, diagonal stored FP32).
 * Each time the FP32 residual has dropped by *inner_tol, the FP32 correction
 * is added to x in FP64 and r = f - A x is recomputed with the FP64 operator.
 * NEKGPU_OPT_MIXED_MODE 1 (default) puts that r back into the running FP32
 * PCG and keeps its search direction (default *inner_tol 1e-2 when NULL);
 * mode 0 starts a fresh FP32 PCG on it (default *inner_tol 1e-5).  Stops when
 * the FP64 norm sqrt(sum r^2 mult binv / vol) reaches |tin| (tin >= 0) or
 * |tin| * its initial value (tin < 0).  *maxit caps the FP32 iterations (of
 * the whole solve in mode 1, of each inner solve in mode 0).  Outputs: outer
 * steps (FP64 residual evaluations), total inner iterations, first and last
 * FP64 norms.  No reference counterpart: it replaces cggo
 * (core/hmholtz.f:611) for callers that accept FP32 inner arithmetic. */
int nekgpu_cggo_mixed_dev(const int64_t *handle, double *x, const double *f, const double *h1,
                          const double *h2, const double *mask, const double *mult,
                          const int *imsh, const double *tin, const int *maxit, const int *isd,
                          const double *binv, const double *inner_tol, int *niter_outer,
                          int *niter_inner, double *rbn0, double *rbn2);
/* Several fields of one mesh that share h1, h2, mult and binv -- the velocity
 * components of a time step, which the reference solves one after another
 * (ophinv, core/induct.f:1064-1071) -- solved together by the mixed solve
 * (residual replacement): per field x, f (device arrays, as
 * nekgpu_cggo_mixed_dev) and mask; *nfield <= NEKGPU_MULTI_MAX.  Every FP32
 * iteration of all fields is one operator launch that reads the geometric
 * factors once, one boundary-group launch and one update launch; each field
 * keeps its own scalars and stopping test.  Outputs per field: outer steps,
 * inner iterations, first and last FP64 norms and a status code (0,
 * NEKGPU_ENOTCONV, NEKGPU_ENAN, NEKGPU_EINVAL for a singular system).  Odd
 * lx1 solves the fields one after another.  No reference counterpart. */
#define NEKGPU_MULTI_MAX 3
int nekgpu_cggo_mixed_multi_dev(const int64_t *handle, const int *nfield, double *const *x,
                                const double *const *f, const double *h1, const double *h2,
                                const double *const *mask, const double *mult, const int *imsh,
                                const double *tin, const int *maxit, const int *isd,
                                const double *binv, const double *inner_tol, int *niter_outer,
                                int *niter_inner, double *rbn0, double *rbn2, int *status);
/* hmholtz (core/hmholtz.f:2-69) with the mixed-precision solve, host arrays. */
int nekgpu_hmholtz_mixed(const int64_t *handle, double *u, double *rhs, const double *h1,
                         const double *h2, const double *mask, const double *mult,
                         const int *imsh, const double *tli, const int *maxit, const int *isd,
                         const double *binv, const double *inner_tol, int *niter_outer,
                         int *niter_inner, double *rbn0, double *rbn2);

/* ---- adjoint with respect to the viscosity h1 -------------------------- */
/* gh1[p] = d(lam^T A(h1) u)/d h1[p] = (grad lam)_p . (G_p grad u)_p for every
 * local point p (A is linear in h1; grad is the reference-element gradient
 * and G_p the geometric factors of core/coef.f:633-784).  For J(u) with
 * A(h1) u = f and adjoint A lam = dJ/du, dJ/dh1 = -gh1.  No reference
 * counterpart (the reference's adjoint, core/perturb.f, is the adjoint
 * Navier-Stokes equation, not a derivative of axhelm). */
int nekgpu_axhelm_adjoint_h1(const int64_t *handle, double *gh1, const double *lam,
                             const double *u);
int nekgpu_axhelm_adjoint_h1_dev(const int64_t *handle, double *gh1, const double *lam,
                                 const double *u);
/* Adjoint solve A lam = g: the operator is symmetric, so this is cggo
 * (core/hmholtz.f:611) with the same arguments; provided as its own entry
 * point so adjoint code reads as such. */
int nekgpu_cggo_adjoint_dev(const int64_t *handle, double *lam, const double *g,
                            const double *h1, const double *h2, const double *mask,
                            const double *mult, const int *imsh, const double *tin,
                            const int *maxit, const int *isd, const double *binv,
                            const int *maxcg, int *niter, double *rbn0, double *rbn2);

/* ---- batched solves ---------------------------------------------------- */
/* Many independent problems (each its own mesh, order and size) solved
 * together: every PCG phase is one launch over all problems, iterations are
 * replayed as captured CUDA graphs, and every problem stops at its own
 * convergence test.  No reference counterpart: the reference solves one
 * field per hmholtz call (velocity components one after another,
 * core/induct.f:1064-1071); this runs such solves, and unrelated problems,
 * side by side on one GPU. */
int nekgpu_batch_create(const int *device, int64_t *batch);
/* Add one problem's mesh (arguments as nekgpu_setup); *index receives its slot. */
int nekgpu_batch_add(const int64_t *batch, const int *lx1, const int *nel, const double *dxm1,
                     const double *g1, const double *g2, const double *g3, const double *g4,
                     const double *g5, const double *g6, const double *bm1,
                     const int64_t *glo_num, int *index);
/* Solve all problems (device arrays, one pointer per problem, in slot order).
 * Per problem: the same inputs and stopping rule as nekgpu_cggo_dev (tin < 0
 * relative; no 900 cap: *maxit iterations at most).  *mixed selects the
 * FP32-inner / FP64-defect-correction form: 1 with residual replacement into
 * each problem's running FP32 PCG (default *inner_tol 1e-2 when NULL), 2
 * restarted per outer step (default *inner_tol 1e-5); 0 is plain FP64.
 * Outputs per problem: niter (PCG iterations; total inner iterations when
 * mixed), nouter (outer steps, mixed only; may be NULL), rbn0, rbn2 and a
 * status code (0, NEKGPU_ENOTCONV, NEKGPU_ENAN, ...). */
int nekgpu_batch_solve_dev(const int64_t *batch, const int *nprob, double *const *x,
                           const double *const *f, const double *const *h1,
                           const double *const *h2, const double *const *mask,
                           const double *const *mult, const double *const *binv,
                           const double *tin, const int *maxit, const int *mixed,
                           const double *inner_tol, int *niter, int *nouter, double *rbn0,
                           double *rbn2, int *status);
/* Operator block size of the batched solve in precision 0 (FP64) or 1 (FP32):
 * picked by timing 128- and 256-thread blocks on the first solve of a problem
 * set (every size gives identical results), or pinned with
 * nekgpu_batch_set_shape (*threads 128 or 256; 0 returns to tuning).
 * *threads = 0 before the first solve; *ms is the tuned launch time.  No
 * reference counterpart.  A 128-thread block is a candidate only when every
 * problem's lx1^2 <= 128. */
int nekgpu_batch_shape(const int64_t *batch, const int *precision, int *threads, double *ms);
/* *on = 1: each batch segment -- the iterations until every
 * problem has stopped, or until every problem's FP32 residual has dropped by
 * inner_tol in the mixed form -- is one persistent cooperative launch whose
 * resident blocks run the operator, boundary-group and update phases of all
 * problems with grid-wide barriers between them (bounded waits: a barrier
 * that does not complete within seconds fails the solve with NEKGPU_ECUDA
 * and leaves the GPU usable).  Its block size is 256 threads.  *on = 0
 * (default): per iteration one operator launch per polynomial order present
 * (FP32: the TMA-staged body where it applies and times faster) plus the
 * boundary-group and update launches, replayed as a captured CUDA graph, with
 * the plain operator's block size tuned as nekgpu_batch_shape says.  Both
 * forms give results within the FP64 tolerance of each other (FP64 solves:
 * identical).  No reference counterpart. */
int nekgpu_batch_set_persistent(const int64_t *batch, const int *on);
int nekgpu_batch_set_shape(const int64_t *batch, const int *precision, const int *threads);
/* The FP32 operator body each polynomial order runs in the batch:
 * forms[lx1] (NEKGPU_MAX_LX1 + 1 entries) is 1 for the TMA-staged body, 0
 * for the plain one, -1 where no order lx1 has been timed yet (the first
 * mixed solve times every order present where the TMA body applies, and the
 * verdict stays for the batch).  No reference counterpart. */
int nekgpu_batch_operator_forms(const int64_t *batch, int *forms);
int nekgpu_batch_last_error(const int64_t *batch, char *buf, const int *buflen);
int nekgpu_batch_destroy(int64_t *batch);

/* ---- projection onto previous solutions (core/navier4.f:562-1188) --------- */
/* hsolve with projection (navier4.f:562, the ifstdh = .false. branch): the
 * right-hand side r is masked by vmk and dssum'ed in place, its part in the
 * span of the space's stored B = A X is removed (project1, :636), the rest is
 * solved as hmhzpf does (:513: chktcg1 on tli, then cggo with that tolerance;
 * param(22) is the caller's business), and the solution u gets the matching
 * part of span(X) back and joins the space (project2, :1129; proj_ortho,
 * :852).  A change of h1 or h2 since the space was built triggers B = A X
 * and a full re-orthonormalisation (iproj_chk :788, proj_ortho_full_cgs2
 * :1060).  The space lives on the device inside the handle, selected by
 * *space (0 <= *space < NEKGPU_PROJ_SPACES; the reference's per-field approx
 * / napprox arrays); it holds at most mmx vectors (default
 * NEKGPU_PROJ_DEFAULT = (mxprev - 4) / 2 with the reference's mxprev = 20).
 * Outputs as nekgpu_cggo_dev plus *m (vectors in the space afterwards). */
#define NEKGPU_PROJ_SPACES 16
#define NEKGPU_PROJ_MAX 16
#define NEKGPU_PROJ_DEFAULT 8
int nekgpu_hsolve_dev(const int64_t *handle, const int *space, double *u, double *r,
                      const double *h1, const double *h2, const double *vmk, const double *vml,
                      const int *imsh, const double *tli, const int *maxit, const int *isd,
                      const double *bi, const int *maxcg, int *niter, double *rbn0,
                      double *rbn2, int *m);
/* The same with host arrays (u out, r in/out). */
int nekgpu_hsolve(const int64_t *handle, const int *space, double *u, double *r,
                  const double *h1, const double *h2, const double *vmk, const double *vml,
                  const int *imsh, const double *tli, const int *maxit, const int *isd,
                  const double *bi, const int *maxcg, int *niter, double *rbn0, double *rbn2,
                  int *m);
/* Empty space *space and set its capacity to *mmx vectors (1..NEKGPU_PROJ_MAX). */
int nekgpu_proj_setup(const int64_t *handle, const int *space, const int *mmx);
/* Number of vectors in space *space. */
int nekgpu_proj_count(const int64_t *handle, const int *space, int *m);

/* ---- operator launch shapes (autotuner) ---------------------------------- */
/* No counterpart in the reference.  The operator's launch shape is the kernel
 * kind (0: plain-load kernel, 1: TMA-staged FP32 kernel) and the number of
 * elements each thread block owns.  Every shape gives identical results (the
 * per-point arithmetic does not depend on the block, and the PCG's partial
 * sums are per element); only the speed differs.  precision: 0 FP64, 1 FP32
 * (the mixed solve's inner PCG).
 * nekgpu_autotune: times every candidate shape of the fused PCG operator on
 *   this mesh now, for coefficient modes h1mode (0 uniform, 1 per point) and
 *   h2mode (0 none, 1 uniform, 2 per point), and keeps the fastest; a mesh
 *   already tuned in this precision, or one of the same kind tuned earlier in
 *   the process (device, lx1, nel, modes), keeps that pick without timing.
 *   Call it before a stream capture that contains a solve.
 * nekgpu_ax_shape: the shape in use (the built-in one while untuned; *ms = 0).
 * nekgpu_set_ax_shape: pins a shape from nekgpu_ax_candidates (kind -1: back
 *   to built-in / tuning), e.g. to replay a recorded pick.
 * nekgpu_ax_candidates: on entry *count = room in kinds/epbs; on return the
 *   number of candidates. */
int nekgpu_autotune(const int64_t *handle, const int *precision, const int *h1mode,
                    const int *h2mode, int *kind, int *epb, double *ms);
int nekgpu_ax_shape(const int64_t *handle, const int *precision, int *kind, int *epb,
                    double *ms);
/* Boundary-group (dssum) kernel of the PCG iteration: threads per block and
 * the shift applied to the default groups per thread (2^gshift).  The FP32
 * inner solve's shape is tuned with the operator's (its rho does not depend
 * on it); the FP64 solve keeps the default (its boundary rho partials are
 * per block). */
int nekgpu_gs_shape(const int64_t *handle, const int *precision, int *threads, int *gshift,
                    double *ms);
/* Pins the FP32 boundary-group kernel shape (threads 128, 256 or 512; gshift
 * -1, 0 or 1); *threads = 0 returns to the default / tuning.  A pinned
 * operator shape (nekgpu_set_ax_shape) skips the tuning of both. */
int nekgpu_set_gs_shape(const int64_t *handle, const int *threads, const int *gshift);
int nekgpu_set_ax_shape(const int64_t *handle, const int *precision, const int *kind,
                        const int *epb);
int nekgpu_ax_candidates(const int64_t *handle, const int *precision, int *kinds, int *epbs,
                         int *count);

/* ---- timing of the last solve (device time, CUDA events) ----------------- */
/* ms_total: whole call on the device; ms_axhelm: summed axhelm-kernel time of
 * the last cggo when the handle's kernel timing is on (nekgpu_set_timing). */
int nekgpu_set_timing(const int64_t *handle, const int *on);
int nekgpu_last_timing(const int64_t *handle, double *ms_total, double *ms_axhelm,
                       int *n_axhelm);
/* The same per-launch timing split over the three kernels of a PCG
 * iteration (operator; boundary-group sum, mask and rho; update), summed over
 * the timed iterations of the last solve. */
int nekgpu_last_kernel_times(const int64_t *handle, double *ms_axhelm, double *ms_gs,
                             double *ms_update, int *iterations);
/* Kernels this library has launched in the process so far (all handles). */
int nekgpu_launch_count(int64_t *count);

#ifdef __cplusplus
}
#endif
#endif
