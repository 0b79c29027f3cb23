// impl.cuh -- handle, mesh and solver internals shared by the library's TUs.
#pragma once
#include <memory>
#include <string>
#include <vector>

#include "axhelm.cuh"
#include "common.cuh"
#include "gs.cuh"
#include "nekgpu.h"

namespace nekgpu {

// Device copy of a field buffer, grown on demand.
template <typename T>
struct DevBuf {
  T* ptr = nullptr;
  size_t cap = 0;
  cudaError_t ensure(size_t n) {
    if (n <= cap) return cudaSuccess;
    cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
    cudaError_t e = cudaMalloc(&ptr, std::max<size_t>(n, 1) * sizeof(T));
    if (e == cudaSuccess) cap = n;
    return e;
  }
  void release() {
    cudaFree(ptr);
    ptr = nullptr;
    cap = 0;
  }
  ~DevBuf() { cudaFree(ptr); }
};

// Operator data in one precision.
template <typename T>
struct OpData {
  T* G = nullptr;    // [nel][6][P]
  T* bm1 = nullptr;  // [n]
  T* D = nullptr;    // [lx1*lx1] row-major
  void release() {
    cudaFree(G);
    cudaFree(bm1);
    cudaFree(D);
    G = bm1 = D = nullptr;
  }
};

// Launch shape of the operator in one precision: kind 0 is axhelm_kernel
// (axhelm.cuh) with `epb` elements per block, kind 1 the TMA-staged FP32
// kernel (axhelm_tma.cuh) with `epb` elements per block (0: its built-in
// count); kind -1 means "not tuned: built-in shape".  `ms` is the tuned
// launch time.  Every shape gives the same results (per-element partials).
struct AxShapeSel {
  int kind = -1;
  int epb = 0;
  float ms = 0.f;
};

struct Mesh {
  int nx1 = 0, nel = 0;
  int64_t n = 0;
  OpData<double> f64;
  OpData<float> f32;  // built on first mixed-precision use
  bool has_f32 = false;
  GsMaps gs;
  double vol = 0.0;  // glsum(bm1) (core/coef.f:1181)
  int* dev_err = nullptr;  // device flag raised by a kernel whose bounded wait expired
  bool use_tma = true;     // TMA-staged operator where lx1 and alignment allow
  std::vector<double> h_D;  // lx1*lx1 row-major (host copy)
  AxShapeSel ax_sel[2];     // [0] FP64, [1] FP32 (see tune.cu)
  // boundary-group kernel shape tuned per precision (gs.cls_tuned), as
  // (threads, groups-per-thread shift) and its launch time
  int gs_gshift[2] = {0, 0};
  float gs_ms[2] = {0.f, 0.f};
  // metric terms rxm1..tzm1 (nine arrays of n: rx ry rz sx sy sz tx ty tz),
  // jacm1 and w3m1 (nx1^3), kept when the geometry is formed from
  // coordinates (geom.cu); the gradient-type operators need them (gradops.cu)
  DevBuf<double> rst, jac, w3, w1;  // w1: the nx1 GLL weights
  bool has_rst = false;
  // double-float form of the FP64 operator (axhelm_df.cuh): (hi, lo) pairs
  // of G1..G6 and D, kept while NEKGPU_OPT_DF is on
  bool use_df = false, has_df = false;
  DevBuf<float2> Gdf, Ddf;
};

// Coefficient descriptor after uniformity detection.
template <typename T>
struct Coef {
  int h1mode = 0, h2mode = 0;  // see AxArgs
  T h1s = T(1), h2s = T(0);
  const T* h1 = nullptr;
  const T* h2 = nullptr;
  const T* hbm = nullptr;  // h2 * bm1 per point when a solve has formed it (AxArgs::hbm)
  const int* perm = nullptr;  // FP32 inner PCG in face order: AxArgs::perm
};

// Work space of one PCG precision.
template <typename T>
struct PcgWork {
  DevBuf<T> r, w, p, d, mult, binv, mask, segmask, segmsum, x, f, h1, h2;
  DevBuf<T> md, mb;  // folded update weights mult*d, mult*binv (fused multiply-add form)
  DevBuf<T> hbm;     // h2 * bm1 of the current solve
};

// One projection space of previous solutions (proj.cu): X and B = A X, each
// mmx vectors of n back to back, xbar / bbar, and the h1 / h2 the space was
// built with.
struct ProjSpace {
  int mmx = 0, m = 0;
  DevBuf<double> xx, bb, xbar, bbar, h1old, h2old;
};

// One field of the multi-field mixed solve (multi.cu): its FP32 PCG vectors,
// FP32 mask and boundary-group mask, FP64 residual and scalars.
struct MultiField {
  DevBuf<float> mask, segmask;
  DevBuf<double> r64;
  DevBuf<CgScalars> cg;
  CgScalars* cg_host = nullptr;  // pinned
  ~MultiField() { cudaFreeHost(cg_host); }
};

// Interface exchange maps of an element shard (vecops.cu).
struct ShardIface;
struct ShardIfaceDeleter {
  void operator()(ShardIface* p) const;
};

// Matrices and fine-grid metric terms of the dealiased convective term (dealias.cu).
struct Dealias;
struct DealiasDeleter {
  void operator()(Dealias* p) const;
};

// An algebraic multigrid hierarchy on the device (amg.cu).
struct AmgDev;
struct AmgDevDeleter {
  void operator()(AmgDev* p) const;
};

// The FP32 inner PCG's face-ordered element layout (perm.cu).
struct PermLayout;
struct PermLayoutDeleter {
  void operator()(PermLayout* p) const;
};

// The FP32 inner PCG's assembled-boundary layout (split.cu).
struct SplitLayout;
struct SplitLayoutDeleter {
  void operator()(SplitLayout* p) const;
};

// The pressure preconditioner h1mg_solve on the device (h1mg.cu).
struct MgDev;
struct MgDevDeleter {
  void operator()(MgDev* p) const;
};

struct Handle {
  int device = 0;
  cudaStream_t stream = nullptr;
  Mesh mesh;
  bool has_mesh = false;
  std::string err;
  CgScalars* cg = nullptr;       // device
  CgScalars* cg_host = nullptr;  // pinned mirror
  DevBuf<double> partialA, partialB, partialC, red;
  // multi-field solve: r, p, w, x of every field, field c at c * n
  DevBuf<float> mfr, mfp, mfw, mfx;
  // GMRES (gmres.cu): Arnoldi and preconditioned vectors, work vectors,
  // Jacobi diagonal, coefficient staging
  DevBuf<double> gm_V, gm_Z, gm_r, gm_w, gm_x, gm_d, gm_c;
  int* flag = nullptr;           // device int scratch
  PcgWork<double> w64;
  PcgWork<float> w32;
  DevBuf<double> io0, io1, io2, io3, io4, io5, io6, io7, io8;  // host-path staging
  // the stress formulation's solve (stress.cu): dpc, p, pp, ap (3 each), and
  // the reductions' block partials
  DevBuf<double> sfw[10], sf_part;
  bool exact = false;  // unfused FP64 arithmetic in the reference's order
  int istep = 0;       // reference time-step index (cggo's "at least one iteration" rule)
  // timing
  bool timing = false;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr, evt0 = nullptr, evt1 = nullptr;
  cudaEvent_t ev_enter = nullptr;  // handle_enter's marker on the legacy default stream
  std::vector<cudaEvent_t> ax_ev;  // per-launch operator timing pool
  double ms_total = 0.0, ms_axhelm = 0.0, ms_gs = 0.0, ms_update = 0.0;
  int n_axhelm = 0;
  // graph cache for the PCG iteration chunk: the captured launches depend on
  // every pointer and coefficient below, so any change recaptures.
  struct GraphKey {
    const void* ptr[15] = {};
    int ints[6] = {-1, -1, -1, -1, -1, -1};
    double dbl[2] = {0, 0};
    bool operator==(const GraphKey& o) const {
      for (int i = 0; i < 15; ++i)
        if (ptr[i] != o.ptr[i]) return false;
      for (int i = 0; i < 6; ++i)
        if (ints[i] != o.ints[i]) return false;
      return dbl[0] == o.dbl[0] && dbl[1] == o.dbl[1];
    }
  };
  GraphKey gkey;
  cudaGraphExec_t gexec = nullptr;
  int gchunk = 0;  // iterations captured in gexec
  int graph_chunk = 16;
  bool own_stream = true;
  bool use_graph = true;
  int mixed_mode = 1;  // see mixed_solve
  bool mcor = false;   // current FP64 solve has cggo's null-space correction
  bool autotune = true;  // time the operator's launch shapes on first solve (tune.cu)
  std::vector<std::unique_ptr<ProjSpace>> proj;  // projection spaces by index (proj.cu)
  std::vector<std::unique_ptr<MultiField>> multi;  // fields of the multi-field solve
  DevBuf<double> mpartialA, mpartialB, mpartialC;
  DevBuf<unsigned int> mcounter;
  DevBuf<CgScalars> cg_tune;  // scalars of the tuning launches (beta = 0, not done)
  // pressure preconditioner of hmh_gmres / hmh_flex_cg: h1mg_solve once set
  // up (nekgpu_h1mg_setup), else the Jacobi diagonal
  std::unique_ptr<MgDev, MgDevDeleter> mg;
  // interface points shared with other shards (nekgpu_iface_setup)
  std::unique_ptr<ShardIface, ShardIfaceDeleter> iface;
  // the dealiased convective term once nekgpu_dealias_setup has run
  std::unique_ptr<Dealias, DealiasDeleter> dealias;
  DevBuf<int> p4_fbc;  // crespsp's face types, staged per call
  // the mixed solve's FP32 inner PCG in the assembled-boundary layout
  // (split.cu), built on first use per mesh when use_split is on
  // (NEKGPU_OPT_SPLIT; off by default: slower than the element-local form
  // on this GPU, see split.cu)
  std::unique_ptr<SplitLayout, SplitLayoutDeleter> split;
  bool use_split = false;
  // the mixed solve's FP32 inner PCG with each element's points in face
  // order (perm.cu), built on first use per mesh when use_perm is on
  // (NEKGPU_OPT_FACE_ORDER; off by default, see perm.cu).  gs32: the maps the
  // FP32 PCG uses while a solve runs in that layout (nullptr: the mesh's own)
  std::unique_ptr<PermLayout, PermLayoutDeleter> perm;
  bool use_perm = false;
  // coarse solve of the pressure preconditioner: X X^T (false, the
  // reference's param(40) = 0) or AMG (true, param(40) = 1;
  // NEKGPU_OPT_COARSE), read by nekgpu_h1mg_setup
  bool coarse_amg = false;
  // the crs_amg-style coarse solver of nekgpu_crs_amg_setup / _solve_dev
  std::unique_ptr<AmgDev, AmgDevDeleter> crs_amg;
  int64_t crs_n = 0;
  bool crs_null = false;
  const GsMaps* gs32 = nullptr;
};

// Double-float FP64 operator (axhelm_df.cu): the mesh's Gdf / Ddf pairs.
cudaError_t launch_axhelm_df(const Mesh& m, const AxArgs<double>& a, bool fused, int epb,
                             int* nparts, cudaStream_t s);
int build_df(Handle& h);

// ---- operator entry points (axhelm_*.cu) ---------------------------------
// Plain operator: au = A u.  Returns cudaError_t of the launch.
template <typename T, bool EXACT>
cudaError_t launch_axhelm(const Mesh& m, const OpData<T>& op, T* au, const T* u, const Coef<T>& c,
                          cudaStream_t s);
// Fused PCG form (see axhelm.cuh).  Returns number of blocks (partials written).
template <typename T, bool EXACT>
cudaError_t launch_axhelm_cg(const Mesh& m, const OpData<T>& op, T* w, T* p, const T* r,
                             const T* d, const Coef<T>& c, const CgScalars* cg, double* partial,
                             int* nblocks, cudaStream_t s);
int axhelm_blocks(int nx1, int nel);
// Autotuner (tune.cu): times the fused operator's candidate launch shapes on
// this mesh (work vectors r, p, w of `wk` as scratch, zeroed) and keeps the
// fastest in mesh.ax_sel; a process-wide cache keyed by device, lx1, nel and
// coefficient modes makes later meshes of the same kind reuse the pick.
// Returns 0 or a negative status.  Must not run inside a stream capture.
template <typename T>
int tune_operator(Handle& h, const OpData<T>& op, PcgWork<T>& wk, const Coef<T>& c);
// Candidate shapes for lx1 = nx and precision prec (0 FP64, 1 FP32).
std::vector<AxShapeSel> ax_candidates(int nx, int prec, bool tma);
// The shape a launch in precision prec uses now (the built-in one, with its
// elements per block filled in, while the mesh is untuned).
AxShapeSel ax_shape_in_use(const Mesh& m, int prec);
// gh1_p = d(lam^T A(h1) u)/d h1_p for every local point (adjoint.cu).
cudaError_t axhelm_adjoint_h1(const Mesh& m, double* gh1, const double* lam, const double* u,
                              cudaStream_t s);

// ---- solver / vector kernels (pcg.cu) ---------------------------------------
template <typename T>
int detect_coef(Handle& h, const T* h1, const T* h2, int64_t n, Coef<T>& c);
template <typename T>
cudaError_t setprec(Handle& h, const OpData<T>& op, T* d, const Coef<T>& c);
// element-local Jacobi diagonal, before dssum and reciprocal (pcg.cu)
int setprec_local_f64(Handle& h, double* d, const Coef<double>& c);
int setprec_f64(Handle& h, double* d, const Coef<double>& c);
double device_sum(Handle& h, int kind, const double* a, const double* b, const double* c,
                  int64_t n, int* status);

struct PcgResult {
  int niter = 0;
  double rbn0 = 0, rbn2 = 0;
  int status = 0;
};

// cggo on device arrays (f: masked, assembled rhs; x: out).  Precision T.
// dpre: precomputed Jacobi diagonal (device, precision T), or nullptr to
// run setprec (FP64 only).
template <typename T>
PcgResult pcg_solve(Handle& h, const OpData<T>& op, PcgWork<T>& wk, T* x, const T* f,
                    const Coef<T>& c, const T* mask, const T* mult, const T* binv, double tin,
                    int maxiter, int istep, bool exact, const T* dpre = nullptr);
template <typename T>
double device_absmax(Handle& h, const T* a, int64_t n, int* status);
template <typename T>
PcgResult pcg_prepare(Handle& h, PcgWork<T>& wk, T* x, const T* f, const Coef<T>& c,
                      const T* mask, const T* mult, double tin, int maxiter, int istep,
                      const T* dpre, bool* trivial);
int pcg_vec_blocks(int64_t n);
// gradops.cu: op 0 wgradm1 (o1..o3 <- i1), 1 dudxyz (o1 <- i1, m = isd - 1),
// 2 cdtp (o1 <- i1, m, bm1), 3 curl (o1..o3 <- i1..i3); 0 or -1 (lx1).
int launch_gradop(Handle& h, int op, double* o1, double* o2, double* o3, const double* i1,
                  const double* i2, const double* i3, int m, const double* bm1);
void launch_mul_by(Handle& h, double* a, const double* b);
int launch_conv1(Handle& h, double* du, const double* u, const double* vx, const double* vy,
                 const double* vz);
void launch_subcol3(Handle& h, double* bf, const double* ta);
// dealias.cu: fine-grid matrices and metric terms for lxd points; the
// dealiased convective term conv = convect_new(u) / bm1.  0 or an error.
int dealias_setup(Handle& h, int lxd, std::string& err);
int dealias_lxd(const Handle& h);
int convop_dealias(Handle& h, double* conv, const double* u, const double* vx, const double* vy,
                   const double* vz);

// h1mg.cu: z = M rhs with the set-up preconditioner (rhs masked in place,
// as h1mg_solve leaves it); 0, -3 or -6 (not set up).  Setup from host
// coordinates, mask or face types, and the fine numbering; 0 or NEKGPU_E*.
int h1mg_apply(Handle& h, double* z, double* rhs);
int h1mg_setup(Handle& h, const double* x, const double* y, const double* z, const double* mask,
               const int64_t* glo, const int* fbc, bool null_space);

// hmh_flex_cg with the Jacobi preconditioner (gmres.cu); 0, -3, -4 or -5.
int flex_cg_solve(Handle& h, double* res, const double* h1, const double* h2, const double* wt,
                  const double* mask, double tol, int maxit, bool null_space, int* niter,
                  double* div0, double* rnorm);
// hmh_gmres with the Jacobi preconditioner (gmres.cu); 0, -3, -4 or -5.
int gmres_solve(Handle& h, double* res, const double* h1, const double* h2, const double* wt,
                const double* mask, double tol, int maxit, int m, bool null_space, int* niter,
                double* div0, double* rnorm);
// Sets *bad when an element-interior point (not in a boundary group) has mask
// or multiplicity other than 1 (FP32 arrays; the fused operator assumes 1).
void launch_interior_check(Handle& h, const float* mask, const float* mult, int* bad);
// Per-solve data of a prepared solve: the update kernel's folded weights
// (fused multiply-add form) and, for FP64, h2*bm1 (sets c.hbm).
template <typename T>
int pcg_solve_extras(Handle& h, const OpData<T>& op, PcgWork<T>& wk, const T* mult, const T* binv,
                     Coef<T>& c, bool exact);
// Iteration-1 check of a prepared solve (no update), then the iterations.
template <typename T>
int pcg_first_check(Handle& h, PcgWork<T>& wk, T* x, const T* mult, const T* binv, bool exact);
template <typename T>
PcgResult pcg_iterate(Handle& h, const OpData<T>& op, PcgWork<T>& wk, T* x, const Coef<T>& c,
                      const T* mult, const T* binv, bool exact);

// Mixed-precision helpers (mixed.cu), used by the batched solver too.
int ensure_f32(Handle& h);
void cast_to_f32(Handle& h, float* o, const double* a, double scale, int64_t n);
void axpy_f32(Handle& h, double* x, const float* e, double scale, int64_t n);
// r = f - mask * dssum(A x) (FP64); returns cggo's norm of r, or -1 on error.
double outer_residual(Handle& h, double* r, const double* f, const double* x,
                      const Coef<double>& c, const double* mask, const double* mult,
                      const double* binv, double* w);
double norm64(Handle& h, const double* r, const double* mult, const double* binv);

// Mixed precision (mixed.cu): FP32 inner PCG in an FP64 defect-correction loop.
struct MixedResult {
  int outer = 0, inner = 0;
  int restarts = 0;  // mode 1: replacements that also restarted the direction
  double rbn0 = 0, rbn2 = 0;
  int status = 0;
};
// Projection onto previous solutions (proj.cu).
int proj_space(Handle& h, int space, ProjSpace** out);
int proj_alloc(Handle& h, ProjSpace& P);
int proj_project1(Handle& h, ProjSpace& P, double* b, const Coef<double>& c, const double* h1,
                  const double* h2, const double* msk, const double* w);
int proj_project2(Handle& h, ProjSpace& P, double* x, const Coef<double>& c, const double* msk,
                  const double* w);
// Residual replacement into the running FP32 PCG (see mixed.cu).
int mixed_replace(Handle& h, double& scale, double inner_tol, int* restarts,
                  const int* perm = nullptr);
// The same for any FP32 PCG: its vectors, the FP64 residual, its scalars.
struct ReplaceTarget {
  float* r32;
  float* p32;
  float* x32;
  const float* d32;
  const float* mult32;
  const float* binv32;
  const double* r64;
  CgScalars* cg_dev;
  CgScalars* cg_host;
  const int* perm = nullptr;  // face-ordered FP32 vectors (perm.cu): r32 cast through it
};
int mixed_replace_into(Handle& h, const ReplaceTarget& t, double& scale, double inner_tol,
                       int* restarts);
// mode 0: each outer step is a fresh FP32 PCG to inner_tol (restarted);
// mode 1: one FP32 PCG whose residual is replaced by the FP64 one whenever it
// has dropped by inner_tol, keeping the search direction (reliable updates).
MixedResult mixed_solve(Handle& h, double* x, const double* f, const double* h1,
                        const double* h2, const double* mask, const double* mult,
                        const double* binv, double tin, int maxit, double inner_tol,
                        int mode = 0);

void set_error(Handle& h, const std::string& msg);

// ---- algebraic multigrid on the device (amg.cu) ---------------------------
struct AmgPlan;
int amg_upload(const AmgPlan& p, std::unique_ptr<AmgDev, AmgDevDeleter>& out, cudaStream_t s);
// y = one V-cycle applied to v (unknowns' order, n values each)
void amg_apply_dev(AmgDev& a, double* y, const double* v, cudaStream_t s);

// ---- the FP32 inner PCG in the face-ordered element layout (perm.cu) -----
std::vector<int> face_order(int nx);
bool perm_eligible(const Handle& h);
int perm_setup(Handle& h);
const int* perm_pt_pos(const Handle& h);
const GsMaps* perm_maps(const Handle& h);
// o (face-ordered FP32) = scale * a (natural FP64); x (natural) += scale * e32
void perm_cast(Handle& h, float* o, const double* a, double scale);
void perm_axpy(Handle& h, double* x, const float* e32, double scale);

// ---- the FP32 inner PCG in the assembled-boundary layout (split.cu) ------
// Eligible meshes: even lx1 in 4..12, interior points private to their
// element, the TMA-staged operator on.
bool split_eligible(const Handle& h);
int split_setup(Handle& h);
int split_load(Handle& h, const double* r64, double inv_scale, const double* d64,
               const double* binv64, const double* mask64);
int split_first_check(Handle& h, const Coef<float>& c);
PcgResult split_iterate(Handle& h, const Coef<float>& c);
void split_axpy(Handle& h, double* x64, double scale);
int split_replace(Handle& h, const double* r64, double& scale, double inner_tol, int* restarts);

// Handle life cycle and mesh upload (capi.cu); `shared` != nullptr makes the
// handle use that stream instead of creating one.
int handle_open(Handle& h, int device, cudaStream_t shared, std::string& err);
void handle_close(Handle& h);
// Start of every call on a handle: make the handle's device current and make
// the handle's stream wait for all work already queued on the legacy default
// stream (torch's default stream, cudaMemcpy, kernels launched on stream 0).
// The handle's stream is non-blocking, so without this wait a kernel of the
// call could read an input the caller's last kernel has not finished writing.
cudaError_t handle_enter(Handle& h);
// End of every call: wait for the handle's stream and report the first error
// it met, so that the caller may read the outputs from any stream.
cudaError_t handle_leave(Handle& h);
int handle_setup(Handle& h, int lx1, int nel, const double* dxm1, const double* const* g6,
                 const double* bm1, const int64_t* glo_num, std::string& err);

// Returns true (and records `where`) when a CUDA error is pending.
inline bool cuda_pending(Handle& h, const char* where) {
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) return false;
  h.err = std::string(where) + ": " + cudaGetErrorString(e);
  return true;
}

}  // namespace nekgpu
