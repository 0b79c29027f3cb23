// h1mg.h -- host plan of the pressure preconditioner h1mg_solve
// (core/hsmg.f:1855-1949, if_hybrid = .false.): level orders, numberings,
// masks, weights, fast-diagonalisation matrices and the coarse inverse.
// Built on the host once (h1mg_plan.cpp), uploaded and applied on the device
// (h1mg.cu).  Plain C++: included by host and device translation units.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace nekgpu {

constexpr int kMgMaxLev = 4;

// A^-1 = X X^T in nested-dissection order (xxt.cpp): perm[k] = the unknown
// numbered k; X by columns (cptr/cidx/cval: rows i of column j) and by rows
// (rptr/ridx/rval: columns j of row i, ascending), both in that order.
struct XxtFactor {
  int64_t n = 0;
  std::vector<int> perm;
  std::vector<int64_t> cptr, rptr;
  std::vector<int> cidx, ridx;
  std::vector<double> cval, rval;
};

// Factor the symmetric positive definite n x n matrix (CSR, both triangles)
// whose unknowns sit at xyz (3 per unknown).  Returns 0 or NEKGPU_EINVAL.
int xxt_factor(XxtFactor& f, int64_t n, const std::vector<int64_t>& ptr,
               const std::vector<int>& idx, const std::vector<double>& val, const double* xyz,
               std::string& err);

// Algebraic multigrid of a coarse matrix (amg_plan.cpp): the reference's crs_amg
// hierarchy (core/crs_amg.c), level l holding its F points at
// [off[l], off[l+1]) of the plan's order (perm[k] = the unknown at position
// k).  W: interpolation from the coarser points (nf x nc, CSR), WT its
// transpose, AFP = AFF W + A_FC the F rows of A P (P = [W; I]; kept in the
// afc_* arrays) and AFF the F-F block of the level's matrix,
// dff the scaled inverse diagonal of AFF, cheb_m / cheb_rho the Chebyshev
// smoother.  The last level has one unknown: x = dff b.
struct AmgLevel {
  int64_t nf = 0, nc = 0;
  int cheb_m = 1;
  double cheb_rho = 0.0;
  std::vector<double> dff;
  std::vector<int64_t> w_ptr, wt_ptr, afc_ptr, aff_ptr;
  std::vector<int> w_idx, wt_idx, afc_idx, aff_idx;
  std::vector<double> w_val, wt_val, afc_val, aff_val;
};
struct AmgPlan {
  int64_t n = 0;
  std::vector<int64_t> perm, off;
  std::vector<AmgLevel> lev;
};
// Hierarchy of the symmetric positive definite n x n matrix (CSR, both
// triangles, columns ascending).  Returns 0 or NEKGPU_EINVAL.
int amg_setup(AmgPlan& p, int64_t n, const std::vector<int64_t>& ptr, const std::vector<int>& idx,
              const std::vector<double>& val, std::string& err);
// One V-cycle (amg_exec, core/crs_amg.c:129-186) in the plan's order; b is
// overwritten.
void amg_apply_host(const AmgPlan& p, double* x, double* b);

struct MgLevelPlan {
  int nx = 0;                         // points per direction (order + 1)
  int64_t n = 0;                      // nx^3 nel
  std::vector<int64_t> glo, glo_ext;  // level and extended ((nx+2)^3) numberings
  std::vector<double> mask;           // 0 on Dirichlet points, else 1
  std::vector<double> rwt;            // 1 / multiplicity (restriction weights)
  std::vector<double> swt;            // Schwarz weights (levels above 0)
  std::vector<double> S;              // [e][d][nl*nl]: column j = eigenvector j
  std::vector<double> dinv;           // [e][nl^3]: 1/(lam_r + lam_s + lam_t) or 0
  std::vector<double> jh;             // nx x nx(l-1), column-major (levels above 0)
  std::vector<double> z, w, ah;       // GLL points, weights, 1-D stiffness
};

struct MgPlan {
  int nx1 = 0, nel = 0, lmax = 0;
  bool null_space = false;
  int order[kMgMaxLev] = {0, 0, 0, 0};
  MgLevelPlan lev[kMgMaxLev];  // lev[0]: order 1 (one point per vertex)
  std::vector<int> fbc;        // 6 face types per element
  std::vector<int64_t> vrank;  // 8 ranked vertex ids per element
  std::vector<double> lenl, lenm, lenr;  // element widths [3 e + d]
  int64_t nc = 0, nsolve = 0;  // coarse unknowns, and those in the inverse
  std::vector<int64_t> cid;    // per level-0 point: coarse unknown or -1
  std::vector<double> ccoord;  // coordinates of the coarse unknowns (3 each)
  XxtFactor xxt;               // of the first nsolve unknowns
  bool use_amg = false;        // coarse solve by AMG (crs_amg) instead of X X^T
  AmgPlan amg;                 // of the first nsolve unknowns, when use_amg
};

// Level orders of h1mg_setup_mg_nx (core/hsmg.f:2272-2338) in 3-D; returns lmax.
int h1mg_levels(int lx1, int* order);

// Face types (get_fast_bc, core/fast3d.f:802-870) read from a numbering and
// mask: per element r-, r+, s-, s+, t-, t+; 0 when the face's point (1, 1)
// is shared (interior or periodic face), else 1 when it is masked
// (Dirichlet), else 2 (Neumann).  nx >= 3.
void h1mg_face_types(int nx, int nel, const int64_t* glo, const double* mask, int* fbc);

// Everything but the coarse inverse.  x, y, z: fine GLL coordinates; glo:
// fine numbering; mask: fine pressure mask (used only when fbc is null);
// fbc: face types or null.  Returns 0 or an NEKGPU_E* code.
int h1mg_plan(MgPlan& p, int nx1, int nel, const int64_t* glo, const double* x, const double* y,
              const double* z, const double* mask, const int* fbc, bool null_space,
              std::string& err);

// The trilinear basis b_j (j = 0..7, bit 0 r, bit 1 s, bit 2 t) at the fine
// GLL points (gen_crs_basis, core/navier8.f:1689-1731): 8 nx1^3 values.
void h1mg_coarse_basis(int nx1, std::vector<double>& b);

// Coarse factor from the element matrices a[e][i + 8 j] = b_i^T A_e b_j
// (get_local_crs_galerkin, core/navier8.f:1648-1687).  Returns 0 or an error.
int h1mg_plan_coarse(MgPlan& p, const double* elem, std::string& err);

// One 1-D fast-diagonalisation operator (hsmg_setup_fast1d, core/hsmg.f:
// 783-881): s (nl x nl, column j = vector j, rows of excluded points zeroed)
// and lam ascending, nl = n + 3.
void h1mg_fast1d(double* s, double* lam, int lbc, int rbc, double ll, double lm, double lr,
                 const double* ah, const double* bh, int n);

// Records msg as the calling thread's nekmesh_last_error; returns code.
int mesh_fail(int code, const std::string& msg);

}  // namespace nekgpu
