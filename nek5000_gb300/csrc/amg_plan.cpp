// amg_plan.cpp -- host setup of the algebraic multigrid coarse solve of the
// pressure preconditioner (the reference's crs_amg, param(40) = 1,
// core/drive2.f:1789-1797).
//
// The reference applies a hierarchy that an external tool builds with hypre
// (tools/nekamg_setup) and writes to amg*.dat files; its solve (amg_exec,
// core/crs_amg.c:129-186) is a reduction-based V-cycle.  Each level splits its
// unknowns into F points, handled on that level, and C points, passed on:
//
//   down   b_C += W^T b_F                     (every level, fine to coarse)
//   bottom x = Dff b                          (the last level has one unknown)
//   up     x_F = W x_C ; b_F -= AfP x_C ;
//          c = Chebyshev(Aff, Dff, m, rho) b_F ; x_F += c
//
// with W the interpolation from the C points, AfP = Aff W + A_FC the F rows of
// A P (P = [W; I] the prolongation), Dff the scaled inverse diagonal of the
// F-F block, and m Chebyshev steps tuned to rho, the spectral radius of
// I - Dff Aff.  The coarse matrix of the next level is the Galerkin product
// P^T A P with P = [W; I].  This file builds that hierarchy itself, so no
// setup files are needed:
//
//   * the C/F split is the first pass of Ruge and Stueben's coarsening
//     (strong couplings -a_ij >= theta max_k -a_ik, theta = 0.25; C points
//     picked by the count of unassigned points they strongly influence, their
//     strong neighbours become F), followed by a check that makes Aff
//     diagonally dominant: an F point whose F-F off-diagonal row sum exceeds
//     its diagonal joins C;
//   * W: Stueben's direct interpolation, -a_ij / a_ii over the C points j an
//     F point i is coupled to, the negative and the positive couplings each
//     scaled so that the row's off-diagonal sum is kept (constants, the
//     Laplacian's near null space, are interpolated exactly);
//   * the smoother as the reference's setup tool makes it: the extreme
//     eigenvalues [a, b] of D^1/2 Aff D^1/2 (power iterations here, Lanczos
//     there), Dff = 2 / (a + b) diag(Aff)^-1, rho = (b - a) / (b + a), and
//     the fewest Chebyshev steps m whose contraction is below 1 - sqrt(1/2)
//     (its chebsim).
//
// Unknowns are renumbered level by level (F points of level 0 first, then of
// level 1, ...), as the reference's lvl_offset layout keeps them.
#include <algorithm>
#include <cmath>
#include <map>
#include <numeric>
#include <vector>

#include "h1mg.h"
#include "nekgpu.h"

namespace nekgpu {

namespace {

struct Csr {
  int64_t rows = 0, cols = 0;
  std::vector<int64_t> ptr;
  std::vector<int> idx;
  std::vector<double> val;
};

// Rows `rs` and columns `cs` (maps from old index to new, -1 = dropped) of A.
Csr submatrix(const Csr& A, const std::vector<int>& rs, int64_t nr, const std::vector<int>& cs,
              int64_t nc) {
  Csr S;
  S.rows = nr;
  S.cols = nc;
  S.ptr.assign((size_t)nr + 1, 0);
  std::vector<std::vector<std::pair<int, double>>> rows((size_t)nr);
  for (int64_t i = 0; i < A.rows; ++i) {
    const int ri = rs[(size_t)i];
    if (ri < 0) continue;
    for (int64_t q = A.ptr[i]; q < A.ptr[i + 1]; ++q) {
      const int cj = cs[(size_t)A.idx[(size_t)q]];
      if (cj >= 0) rows[(size_t)ri].push_back({cj, A.val[(size_t)q]});
    }
  }
  for (int64_t r = 0; r < nr; ++r) {
    auto& v = rows[(size_t)r];
    std::sort(v.begin(), v.end());
    for (auto& e : v) {
      S.idx.push_back(e.first);
      S.val.push_back(e.second);
    }
    S.ptr[(size_t)r + 1] = (int64_t)S.idx.size();
  }
  return S;
}

Csr transpose(const Csr& A) {
  Csr T;
  T.rows = A.cols;
  T.cols = A.rows;
  T.ptr.assign((size_t)T.rows + 1, 0);
  for (int c : A.idx) ++T.ptr[(size_t)c + 1];
  for (int64_t r = 0; r < T.rows; ++r) T.ptr[(size_t)r + 1] += T.ptr[(size_t)r];
  T.idx.resize(A.idx.size());
  T.val.resize(A.val.size());
  std::vector<int64_t> pos(T.ptr.begin(), T.ptr.end() - 1);
  for (int64_t i = 0; i < A.rows; ++i)  // ascending rows: T's columns ascend
    for (int64_t q = A.ptr[i]; q < A.ptr[i + 1]; ++q) {
      const int64_t p = pos[(size_t)A.idx[(size_t)q]]++;
      T.idx[(size_t)p] = (int)i;
      T.val[(size_t)p] = A.val[(size_t)q];
    }
  return T;
}

// C = A B (sparse, rows of C accumulated in a dense work row).
Csr multiply(const Csr& A, const Csr& B) {
  Csr C;
  C.rows = A.rows;
  C.cols = B.cols;
  C.ptr.assign((size_t)C.rows + 1, 0);
  std::vector<double> acc((size_t)B.cols, 0.0);
  std::vector<int> mark((size_t)B.cols, -1), cols;
  for (int64_t i = 0; i < A.rows; ++i) {
    cols.clear();
    for (int64_t q = A.ptr[i]; q < A.ptr[i + 1]; ++q) {
      const int k = A.idx[(size_t)q];
      const double a = A.val[(size_t)q];
      for (int64_t t = B.ptr[k]; t < B.ptr[k + 1]; ++t) {
        const int j = B.idx[(size_t)t];
        if (mark[(size_t)j] != (int)i) {
          mark[(size_t)j] = (int)i;
          acc[(size_t)j] = 0.0;
          cols.push_back(j);
        }
        acc[(size_t)j] += a * B.val[(size_t)t];
      }
    }
    std::sort(cols.begin(), cols.end());
    for (int j : cols) {
      C.idx.push_back(j);
      C.val.push_back(acc[(size_t)j]);
    }
    C.ptr[(size_t)i + 1] = (int64_t)C.idx.size();
  }
  return C;
}

// C = A + B (same shape).
Csr add(const Csr& A, const Csr& B) {
  Csr C;
  C.rows = A.rows;
  C.cols = A.cols;
  C.ptr.assign((size_t)C.rows + 1, 0);
  for (int64_t i = 0; i < A.rows; ++i) {
    std::map<int, double> row;
    for (int64_t q = A.ptr[i]; q < A.ptr[i + 1]; ++q) row[A.idx[(size_t)q]] += A.val[(size_t)q];
    for (int64_t q = B.ptr[i]; q < B.ptr[i + 1]; ++q) row[B.idx[(size_t)q]] += B.val[(size_t)q];
    for (auto& e : row) {
      C.idx.push_back(e.first);
      C.val.push_back(e.second);
    }
    C.ptr[(size_t)i + 1] = (int64_t)C.idx.size();
  }
  return C;
}

double diag_of(const Csr& A, int64_t i) {
  for (int64_t q = A.ptr[i]; q < A.ptr[i + 1]; ++q)
    if (A.idx[(size_t)q] == (int)i) return A.val[(size_t)q];
  return 0.0;
}

// C/F split of A (1 = C).  First pass of Ruge-Stueben, then diagonal
// dominance of the F-F block.
std::vector<char> split_cf(const Csr& A, double theta) {
  const int64_t n = A.rows;
  std::vector<std::vector<int>> S((size_t)n), ST((size_t)n);  // strong: i depends on j
  for (int64_t i = 0; i < n; ++i) {
    double mx = 0.0;
    for (int64_t q = A.ptr[i]; q < A.ptr[i + 1]; ++q)
      if (A.idx[(size_t)q] != (int)i) mx = std::max(mx, -A.val[(size_t)q]);
    if (mx <= 0.0) continue;
    for (int64_t q = A.ptr[i]; q < A.ptr[i + 1]; ++q) {
      const int j = A.idx[(size_t)q];
      if (j != (int)i && -A.val[(size_t)q] >= theta * mx) {
        S[(size_t)i].push_back(j);
        ST[(size_t)j].push_back((int)i);
      }
    }
  }
  std::vector<char> st((size_t)n, 0);  // 0 unassigned, 1 C, 2 F
  std::vector<int> lam((size_t)n);
  for (int64_t i = 0; i < n; ++i) lam[(size_t)i] = (int)ST[(size_t)i].size();
  // bucket priority queue on lam (ties: lowest index first)
  std::multimap<int, int> pq;
  std::vector<std::multimap<int, int>::iterator> where((size_t)n);
  for (int64_t i = 0; i < n; ++i) where[(size_t)i] = pq.insert({-lam[(size_t)i], (int)i});
  auto bump = [&](int j, int d) {
    if (st[(size_t)j]) return;
    pq.erase(where[(size_t)j]);
    lam[(size_t)j] += d;
    where[(size_t)j] = pq.insert({-lam[(size_t)j], j});
  };
  while (!pq.empty()) {
    auto it = pq.begin();
    const int i = it->second;
    pq.erase(it);
    if (st[(size_t)i]) continue;
    st[(size_t)i] = 1;  // C
    for (int j : ST[(size_t)i]) {
      if (st[(size_t)j]) continue;
      st[(size_t)j] = 2;  // F
      pq.erase(where[(size_t)j]);
      for (int k : S[(size_t)j]) bump(k, 1);
    }
    for (int k : S[(size_t)i]) bump(k, -1);
  }
  // F points whose F-F coupling is not dominated by the diagonal join C
  for (int64_t i = 0; i < n; ++i) {
    if (st[(size_t)i] != 2) continue;
    double off = 0.0, d = 0.0;
    for (int64_t q = A.ptr[i]; q < A.ptr[i + 1]; ++q) {
      const int j = A.idx[(size_t)q];
      if (j == (int)i) d = A.val[(size_t)q];
      else if (st[(size_t)j] == 2) off += std::fabs(A.val[(size_t)q]);
    }
    if (!(off < d)) st[(size_t)i] = 1;
  }
  return st;
}

// Extreme eigenvalues [a, b] of M = D^1/2 Aff D^1/2 (D = 1 / diag Aff):
// power iteration for b, then on b I - M for b - a (deterministic start).
void eig_bounds(const Csr& Aff, const std::vector<double>& dinv, double& a, double& b) {
  const int64_t n = Aff.rows;
  std::vector<double> sq((size_t)n), v((size_t)n), w((size_t)n);
  for (int64_t i = 0; i < n; ++i) sq[(size_t)i] = std::sqrt(dinv[(size_t)i]);
  auto apply = [&](const std::vector<double>& x, std::vector<double>& y) {
    for (int64_t i = 0; i < n; ++i) {
      double s = 0.0;
      for (int64_t q = Aff.ptr[i]; q < Aff.ptr[i + 1]; ++q)
        s += Aff.val[(size_t)q] * sq[(size_t)Aff.idx[(size_t)q]] * x[(size_t)Aff.idx[(size_t)q]];
      y[(size_t)i] = sq[(size_t)i] * s;
    }
  };
  auto power = [&](double shift) {  // largest eigenvalue of shift I - M (shift 0: of M)
    for (int64_t i = 0; i < n; ++i) v[(size_t)i] = 1.0 + 0.37 * std::sin(1.0 + (double)i);
    double lam = 0.0;
    for (int it = 0; it < 40; ++it) {
      double nv = 0.0;
      for (double x : v) nv += x * x;
      nv = std::sqrt(nv);
      if (nv == 0.0) return 0.0;
      for (double& x : v) x /= nv;
      apply(v, w);
      if (shift != 0.0)
        for (int64_t i = 0; i < n; ++i) w[(size_t)i] = shift * v[(size_t)i] - w[(size_t)i];
      double vw = 0.0;
      for (int64_t i = 0; i < n; ++i) vw += v[(size_t)i] * w[(size_t)i];
      lam = vw;  // Rayleigh quotient
      v.swap(w);
    }
    return lam;
  };
  b = power(0.0) * 1.05;  // power iteration approaches from below: widen
  a = std::max(0.0, b - power(b) * 1.05);
  if (!(a > 0.0)) a = 1e-3 * b;
}

// chebsim (the reference's setup tool): Chebyshev steps m whose contraction
// falls below tol for the Jacobi radius rho.
int cheb_steps(double rho, double tol) {
  const double alpha = 0.25 * rho * rho;
  int m = 1;
  double cp = 1.0, c = rho, gamma = 1.0;
  while (c > tol && m < 12) {
    ++m;
    const double d = alpha * (1.0 + gamma);
    gamma = d / (1.0 - d);
    const double cn = (1.0 + gamma) * rho * c - gamma * cp;
    cp = c;
    c = cn;
  }
  return m;
}

// Columns renumbered by newc (entries of each row re-sorted).
void permute_cols(std::vector<int64_t>& ptr, std::vector<int>& idx, std::vector<double>& val,
                  const std::vector<int>& newc) {
  const int64_t rows = (int64_t)ptr.size() - 1;
  std::vector<std::pair<int, double>> row;
  for (int64_t r = 0; r < rows; ++r) {
    row.clear();
    for (int64_t q = ptr[(size_t)r]; q < ptr[(size_t)r + 1]; ++q)
      row.push_back({newc[(size_t)idx[(size_t)q]], val[(size_t)q]});
    std::sort(row.begin(), row.end());
    int64_t q = ptr[(size_t)r];
    for (auto& e : row) {
      idx[(size_t)q] = e.first;
      val[(size_t)q] = e.second;
      ++q;
    }
  }
}

// Rows reordered: row newr[i] of the result is row i of the input.
void permute_rows(std::vector<int64_t>& ptr, std::vector<int>& idx, std::vector<double>& val,
                  const std::vector<int>& newr) {
  const int64_t rows = (int64_t)ptr.size() - 1;
  std::vector<int> inv((size_t)rows);
  for (int64_t i = 0; i < rows; ++i) inv[(size_t)newr[(size_t)i]] = (int)i;
  std::vector<int64_t> np((size_t)rows + 1, 0);
  std::vector<int> ni;
  std::vector<double> nv;
  ni.reserve(idx.size());
  nv.reserve(val.size());
  for (int64_t r = 0; r < rows; ++r) {
    const int src = inv[(size_t)r];
    for (int64_t q = ptr[(size_t)src]; q < ptr[(size_t)src + 1]; ++q) {
      ni.push_back(idx[(size_t)q]);
      nv.push_back(val[(size_t)q]);
    }
    np[(size_t)r + 1] = (int64_t)ni.size();
  }
  ptr.swap(np);
  idx.swap(ni);
  val.swap(nv);
}

void store(const Csr& A, std::vector<int64_t>& ptr, std::vector<int>& idx,
           std::vector<double>& val) {
  ptr = A.ptr;
  idx = A.idx;
  val = A.val;
}

}  // namespace

int amg_setup(AmgPlan& P, int64_t n, const std::vector<int64_t>& ptr, const std::vector<int>& idx,
              const std::vector<double>& val, std::string& err) {
  P = AmgPlan();
  P.n = n;
  if (n < 1) return 0;
  Csr A;
  A.rows = A.cols = n;
  A.ptr = ptr;
  A.idx = idx;
  A.val = val;
  // cur[k] = original unknown of the current level's row k
  std::vector<int64_t> cur((size_t)n);
  std::iota(cur.begin(), cur.end(), 0);
  P.perm.reserve((size_t)n);
  P.off.push_back(0);
  for (int guard = 0; guard < 64; ++guard) {
    const int64_t m = A.rows;
    AmgLevel L;
    if (m == 1) {  // bottom: one unknown
      const double d = diag_of(A, 0);
      if (!(d > 0.0)) {
        err = "amg: the coarse matrix is not positive definite";
        return NEKGPU_EINVAL;
      }
      L.nf = 1;
      L.nc = 0;
      L.dff = {1.0 / d};
      P.perm.push_back(cur[0]);
      P.off.push_back(P.off.back() + 1);
      P.lev.push_back(std::move(L));
      return 0;
    }
    std::vector<char> st = split_cf(A, 0.25);
    int64_t nf = 0, nc = 0;
    for (char c : st) (c == 2 ? nf : nc) += 1;
    if (nc == m) {  // nothing strongly coupled: keep one C point
      std::fill(st.begin(), st.end(), 2);
      st[(size_t)(m - 1)] = 1;
      nf = m - 1;
      nc = 1;
    } else if (nf == m) {
      st[(size_t)(m - 1)] = 1;
      nf = m - 1;
      nc = 1;
    }
    std::vector<int> fmap((size_t)m, -1), cmap((size_t)m, -1);
    int64_t fi = 0, ci = 0;
    {
      // this level's rows in the plan's order (F first, then C).  Every
      // earlier level's W, AfP columns and W^T rows that reach this block
      // (plan positions off.back() .. n) indexed it in row order: renumber
      const int64_t ob = P.off.back();
      std::vector<int> pos((size_t)m);
      int64_t pf = 0, pc = nf;
      for (int64_t i = 0; i < m; ++i) pos[(size_t)i] = (int)(st[(size_t)i] == 2 ? pf++ : pc++);
      for (size_t l = 0; l < P.lev.size(); ++l) {
        AmgLevel& Q = P.lev[l];
        const int64_t base = P.off[l + 1];  // plan position of Q's column 0
        std::vector<int> newc((size_t)Q.nc);
        for (int64_t c = 0; c < Q.nc; ++c) {
          const int64_t g = base + c;
          newc[(size_t)c] = g >= ob ? (int)(ob + pos[(size_t)(g - ob)] - base) : (int)c;
        }
        permute_cols(Q.w_ptr, Q.w_idx, Q.w_val, newc);
        permute_cols(Q.afc_ptr, Q.afc_idx, Q.afc_val, newc);
        permute_rows(Q.wt_ptr, Q.wt_idx, Q.wt_val, newc);
      }
    }
    std::vector<int64_t> next;
    for (int64_t i = 0; i < m; ++i) {
      if (st[(size_t)i] == 2) {
        fmap[(size_t)i] = (int)fi++;
        P.perm.push_back(cur[(size_t)i]);
      } else {
        cmap[(size_t)i] = (int)ci++;
        next.push_back(cur[(size_t)i]);
      }
    }
    const Csr Aff = submatrix(A, fmap, nf, fmap, nf);
    const Csr Afc = submatrix(A, fmap, nf, cmap, nc);
    const Csr Acf = submatrix(A, cmap, nc, fmap, nf);
    const Csr Acc = submatrix(A, cmap, nc, cmap, nc);
    L.nf = nf;
    L.nc = nc;
    L.dff.resize((size_t)nf);
    for (int64_t i = 0; i < nf; ++i) {
      const double d = diag_of(Aff, i);
      if (!(d > 0.0)) {
        err = "amg: a non-positive diagonal (the coarse matrix is not positive definite)";
        return NEKGPU_EINVAL;
      }
      L.dff[(size_t)i] = 1.0 / d;
    }
    // W: direct interpolation (Stueben) from the C points an F point is
    // coupled to, each sign's weights scaled so that the row's off-diagonal
    // sum is kept (constants are interpolated exactly where A's rows sum to 0)
    Csr W = Afc;
    {
      std::vector<int64_t> frow((size_t)nf);
      for (int64_t r = 0; r < m; ++r)
        if (fmap[(size_t)r] >= 0) frow[(size_t)fmap[(size_t)r]] = r;
      for (int64_t i = 0; i < nf; ++i) {
        const int64_t r = frow[(size_t)i];
        double aii = 0.0, neg = 0.0, pos = 0.0, negc = 0.0, posc = 0.0;
        for (int64_t q = A.ptr[r]; q < A.ptr[r + 1]; ++q) {
          const int j = A.idx[(size_t)q];
          const double a = A.val[(size_t)q];
          if (j == (int)r) {
            aii = a;
            continue;
          }
          (a < 0 ? neg : pos) += a;
          if (cmap[(size_t)j] >= 0) (a < 0 ? negc : posc) += a;
        }
        double al = negc != 0.0 ? neg / negc : 0.0, be = 0.0;
        if (posc > 0.0) be = pos / posc;
        else aii += pos;
        for (int64_t q = W.ptr[i]; q < W.ptr[i + 1]; ++q) {
          const double a = W.val[(size_t)q];
          W.val[(size_t)q] = -(a < 0 ? al : be) * a / aii;
        }
      }
    }
    // Chebyshev smoother (the reference's setup tool): D scaled by 2/(a+b),
    // rho = (b-a)/(b+a), m steps for a contraction of 1 - sqrt(1 - 0.5)
    if (nf > 1) {
      double ea = 0.0, eb = 0.0;
      eig_bounds(Aff, L.dff, ea, eb);
      for (double& d : L.dff) d *= 2.0 / (ea + eb);
      L.cheb_rho = (eb - ea) / (eb + ea);
      L.cheb_m = cheb_steps(L.cheb_rho, 1.0 - std::sqrt(1.0 - 0.5));
    } else {
      L.cheb_rho = 0.0;
      L.cheb_m = 1;
    }
    // next level: P^T A P = Acc + Acf W + W^T Afc + W^T Aff W
    const Csr WT = transpose(W);
    // AfP = the F rows of A P = Aff W + A_FC; the next level's matrix is
    // P^T A P = W^T AfP + Acf W + Acc
    const Csr AfP = add(multiply(Aff, W), Afc);
    Csr Ac = add(add(Acc, multiply(Acf, W)), multiply(WT, AfP));
    store(W, L.w_ptr, L.w_idx, L.w_val);
    store(WT, L.wt_ptr, L.wt_idx, L.wt_val);
    store(AfP, L.afc_ptr, L.afc_idx, L.afc_val);
    store(Aff, L.aff_ptr, L.aff_idx, L.aff_val);
    P.off.push_back(P.off.back() + nf);
    P.lev.push_back(std::move(L));
    A = std::move(Ac);
    cur.swap(next);
  }
  err = "amg: the hierarchy did not reach one unknown";
  return NEKGPU_EINVAL;
}

// amg_exec (core/crs_amg.c:129-186) on the host, in the plan's order: b, x of
// n values (b is overwritten).  The device applies the same steps.
void amg_apply_host(const AmgPlan& P, double* x, double* b) {
  const int nl = (int)P.lev.size();
  std::vector<double> buf, c, cold, r;
  for (int l = 0; l + 1 < nl; ++l) {  // b_{l+1} += W^T b_l
    const AmgLevel& L = P.lev[(size_t)l];
    const int64_t o = P.off[(size_t)l], oc = P.off[(size_t)l + 1];
    for (int64_t j = 0; j < L.nc; ++j) {
      double s = 0.0;
      for (int64_t q = L.wt_ptr[(size_t)j]; q < L.wt_ptr[(size_t)j + 1]; ++q)
        s += L.wt_val[(size_t)q] * b[o + L.wt_idx[(size_t)q]];
      b[oc + j] += s;
    }
  }
  {
    const int64_t i = P.off[(size_t)nl - 1];
    x[i] = P.lev[(size_t)nl - 1].dff[0] * b[i];
  }
  for (int l = nl - 2; l >= 0; --l) {
    const AmgLevel& L = P.lev[(size_t)l];
    const int64_t o = P.off[(size_t)l], oc = P.off[(size_t)l + 1], nf = L.nf;
    double* bl = b + o;
    double* xl = x + o;
    const double* xc = x + oc;
    for (int64_t i = 0; i < nf; ++i) {  // x_l = W x_c ; b_l -= AfP x_c
      double s = 0.0, t = 0.0;
      for (int64_t q = L.w_ptr[(size_t)i]; q < L.w_ptr[(size_t)i + 1]; ++q)
        s += L.w_val[(size_t)q] * xc[L.w_idx[(size_t)q]];
      for (int64_t q = L.afc_ptr[(size_t)i]; q < L.afc_ptr[(size_t)i + 1]; ++q)
        t += L.afc_val[(size_t)q] * xc[L.afc_idx[(size_t)q]];
      xl[i] = s;
      bl[i] = bl[i] - t;
    }
    c.assign((size_t)nf, 0.0);
    cold.assign((size_t)nf, 0.0);
    r.assign((size_t)nf, 0.0);
    for (int64_t i = 0; i < nf; ++i) c[(size_t)i] = L.dff[(size_t)i] * bl[i];
    auto resid = [&]() {  // r = b_l - Aff c
      for (int64_t i = 0; i < nf; ++i) {
        double s = 0.0;
        for (int64_t q = L.aff_ptr[(size_t)i]; q < L.aff_ptr[(size_t)i + 1]; ++q)
          s += L.aff_val[(size_t)q] * c[(size_t)L.aff_idx[(size_t)q]];
        r[(size_t)i] = bl[i] - s;
      }
    };
    const int m = L.cheb_m;
    double alpha = 0.0, beta = 0.0, gamma = 0.0;
    if (m > 1) {
      alpha = L.cheb_rho / 2.0;
      alpha *= alpha;
      gamma = 2.0 * alpha / (1.0 - 2.0 * alpha);
      beta = 1.0 + gamma;
      resid();
      c.swap(cold);
      for (int64_t i = 0; i < nf; ++i)
        c[(size_t)i] = beta * (cold[(size_t)i] + L.dff[(size_t)i] * r[(size_t)i]);
    }
    for (int ci = 3; ci <= m; ++ci) {
      gamma = alpha * beta;
      gamma = gamma / (1.0 - gamma);
      beta = 1.0 + gamma;
      resid();
      c.swap(cold);  // c now holds c_{i-1}
      for (int64_t i = 0; i < nf; ++i)
        c[(size_t)i] = beta * (cold[(size_t)i] + L.dff[(size_t)i] * r[(size_t)i]) - gamma * c[(size_t)i];
    }
    for (int64_t i = 0; i < nf; ++i) xl[i] += c[(size_t)i];
  }
  (void)buf;
}

}  // namespace nekgpu

// ---- host-only inspection entry points (nekmesh.h) ----------------------------
#include <memory>
#include <mutex>

namespace {
std::mutex g_amg_mu;
std::map<int64_t, std::unique_ptr<nekgpu::AmgPlan>> g_amg;
int64_t g_amg_next = 1;

nekgpu::AmgPlan* amg_get(const int64_t* h) {
  if (!h) return nullptr;
  std::lock_guard<std::mutex> lk(g_amg_mu);
  auto it = g_amg.find(*h);
  return it == g_amg.end() ? nullptr : it->second.get();
}
}  // namespace

extern "C" int nekmesh_amg_setup(const int64_t* n, const int64_t* ptr, const int* idx,
                                 const double* val, int64_t* plan) {
  using namespace nekgpu;
  if (!n || !ptr || !idx || !val || !plan || *n < 1)
    return mesh_fail(NEKGPU_EINVAL, "amg_setup: bad arguments");
  std::vector<int64_t> p(ptr, ptr + *n + 1);
  std::vector<int> ix(idx, idx + p[(size_t)*n]);
  std::vector<double> v(val, val + p[(size_t)*n]);
  std::unique_ptr<AmgPlan> a(new AmgPlan());
  std::string err;
  const int rc = amg_setup(*a, *n, p, ix, v, err);
  if (rc) return mesh_fail(rc, err);
  std::lock_guard<std::mutex> lk(g_amg_mu);
  *plan = g_amg_next++;
  g_amg[*plan] = std::move(a);
  return NEKGPU_OK;
}

extern "C" int nekmesh_amg_layout(const int64_t* plan, int* nlev, int64_t* off, int64_t* perm) {
  using namespace nekgpu;
  AmgPlan* a = amg_get(plan);
  if (!a || !nlev) return mesh_fail(NEKGPU_EINVAL, "amg_layout: unknown plan");
  *nlev = (int)a->lev.size();
  if (off) std::copy(a->off.begin(), a->off.end(), off);
  if (perm) std::copy(a->perm.begin(), a->perm.end(), perm);
  return NEKGPU_OK;
}

extern "C" int nekmesh_amg_level(const int64_t* plan, const int* lev, int64_t* sizes, int* m,
                                 double* rho, double* dff, int64_t* w_ptr, int* w_idx,
                                 double* w_val, int64_t* wt_ptr, int* wt_idx, double* wt_val,
                                 int64_t* afc_ptr, int* afc_idx, double* afc_val,
                                 int64_t* aff_ptr, int* aff_idx, double* aff_val) {
  using namespace nekgpu;
  AmgPlan* a = amg_get(plan);
  if (!a || !lev || *lev < 0 || *lev >= (int)a->lev.size() || !sizes)
    return mesh_fail(NEKGPU_EINVAL, "amg_level: bad arguments");
  const AmgLevel& L = a->lev[(size_t)*lev];
  sizes[0] = L.nf;
  sizes[1] = L.nc;
  sizes[2] = (int64_t)L.w_idx.size();
  sizes[3] = (int64_t)L.wt_idx.size();
  sizes[4] = (int64_t)L.afc_idx.size();
  sizes[5] = (int64_t)L.aff_idx.size();
  if (m) *m = L.cheb_m;
  if (rho) *rho = L.cheb_rho;
  auto cp = [](const auto& v, auto* out) {
    if (out) std::copy(v.begin(), v.end(), out);
  };
  cp(L.dff, dff);
  cp(L.w_ptr, w_ptr);
  cp(L.w_idx, w_idx);
  cp(L.w_val, w_val);
  cp(L.wt_ptr, wt_ptr);
  cp(L.wt_idx, wt_idx);
  cp(L.wt_val, wt_val);
  cp(L.afc_ptr, afc_ptr);
  cp(L.afc_idx, afc_idx);
  cp(L.afc_val, afc_val);
  cp(L.aff_ptr, aff_ptr);
  cp(L.aff_idx, aff_idx);
  cp(L.aff_val, aff_val);
  return NEKGPU_OK;
}

extern "C" int nekmesh_amg_apply(const int64_t* plan, double* x, double* b) {
  using namespace nekgpu;
  AmgPlan* a = amg_get(plan);
  if (!a || !x || !b) return mesh_fail(NEKGPU_EINVAL, "amg_apply: bad arguments");
  amg_apply_host(*a, x, b);
  return NEKGPU_OK;
}

extern "C" int nekmesh_amg_free(int64_t* plan) {
  using namespace nekgpu;
  if (!plan) return mesh_fail(NEKGPU_EINVAL, "amg_free: null");
  std::lock_guard<std::mutex> lk(g_amg_mu);
  g_amg.erase(*plan);
  *plan = 0;
  return NEKGPU_OK;
}
