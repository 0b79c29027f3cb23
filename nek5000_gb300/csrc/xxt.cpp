// xxt.cpp -- the coarse solve's factor A^-1 = X X^T (the form of crs_xxt,
// core/crs_xxt.c:863-975, after Tufo and Fischer), on one process: the
// unknowns are ordered by nested dissection (recursive coordinate bisection,
// each separator numbered after the two halves it separates), A = L L^T is
// factored in that order (up-looking sparse Cholesky over the elimination
// tree, as in T. Davis, "Direct Methods for Sparse Linear Systems", SIAM
// 2006, ch. 4), and X = L^-T column by column: column j is non-zero only on
// the descendants of j in the elimination tree, so X stays sparse -- about
// n^(5/3) entries for a 3-D vertex grid against n^2 for a dense inverse.
// The device applies x = X (X^T b) as two row-parallel sparse products.
#include <algorithm>
#include <cmath>
#include <numeric>
#include <thread>

#include "h1mg.h"
#include "nekgpu.h"

namespace nekgpu {
namespace {

// nested dissection by coordinate bisection on the graph (ptr, idx)
struct Nd {
  const std::vector<int64_t>& ptr;
  const std::vector<int>& idx;
  const double* xyz;
  std::vector<int> side;  // scratch: 0 none, 1 left, 2 right
  std::vector<int> order;

  void run(std::vector<int>& nodes) {
    if (nodes.size() <= 48) {
      std::sort(nodes.begin(), nodes.end());
      order.insert(order.end(), nodes.begin(), nodes.end());
      return;
    }
    double lo[3], hi[3];
    for (int d = 0; d < 3; ++d) {
      lo[d] = hi[d] = xyz[3 * (size_t)nodes[0] + d];
    }
    for (int v : nodes)
      for (int d = 0; d < 3; ++d) {
        lo[d] = std::min(lo[d], xyz[3 * (size_t)v + d]);
        hi[d] = std::max(hi[d], xyz[3 * (size_t)v + d]);
      }
    int ax = 0;
    for (int d = 1; d < 3; ++d)
      if (hi[d] - lo[d] > hi[ax] - lo[ax]) ax = d;
    std::vector<int> s(nodes);
    const size_t mid = s.size() / 2;
    std::nth_element(s.begin(), s.begin() + mid, s.end(), [&](int a, int b) {
      const double xa = xyz[3 * (size_t)a + ax], xb = xyz[3 * (size_t)b + ax];
      return xa < xb || (xa == xb && a < b);
    });
    for (size_t q = 0; q < s.size(); ++q) side[s[q]] = q < mid ? 1 : 2;
    std::vector<int> L, R, S;
    for (int v : nodes) {
      if (side[v] == 2) {
        R.push_back(v);
        continue;
      }
      bool sep = false;
      for (int64_t q = ptr[v]; q < ptr[v + 1] && !sep; ++q) sep = side[idx[q]] == 2;
      (sep ? S : L).push_back(v);
    }
    for (int v : nodes) side[v] = 0;
    if (L.empty() || R.empty()) {  // no split possible: number as is
      std::sort(nodes.begin(), nodes.end());
      order.insert(order.end(), nodes.begin(), nodes.end());
      return;
    }
    run(L);
    run(R);
    std::sort(S.begin(), S.end());
    order.insert(order.end(), S.begin(), S.end());
  }
};

template <typename F>
void parallel_cols(int64_t n, F&& f) {
  unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  if (n < 256) nt = 1;
  if (nt == 1) {
    for (int64_t j = 0; j < n; ++j) f(j);
    return;
  }
  std::vector<std::thread> th;
  for (unsigned t = 0; t < nt; ++t)
    th.emplace_back([&, t]() {
      for (int64_t j = (int64_t)n - 1 - t; j >= 0; j -= nt) f(j);  // large columns first
    });
  for (auto& x : th) x.join();
}

}  // namespace

int xxt_factor(XxtFactor& f, int64_t n, const std::vector<int64_t>& ptr,
               const std::vector<int>& idx, const std::vector<double>& val, const double* xyz,
               std::string& err) {
  f = XxtFactor();
  f.n = n;
  if (n == 0) {
    f.cptr.assign(1, 0);
    f.rptr.assign(1, 0);
    return NEKGPU_OK;
  }
  // ---- ordering
  Nd nd{ptr, idx, xyz, std::vector<int>((size_t)n, 0), {}};
  std::vector<int> all((size_t)n);
  std::iota(all.begin(), all.end(), 0);
  nd.run(all);
  f.perm = nd.order;  // new -> old
  std::vector<int> inv((size_t)n);
  for (int64_t k = 0; k < n; ++k) inv[f.perm[k]] = (int)k;
  // ---- permuted upper triangle by columns: for column k, rows i <= k
  std::vector<std::vector<std::pair<int, double>>> up((size_t)n);
  for (int64_t r = 0; r < n; ++r)
    for (int64_t q = ptr[r]; q < ptr[r + 1]; ++q) {
      const int a = inv[r], b = inv[idx[q]];
      if (a <= b) up[b].push_back({a, val[q]});
    }
  // ---- elimination tree (Davis, cs_etree)
  std::vector<int> parent((size_t)n, -1), anc((size_t)n, -1);
  for (int64_t k = 0; k < n; ++k)
    for (auto& e : up[k]) {
      int i = e.first;
      while (i != -1 && i < k) {
        const int next = anc[i];
        anc[i] = (int)k;
        if (next == -1) parent[i] = (int)k;
        i = next;
      }
    }
  // ---- up-looking Cholesky: row k of L from the sparse solve L11 x = A(0:k, k)
  std::vector<std::vector<std::pair<int, double>>> col((size_t)n);  // L(i, j), i > j, by column j
  std::vector<double> diag((size_t)n), x((size_t)n, 0.0);
  std::vector<int> mark((size_t)n, -1), stack, pat;
  for (int64_t k = 0; k < n; ++k) {
    double d = 0.0;
    pat.clear();
    mark[k] = (int)k;
    for (auto& e : up[k]) {
      const int i = e.first;
      if (i == k) {
        d += e.second;
        continue;
      }
      x[i] += e.second;
      stack.clear();  // ereach: walk up the tree from i to a marked node
      int j = i;
      while (mark[j] != k) {
        stack.push_back(j);
        mark[j] = (int)k;
        j = parent[j];
      }
      for (auto it = stack.rbegin(); it != stack.rend(); ++it) pat.push_back(*it);
    }
    // pat holds ascending-path segments appended top-down; a topological
    // order (every j before its ancestors) is the ascending index order
    std::sort(pat.begin(), pat.end());
    for (int j : pat) {
      const double lkj = x[j] / diag[j];
      x[j] = 0.0;
      for (auto& e : col[j])
        if (e.first < k) x[e.first] -= e.second * lkj;
      d -= lkj * lkj;
      col[j].push_back({(int)k, lkj});
    }
    if (!(d > 0.0)) {
      err = "coarse factor: matrix not positive definite";
      return NEKGPU_EINVAL;
    }
    diag[k] = std::sqrt(d);
  }
  // ---- X = L^-T: column j solves L^T x = e_j; non-zero on the subtree of j,
  // which lies in [first[j], j]
  std::vector<int> first((size_t)n);
  for (int64_t j = 0; j < n; ++j) first[j] = (int)j;
  for (int64_t j = 0; j < n; ++j)
    if (parent[j] >= 0) first[parent[j]] = std::min(first[parent[j]], first[j]);
  std::vector<std::vector<std::pair<int, double>>> xc((size_t)n);
  parallel_cols(n, [&](int64_t j) {
    const int lo = first[j];
    std::vector<double> v((size_t)(j - lo + 1), 0.0);
    v[j - lo] = 1.0 / diag[j];
    for (int64_t i = j - 1; i >= lo; --i) {
      double s = 0.0;
      for (auto& e : col[i]) {
        if (e.first > j) break;  // rows beyond j are zero in this column
        s += e.second * v[e.first - lo];
      }
      v[i - lo] = -s / diag[i];
    }
    auto& out = xc[j];
    for (int64_t i = lo; i <= j; ++i)
      if (v[i - lo] != 0.0) out.push_back({(int)i, v[i - lo]});
  });
  // ---- both layouts: columns (X^T b) and rows (X y)
  f.cptr.assign((size_t)n + 1, 0);
  for (int64_t j = 0; j < n; ++j) f.cptr[j + 1] = f.cptr[j] + (int64_t)xc[j].size();
  f.cidx.resize(f.cptr[n]);
  f.cval.resize(f.cptr[n]);
  f.rptr.assign((size_t)n + 1, 0);
  for (int64_t j = 0; j < n; ++j) {
    int64_t q = f.cptr[j];
    for (auto& e : xc[j]) {
      f.cidx[q] = e.first;
      f.cval[q] = e.second;
      ++q;
      ++f.rptr[e.first + 1];
    }
  }
  for (int64_t i = 0; i < n; ++i) f.rptr[i + 1] += f.rptr[i];
  f.ridx.resize(f.rptr[n]);
  f.rval.resize(f.rptr[n]);
  std::vector<int64_t> fill(f.rptr.begin(), f.rptr.end() - 1);
  for (int64_t j = 0; j < n; ++j)  // ascending j within every row
    for (auto& e : xc[j]) {
      f.ridx[fill[e.first]] = (int)j;
      f.rval[fill[e.first]] = e.second;
      ++fill[e.first];
    }
  return NEKGPU_OK;
}

}  // namespace nekgpu

// ---- host-only entry point (nekmesh.h) -----------------------------------------
extern "C" int nekmesh_xxt_factor(const int64_t* n, const int64_t* ptr, const int* idx,
                                  const double* val, const double* xyz, int64_t* nnz, int* perm,
                                  int64_t* cptr, int* cidx, double* cval) {
  using namespace nekgpu;
  if (!n || !ptr || !idx || !val || !xyz || !nnz || *n < 0)
    return mesh_fail(NEKGPU_EINVAL, "xxt_factor: bad arguments");
  std::vector<int64_t> p(ptr, ptr + *n + 1);
  std::vector<int> ix(idx, idx + p[*n]);
  std::vector<double> v(val, val + p[*n]);
  XxtFactor f;
  std::string err;
  const int rc = xxt_factor(f, *n, p, ix, v, xyz, err);
  if (rc) return mesh_fail(rc, err);
  *nnz = f.cptr[*n];
  if (perm) std::copy(f.perm.begin(), f.perm.end(), perm);
  if (cptr) std::copy(f.cptr.begin(), f.cptr.end(), cptr);
  if (cidx) std::copy(f.cidx.begin(), f.cidx.end(), cidx);
  if (cval) std::copy(f.cval.begin(), f.cval.end(), cval);
  return NEKGPU_OK;
}
