// h1mg_plan.cpp -- host setup of the pressure preconditioner h1mg_solve
// (core/hsmg.f:1855-1949, if_hybrid = .false., as hmh_gmres and hmh_flex_cg
// call it).  Computes once, on the host, what the device apply (h1mg.cu)
// reads: per level the numbering and extended numbering (setupds through
// set_vert, core/dssum.f:1-31), the Dirichlet mask (h1mg_setup_mask
// :2426-2508), restriction weights (hsmg_setup_rstr_wt :987-1067), Schwarz
// weights (h1mg_setup_schwarz_wt_1 :3048-3104), the fast-diagonalisation
// eigenvectors and inverse eigenvalue sums of every element
// (hsmg_setup_fast :701-781) from the element widths (swap_lengths,
// core/fast3d.f:1542-1617), the interpolation matrices (hsmg_setup_intp
// :83-120), and the coarse Galerkin matrix with its X X^T factor (xxt.cpp;
// crs_setup, core/crs_xxt.c:863).
// Compiled without fused multiply-adds (x86 and aarch64 hosts round alike).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <thread>

#include "h1mg.h"
#include "nekgpu.h"
#include "nekmesh.h"

namespace nekgpu {
namespace {

// f(e) for every element, elements split into contiguous chunks over the
// host's threads (each element's output is its own)
template <typename F>
void parallel_elements(int nel, F&& f) {
  unsigned nt = std::max(1u, std::min(64u, std::thread::hardware_concurrency()));
  if (nel < 64) nt = 1;
  if (nt == 1) {
    for (int e = 0; e < nel; ++e) f(e);
    return;
  }
  std::vector<std::thread> th;
  const int chunk = (nel + (int)nt - 1) / (int)nt;
  for (unsigned t = 0; t < nt; ++t)
    th.emplace_back([&, t]() {
      const int e1 = std::min(nel, (int)(t + 1) * chunk);
      for (int e = (int)t * chunk; e < e1; ++e) f(e);
    });
  for (auto& x : th) x.join();
}

// Fornberg's weights (B. Fornberg, SIAM Review 40 (1998) 685-691), the
// recursion fd_weights_full (core/fast3d.f:1294) evaluates: c[j + (n+1) k]
// is the weight of x[j] in the k-th derivative at xx, k <= m.
void fd_weights(double xx, const double* x, int n, int m, double* c) {
  const int ld = n + 1;
  for (int k = 0; k <= m; ++k)
    for (int j = 0; j <= n; ++j) c[j + ld * k] = 0.0;
  double c1 = 1.0, c4 = x[0] - xx;
  c[0] = 1.0;
  for (int i = 1; i <= n; ++i) {
    const int mn = std::min(i, m);
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

// GLL points (roots of (1 - x^2) P'_N, Newton on the Chebyshev-Gauss-Lobatto
// guess) and weights 2 / (N (N+1) P_N(x)^2).
void gll(int np, double* z, double* w) {
  const int N = np - 1;
  for (int i = 0; i < np; ++i) {
    double x = -std::cos(M_PI * i / N);
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = x;  // P_{k-1}, P_k
      for (int k = 1; k < N; ++k) {
        const double p2 = ((2 * k + 1) * x * p1 - k * p0) / (k + 1);
        p0 = p1;
        p1 = p2;
      }
      // f = (x P_N - P_{N-1}), proportional to (1 - x^2) P'_N; f' = (N+1) P_N
      const double dx = (x * p1 - p0) / ((N + 1) * p1);
      x -= dx;
      if (std::fabs(dx) < 1e-16) break;
    }
    z[i] = x;
  }
  z[0] = -1.0;
  z[N] = 1.0;
  for (int i = 0; i < np; ++i) {
    double p0 = 1.0, p1 = z[i];
    for (int k = 1; k < N; ++k) {
      const double p2 = ((2 * k + 1) * z[i] * p1 - k * p0) / (k + 1);
      p0 = p1;
      p1 = p2;
    }
    w[i] = 2.0 / (N * (N + 1) * p1 * p1);
  }
}

// Symmetric eigenproblem by cyclic Jacobi rotations: a (n x n, column-major)
// is destroyed; lam ascending; V columns the eigenvectors in that order.
void jacobi_eig(std::vector<double>& a, int n, double* lam, std::vector<double>& V) {
  std::vector<double> v((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) v[i + n * i] = 1.0;
  auto A = [&](int i, int j) -> double& { return a[i + (size_t)n * j]; };
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        tot += A(i, j) * A(i, j);
        if (i != j) off += A(i, j) * A(i, j);
      }
    if (off <= 1e-32 * tot) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A(p, q);
        if (apq == 0.0) continue;
        const double theta = (A(q, q) - A(p, p)) / (2.0 * apq);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          const double akp = A(k, p), akq = A(k, q);
          A(k, p) = c * akp - s * akq;
          A(k, q) = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          const double apk = A(p, k), aqk = A(q, k);
          A(p, k) = c * apk - s * aqk;
          A(q, k) = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          const double vkp = v[k + (size_t)n * p], vkq = v[k + (size_t)n * q];
          v[k + (size_t)n * p] = c * vkp - s * vkq;
          v[k + (size_t)n * q] = s * vkp + c * vkq;
        }
      }
  }
  std::vector<int> ord(n);
  for (int i = 0; i < n; ++i) ord[i] = i;
  std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) { return A(x, x) < A(y, y); });
  V.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) {
    lam[i] = A(ord[i], ord[i]);
    for (int k = 0; k < n; ++k) V[k + (size_t)n * i] = v[k + (size_t)n * ord[i]];
  }
}

// Host gather-scatter for the setup: u <- sum over the copies of each
// non-zero id (op 0) or their product (op 1), in ascending local index.
void host_gs(const std::vector<int64_t>& glo, double* u, int op) {
  const int64_t n = (int64_t)glo.size();
  std::vector<int64_t> ord(n);
  for (int64_t i = 0; i < n; ++i) ord[i] = i;
  std::stable_sort(ord.begin(), ord.end(), [&](int64_t a, int64_t b) { return glo[a] < glo[b]; });
  for (int64_t s = 0; s < n;) {
    int64_t t = s + 1;
    while (t < n && glo[ord[t]] == glo[ord[s]]) ++t;
    if (glo[ord[s]] != 0 && t - s > 1) {
      double acc = u[ord[s]];
      for (int64_t q = s + 1; q < t; ++q) acc = op == 0 ? acc + u[ord[q]] : acc * u[ord[q]];
      for (int64_t q = s; q < t; ++q) u[ord[q]] = acc;
    }
    s = t;
  }
}

int64_t ext_index(int nl, int i, int j, int k) { return i + (int64_t)nl * (j + (int64_t)nl * k); }

// hsmg_extrude on the face regions (:368-423): a1[layer l1] = f1 a1 + f2 a2[layer l2]
void extrude(double* a1, int l1, double f1, const double* a2, int l2, double f2, int nl, int nel) {
  const int64_t nn = (int64_t)nl * nl * nl;
  for (int e = 0; e < nel; ++e) {
    double* u = a1 + e * nn;
    const double* v = a2 + e * nn;
    for (int k = 1; k <= nl - 2; ++k)
      for (int j = 1; j <= nl - 2; ++j) {
        u[ext_index(nl, l1, j, k)] = f1 * u[ext_index(nl, l1, j, k)] + f2 * v[ext_index(nl, l2, j, k)];
        u[ext_index(nl, nl - 1 - l1, j, k)] =
            f1 * u[ext_index(nl, nl - 1 - l1, j, k)] + f2 * v[ext_index(nl, nl - 1 - l2, j, k)];
      }
    for (int k = 1; k <= nl - 2; ++k)
      for (int i = 1; i <= nl - 2; ++i) {
        u[ext_index(nl, i, l1, k)] = f1 * u[ext_index(nl, i, l1, k)] + f2 * v[ext_index(nl, i, l2, k)];
        u[ext_index(nl, i, nl - 1 - l1, k)] =
            f1 * u[ext_index(nl, i, nl - 1 - l1, k)] + f2 * v[ext_index(nl, i, nl - 1 - l2, k)];
      }
    for (int j = 1; j <= nl - 2; ++j)
      for (int i = 1; i <= nl - 2; ++i) {
        u[ext_index(nl, i, j, l1)] = f1 * u[ext_index(nl, i, j, l1)] + f2 * v[ext_index(nl, i, j, l2)];
        u[ext_index(nl, i, j, nl - 1 - l1)] =
            f1 * u[ext_index(nl, i, j, nl - 1 - l1)] + f2 * v[ext_index(nl, i, j, nl - 1 - l2)];
      }
  }
}

}  // namespace

int h1mg_levels(int lx1, int* order) {
  static const int mgn2[10] = {1, 2, 2, 2, 2, 3, 3, 5, 5, 5};
  const int lmax = lx1 == 4 ? 2 : 3;
  int mglx2 = 2 * (lx1 / 4) + 1;  // lx2 = lx1 on the PN-PN pressure
  if (lx1 == 5) mglx2 = 3;
  if (lx1 <= 10) mglx2 = mgn2[std::min(lx1, 10) - 1];
  if (lx1 == 8) mglx2 = 3;
  mglx2 = std::min(3, mglx2);
  order[0] = 1;
  order[1] = mglx2;
  order[2] = mglx2 + 1;
  order[lmax - 1] = lx1 - 1;
  return lmax;
}

void h1mg_face_types(int nx, int nel, const int64_t* glo, const double* mask, int* fbc) {
  const int64_t nxyz = (int64_t)nx * nx * nx, n = nxyz * nel;
  std::vector<int64_t> s(glo, glo + n);
  std::sort(s.begin(), s.end());
  auto shared = [&](int64_t id) {
    if (id == 0) return false;
    auto r = std::equal_range(s.begin(), s.end(), id);
    return r.second - r.first > 1;
  };
  const int m = nx - 1;
  for (int e = 0; e < nel; ++e)
    for (int f = 0; f < 6; ++f) {
      const int fix = (f & 1) ? m : 0;
      int i = 1, j = 1, k = 1;
      if (f < 2) i = fix;
      else if (f < 4) j = fix;
      else k = fix;
      const int64_t p = e * nxyz + i + (int64_t)nx * (j + (int64_t)nx * k);
      fbc[6 * e + f] = shared(glo[p]) ? 0 : (mask[p] == 0.0 ? 1 : 2);
    }
}

void h1mg_fast1d(double* s, double* lam, int lbc, int rbc, double ll, double lm, double lr,
                 const double* ah, const double* bh, int n) {
  const int nl = n + 3, na = n + 1;
  std::vector<double> a((size_t)nl * nl, 0.0), b(nl, 0.0);
  auto A = [&](int i, int j) -> double& { return a[i + (size_t)nl * j]; };
  auto AH = [&](int i, int j) { return ah[i + na * j]; };
  const int i0 = lbc == 1 ? 1 : 0, i1 = rbc == 1 ? n - 1 : n;
  double fac = 2.0 / lm;  // hsmg_setup_fast1d_a
  A(1, 1) = 1.0;
  A(n + 1, n + 1) = 1.0;
  for (int j = i0; j <= i1; ++j)
    for (int i = i0; i <= i1; ++i) A(i + 1, j + 1) = fac * AH(i, j);
  if (lbc == 0) {
    fac = 2.0 / ll;
    A(0, 0) = fac * AH(n - 1, n - 1);
    A(1, 0) = fac * AH(n, n - 1);
    A(0, 1) = fac * AH(n - 1, n);
    A(1, 1) = A(1, 1) + fac * AH(n, n);
  } else {
    A(0, 0) = 1.0;
  }
  if (rbc == 0) {
    fac = 2.0 / lr;
    A(n + 1, n + 1) = A(n + 1, n + 1) + fac * AH(0, 0);
    A(n + 2, n + 1) = fac * AH(1, 0);
    A(n + 1, n + 2) = fac * AH(0, 1);
    A(n + 2, n + 2) = fac * AH(1, 1);
  } else {
    A(n + 2, n + 2) = 1.0;
  }
  fac = 0.5 * lm;  // hsmg_setup_fast1d_b (diagonal)
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
  // A x = lam B x, B diagonal: eigenvectors of B^-1/2 A B^-1/2, scaled back
  std::vector<double> c((size_t)nl * nl), V;
  for (int j = 0; j < nl; ++j)
    for (int i = 0; i < nl; ++i) c[i + (size_t)nl * j] = A(i, j) / std::sqrt(b[i] * b[j]);
  jacobi_eig(c, nl, lam, V);
  for (int j = 0; j < nl; ++j)
    for (int i = 0; i < nl; ++i) s[i + (size_t)nl * j] = V[i + (size_t)nl * j] / std::sqrt(b[i]);
  for (int j = 0; j < nl; ++j) {  // row_zero: excluded points
    if (lbc > 0) s[0 + (size_t)nl * j] = 0.0;
    if (lbc == 1) s[1 + (size_t)nl * j] = 0.0;
    if (rbc > 0) s[nl - 1 + (size_t)nl * j] = 0.0;
    if (rbc == 1) s[nl - 2 + (size_t)nl * j] = 0.0;
  }
}

void h1mg_coarse_basis(int nx1, std::vector<double>& b) {
  std::vector<double> z(nx1), w(nx1);
  gll(nx1, z.data(), w.data());
  const int64_t nxyz = (int64_t)nx1 * nx1 * nx1;
  b.assign(8 * nxyz, 0.0);
  for (int j = 0; j < 8; ++j)
    for (int r = 0; r < nx1; ++r)
      for (int q = 0; q < nx1; ++q)
        for (int p = 0; p < nx1; ++p) {
          const double zr = (j & 1) ? 0.5 * (1 + z[p]) : 0.5 * (1 - z[p]);
          const double zs = (j & 2) ? 0.5 * (1 + z[q]) : 0.5 * (1 - z[q]);
          const double zt = (j & 4) ? 0.5 * (1 + z[r]) : 0.5 * (1 - z[r]);
          b[j * nxyz + p + nx1 * (q + (int64_t)nx1 * r)] = zr * zs * zt;
        }
}

int h1mg_plan(MgPlan& p, int nx1, int nel, const int64_t* glo, const double* x, const double* y,
              const double* z, const double* mask, const int* fbc, bool null_space,
              std::string& err) {
  if (nx1 < 3 || nx1 > 12 || nel <= 0 || !glo || !x || !y || !z || (!fbc && !mask)) {
    err = "h1mg: needs 3 <= lx1 <= 12, the numbering, coordinates and mask or face types";
    return NEKGPU_EINVAL;
  }
  p = MgPlan();
  p.nx1 = nx1;
  p.nel = nel;
  p.null_space = null_space;
  p.lmax = h1mg_levels(nx1, p.order);
  const int64_t nxyz = (int64_t)nx1 * nx1 * nx1, n = nxyz * nel;
  p.fbc.resize(6 * (size_t)nel);
  if (fbc) std::memcpy(p.fbc.data(), fbc, sizeof(int) * 6 * nel);
  else h1mg_face_types(nx1, nel, glo, mask, p.fbc.data());
  for (int q = 0; q < 6 * nel; ++q)
    if (p.fbc[q] < 0 || p.fbc[q] > 2) {
      err = "h1mg: face types must be 0, 1 or 2";
      return NEKGPU_EINVAL;
    }
  // vertex ids: the fine numbering at the corners, ranked 1..nv
  p.vrank.resize(8 * (size_t)nel);
  for (int e = 0; e < nel; ++e)
    for (int c = 0; c < 8; ++c) {
      const int i = (c & 1) * (nx1 - 1), j = ((c >> 1) & 1) * (nx1 - 1), k = (c >> 2) * (nx1 - 1);
      p.vrank[8 * e + c] = glo[e * nxyz + i + nx1 * (j + (int64_t)nx1 * k)];
    }
  {
    std::vector<int64_t> s(p.vrank);
    std::sort(s.begin(), s.end());
    s.erase(std::unique(s.begin(), s.end()), s.end());
    if (!s.empty() && s.front() <= 0) {
      err = "h1mg: an element corner has numbering id 0";
      return NEKGPU_EINVAL;
    }
    for (auto& v : p.vrank) v = (std::lower_bound(s.begin(), s.end(), v) - s.begin()) + 1;
  }
  // element widths (swap_lengths): harmonic-mean face distances over the
  // interior points, weighted by the GLL weight one index lower (plane_space
  // :306-423 indexes w from 1 over points 1..lx1-2), and the neighbours'
  // widths across each face from a dssum of the widths on the face interiors
  std::vector<double> zf(nx1), wf(nx1);
  gll(nx1, zf.data(), wf.data());
  p.lenl.assign(3 * (size_t)nel, 0.0);
  p.lenm.assign(3 * (size_t)nel, 0.0);
  p.lenr.assign(3 * (size_t)nel, 0.0);
  const int m = nx1 - 2, n2 = nx1 - 1;
  auto P = [&](int i, int j, int k) { return (int64_t)i + nx1 * (j + (int64_t)nx1 * k); };
  for (int e = 0; e < nel; ++e) {
    const double *xe = x + e * nxyz, *ye = y + e * nxyz, *ze = z + e * nxyz;
    for (int d = 0; d < 3; ++d) {
      double l2 = 0.0, wsum = 0.0;
      for (int b = 1; b <= m; ++b)
        for (int a = 1; a <= m; ++a) {
          const double weight = wf[a - 1] * wf[b - 1];
          int64_t p1, p2;
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
      p.lenm[3 * e + d] = 1.0 / std::sqrt(l2);
    }
  }
  {
    std::vector<int64_t> gf(glo, glo + n);
    std::vector<double> l((size_t)n, 0.0);
    for (int e = 0; e < nel; ++e) {
      double* le = l.data() + e * nxyz;
      for (int j = 1; j <= m; ++j)
        for (int k = 1; k <= m; ++k) {
          le[P(0, k, j)] = p.lenm[3 * e];
          le[P(n2, k, j)] = p.lenm[3 * e];
          le[P(k, 0, j)] = p.lenm[3 * e + 1];
          le[P(k, n2, j)] = p.lenm[3 * e + 1];
          le[P(k, j, 0)] = p.lenm[3 * e + 2];
          le[P(k, j, n2)] = p.lenm[3 * e + 2];
        }
    }
    host_gs(gf, l.data(), 0);
    for (int e = 0; e < nel; ++e) {
      const double* le = l.data() + e * nxyz;
      p.lenl[3 * e] = le[P(0, 1, 1)] - p.lenm[3 * e];
      p.lenr[3 * e] = le[P(n2, 1, 1)] - p.lenm[3 * e];
      p.lenl[3 * e + 1] = le[P(1, 0, 1)] - p.lenm[3 * e + 1];
      p.lenr[3 * e + 1] = le[P(1, n2, 1)] - p.lenm[3 * e + 1];
      p.lenl[3 * e + 2] = le[P(1, 1, 0)] - p.lenm[3 * e + 2];
      p.lenr[3 * e + 2] = le[P(1, 1, n2)] - p.lenm[3 * e + 2];
    }
  }
  for (int l = 0; l < p.lmax; ++l) {
    MgLevelPlan& L = p.lev[l];
    const int N = p.order[l], nx = N + 1, nl = nx + 2;
    const int64_t lxyz = (int64_t)nx * nx * nx, nn = (int64_t)nl * nl * nl;
    L.nx = nx;
    L.n = lxyz * nel;
    L.z.resize(nx);
    L.w.resize(nx);
    gll(nx, L.z.data(), L.w.data());
    std::vector<double> c(2 * (size_t)(nx + 16)), D((size_t)nx * nx);  // semhat
    for (int i = 0; i <= N; ++i) {
      fd_weights(L.z[i], L.z.data(), N, 1, c.data());
      for (int j = 0; j <= N; ++j) D[i + (size_t)nx * j] = c[j + nx];
    }
    L.ah.assign((size_t)nx * nx, 0.0);
    for (int j = 0; j <= N; ++j)
      for (int i = 0; i <= N; ++i) {
        double a = 0.0;
        for (int k = 0; k <= N; ++k) a = a + D[k + (size_t)nx * i] * L.w[k] * D[k + (size_t)nx * j];
        L.ah[i + (size_t)nx * j] = a;
      }
    if (l > 0) {
      const MgLevelPlan& C = p.lev[l - 1];
      const int nc = C.nx;
      L.jh.assign((size_t)nx * nc, 0.0);
      for (int i = 0; i < nx; ++i) {
        fd_weights(L.z[i], C.z.data(), nc - 1, 1, c.data());
        for (int j = 0; j < nc; ++j) L.jh[i + (size_t)nx * j] = c[j];
      }
    }
    // numberings
    int64_t ngv = 0;
    L.glo.resize(L.n);
    int rc = nekmesh_setvert3d(&nx, &nel, p.vrank.data(), L.glo.data(), &ngv);
    L.glo_ext.resize(nn * nel);
    if (!rc) rc = nekmesh_setvert3d(&nl, &nel, p.vrank.data(), L.glo_ext.data(), &ngv);
    if (rc) {
      err = "h1mg: level numbering failed";
      return rc;
    }
    // mask: Dirichlet faces zeroed, then the product over the copies
    L.mask.assign(L.n, 1.0);
    for (int e = 0; e < nel; ++e)
      for (int f = 0; f < 6; ++f) {
        if (p.fbc[6 * e + f] != 1) continue;
        const int fix = (f & 1) ? nx - 1 : 0;
        for (int b = 0; b < nx; ++b)
          for (int a = 0; a < nx; ++a) {
            int64_t q;
            if (f < 2) q = fix + (int64_t)nx * (a + (int64_t)nx * b);
            else if (f < 4) q = a + (int64_t)nx * (fix + (int64_t)nx * b);
            else q = a + (int64_t)nx * (b + (int64_t)nx * fix);
            L.mask[e * lxyz + q] = 0.0;
          }
      }
    host_gs(L.glo, L.mask.data(), 1);
    L.rwt.assign(L.n, 1.0);
    host_gs(L.glo, L.rwt.data(), 0);
    for (auto& v : L.rwt) v = 1.0 / v;
    if (l == 0) continue;
    // fast diagonalisation of every element's extended operator
    L.S.assign((size_t)nel * 3 * nl * nl, 0.0);
    L.dinv.assign((size_t)nn * nel, 0.0);
    parallel_elements(nel, [&](int e) {
      double lam[3][32];
      for (int d = 0; d < 3; ++d)
        h1mg_fast1d(L.S.data() + ((size_t)e * 3 + d) * nl * nl, lam[d], p.fbc[6 * e + 2 * d],
                    p.fbc[6 * e + 2 * d + 1], p.lenl[3 * e + d], p.lenm[3 * e + d],
                    p.lenr[3 * e + d], L.ah.data(), L.w.data(), N);
      double mx[3];
      for (int d = 0; d < 3; ++d) {  // the largest of lam[1 .. nl-2]
        mx[d] = lam[d][1];
        for (int i = 2; i <= nl - 2; ++i) mx[d] = std::max(mx[d], lam[d][i]);
      }
      const double eps = 1.e-5 * (mx[0] + mx[1] + mx[2]);
      double* de = L.dinv.data() + e * nn;
      int64_t il = 0;
      for (int k = 0; k < nl; ++k)
        for (int j = 0; j < nl; ++j)
          for (int i = 0; i < nl; ++i) {
            const double diag = lam[0][i] + lam[1][j] + lam[2][k];
            de[il++] = diag > eps ? 1.0 / diag : 0.0;
          }
    });
    // Schwarz weights: 1 / the number of extended subdomains over a point
    std::vector<double> A((size_t)nn * nel, 0.0), B((size_t)nn * nel, 1.0);
    extrude(A.data(), 0, 0.0, B.data(), 0, 1.0, nl, nel);
    host_gs(L.glo_ext, B.data(), 0);
    extrude(B.data(), 0, 1.0, A.data(), 0, -1.0, nl, nel);
    extrude(B.data(), 2, 1.0, B.data(), 0, 1.0, nl, nel);
    L.swt.resize(L.n);
    for (int e = 0; e < nel; ++e)
      for (int k = 0; k < nx; ++k)
        for (int j = 0; j < nx; ++j)
          for (int i = 0; i < nx; ++i)
            L.swt[e * lxyz + i + (int64_t)nx * (j + (int64_t)nx * k)] =
                B[e * nn + ext_index(nl, i + 1, j + 1, k + 1)];
    host_gs(L.glo, L.swt.data(), 0);
    for (auto& v : L.swt) v = 1.0 / v;
  }
  // coarse unknowns: the unmasked level-0 ids in ascending order
  const MgLevelPlan& C = p.lev[0];
  std::vector<int64_t> ids;
  for (int64_t i = 0; i < C.n; ++i)
    if (C.mask[i] >= 0.1) ids.push_back(C.glo[i]);
  std::sort(ids.begin(), ids.end());
  ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
  p.nc = (int64_t)ids.size();
  p.nsolve = (null_space && p.nc > 0) ? p.nc - 1 : p.nc;
  if (p.nc >= (int64_t)1 << 31) {
    err = "h1mg: more than 2^31 - 1 coarse unknowns";
    return NEKGPU_EINVAL;
  }
  p.cid.assign(C.n, -1);
  p.ccoord.assign(3 * (size_t)p.nc, 0.0);
  for (int64_t i = 0; i < C.n; ++i)
    if (C.mask[i] >= 0.1) {
      const int64_t c = std::lower_bound(ids.begin(), ids.end(), C.glo[i]) - ids.begin();
      p.cid[i] = c;
      const int64_t e = i / 8, cr = i % 8;  // level-0 point = element corner cr
      const int64_t q = e * nxyz + (cr & 1) * (nx1 - 1) + nx1 * (((cr >> 1) & 1) * (nx1 - 1)) +
                        (int64_t)nx1 * nx1 * ((cr >> 2) * (nx1 - 1));
      p.ccoord[3 * c] = x[q];
      p.ccoord[3 * c + 1] = y[q];
      p.ccoord[3 * c + 2] = z[q];
    }
  return NEKGPU_OK;
}

int h1mg_plan_coarse(MgPlan& p, const double* elem, std::string& err) {
  const int64_t ns = p.nsolve;
  // assemble the unknowns below nsolve (the pinned one left out) by rows
  std::vector<std::vector<std::pair<int, double>>> rows((size_t)ns);
  for (int e = 0; e < p.nel; ++e)
    for (int j = 0; j < 8; ++j)
      for (int i = 0; i < 8; ++i) {
        const int64_t ci = p.cid[8 * e + i], cj = p.cid[8 * e + j];
        if (ci >= 0 && cj >= 0 && ci < ns && cj < ns)
          rows[ci].push_back({(int)cj, elem[64 * (size_t)e + i + 8 * j]});
      }
  std::vector<int64_t> ptr((size_t)ns + 1, 0);
  std::vector<int> idx;
  std::vector<double> val;
  for (int64_t r = 0; r < ns; ++r) {
    auto& v = rows[r];
    std::stable_sort(v.begin(), v.end(),
                     [](const std::pair<int, double>& a, const std::pair<int, double>& b) {
                       return a.first < b.first;
                     });
    for (size_t q = 0; q < v.size();) {  // duplicates summed in element order
      double a = 0.0;
      const int c = v[q].first;
      for (; q < v.size() && v[q].first == c; ++q) a += v[q].second;
      idx.push_back(c);
      val.push_back(a);
    }
    ptr[r + 1] = (int64_t)idx.size();
    std::vector<std::pair<int, double>>().swap(v);
  }
  const int rc = p.use_amg ? amg_setup(p.amg, ns, ptr, idx, val, err)
                           : xxt_factor(p.xxt, ns, ptr, idx, val, p.ccoord.data(), err);
  if (rc && err.find("positive") != std::string::npos)
    err = "h1mg: the coarse matrix is not positive definite (a null space without null_space?)";
  return rc;
}

}  // namespace nekgpu

// ---- host-only entry points (nekmesh.h) --------------------------------------
using namespace nekgpu;

extern "C" int nekmesh_h1mg_levels(const int* lx1, int* order) {
  if (!lx1 || !order || *lx1 < 3 || *lx1 > 12)
    return mesh_fail(NEKGPU_EINVAL, "h1mg_levels: needs 3 <= lx1 <= 12");
  int o[kMgMaxLev];
  const int lmax = h1mg_levels(*lx1, o);
  for (int l = 0; l < lmax; ++l) order[l] = o[l];
  return lmax;
}

extern "C" int nekmesh_face_types(const int* nx, const int* nel, const int64_t* glo_num,
                                  const double* mask, int* fbc) {
  if (!nx || !nel || !glo_num || !mask || !fbc || *nx < 3 || *nel < 1)
    return mesh_fail(NEKGPU_EINVAL, "face_types: bad arguments (nx >= 3)");
  h1mg_face_types(*nx, *nel, glo_num, mask, fbc);
  return NEKGPU_OK;
}

extern "C" int nekmesh_h1mg_level(const int* nx1, const int* nel, const int64_t* glo_num,
                                  const double* x, const double* y, const double* z,
                                  const double* mask, const int* fbc, const int* level, int* nx,
                                  double* lmask, double* rwt, double* swt, double* lengths) {
  if (!nx1 || !nel || !level || !nx) return mesh_fail(NEKGPU_EINVAL, "h1mg_level: null argument");
  MgPlan p;
  std::string err;
  const int rc = h1mg_plan(p, *nx1, *nel, glo_num, x, y, z, mask, fbc, false, err);
  if (rc) return mesh_fail(rc, err);
  if (*level < 0 || *level >= p.lmax) return mesh_fail(NEKGPU_EINVAL, "h1mg_level: no such level");
  const MgLevelPlan& L = p.lev[*level];
  *nx = L.nx;
  if (lmask) std::copy(L.mask.begin(), L.mask.end(), lmask);
  if (rwt) std::copy(L.rwt.begin(), L.rwt.end(), rwt);
  if (swt) {
    if (L.swt.empty()) std::fill(swt, swt + L.n, 0.0);
    else std::copy(L.swt.begin(), L.swt.end(), swt);
  }
  if (lengths)
    for (int e = 0; e < *nel; ++e)
      for (int d = 0; d < 3; ++d) {
        lengths[9 * e + d] = p.lenl[3 * e + d];
        lengths[9 * e + 3 + d] = p.lenm[3 * e + d];
        lengths[9 * e + 6 + d] = p.lenr[3 * e + d];
      }
  return NEKGPU_OK;
}

extern "C" int nekmesh_fdm1d(const int* n, const int* lbc, const int* rbc, const double* ll,
                             const double* lm, const double* lr, double* s, double* lam) {
  if (!n || !lbc || !rbc || !ll || !lm || !lr || !s || !lam || *n < 1 || *n > 13)
    return mesh_fail(NEKGPU_EINVAL, "fdm1d: bad arguments (1 <= n <= 13)");
  const int N = *n, nx = N + 1;
  std::vector<double> z(nx), w(nx), c(2 * (size_t)nx), D((size_t)nx * nx), ah((size_t)nx * nx);
  gll(nx, z.data(), w.data());
  for (int i = 0; i <= N; ++i) {
    fd_weights(z[i], z.data(), N, 1, c.data());
    for (int j = 0; j <= N; ++j) D[i + (size_t)nx * j] = c[j + nx];
  }
  for (int j = 0; j <= N; ++j)
    for (int i = 0; i <= N; ++i) {
      double a = 0.0;
      for (int k = 0; k <= N; ++k) a = a + D[k + (size_t)nx * i] * w[k] * D[k + (size_t)nx * j];
      ah[i + (size_t)nx * j] = a;
    }
  h1mg_fast1d(s, lam, *lbc, *rbc, *ll, *lm, *lr, ah.data(), w.data(), N);
  return NEKGPU_OK;
}
