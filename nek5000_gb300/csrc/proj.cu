// proj.cu -- projection of the right-hand side onto previous solutions, the
// caller side of the Helmholtz solve in time stepping (core/navier4.f:562-1188:
// hsolve, project1, project1_a, proj_matvec, proj_ortho,
// proj_ortho_full_cgs2, project2, project2_a, givens_rotation, hypot).
//
// A projection space holds up to mmx solutions X and B = A X, B-orthonormal
// in the weighted inner product (x, y)_w = sum x w y.  Before a solve the
// right-hand side loses its part in span(B) (project1: two rounds of
// classical Gram-Schmidt); after it the solution gets the matching part of
// span(X) back and is appended to the space (project2), which is then
// re-orthonormalised in O(nm) work (proj_ortho: two Gram-Schmidt rounds, a
// rank test, Givens rotations that carry the newest direction into the
// first vector).  When h1 or h2 has changed, B = A X is recomputed and the
// space fully re-orthonormalised (CGS2) first.
//
// GPU form: every vector pass of the reference that runs over the m vectors
// of the space becomes one kernel over all of them -- the m weighted dot
// products share one read of w and of the other operand, the m axpys of a
// Gram-Schmidt round are applied per point in the reference's k order, and
// the m-1 Givens rotations are applied per point in sequence, so X and B are
// read and written once per step.  Pointwise arithmetic is rounded exactly
// as the reference's (no fused multiply-add); the dot products are tree sums
// in FP64 (deterministic, block partials summed in block order on the host).
#include <cmath>
#include <cstring>

#include "impl.cuh"

namespace nekgpu {
namespace {

constexpr int kThreads = 256;
constexpr int kMaxBlocks = 152 * 8;

inline int blocks(int64_t n) {
  return (int)std::min<int64_t>(std::max<int64_t>((n + kThreads - 1) / kThreads, 1), kMaxBlocks);
}

struct Scalars {
  double v[2 * NEKGPU_PROJ_MAX];
};

__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }

// partial[blk * nd + k] = sum over the block's points of A_k w b (k < m) and,
// with C given, partial[blk * nd + m + k] = sum C_k w d; nd = m or 2m.
// A_k = A + k * stride (the space's vectors are stored back to back).
__global__ void __launch_bounds__(kThreads)
    multidot_kernel(const double* __restrict__ A, const double* __restrict__ C, int64_t stride,
                    int m, const double* __restrict__ w, const double* __restrict__ b,
                    const double* __restrict__ d, int64_t n, double* __restrict__ partial) {
  __shared__ double red[kThreads / 32][2 * NEKGPU_PROJ_MAX];
  const int nd = C ? 2 * m : m;
  double acc[2 * NEKGPU_PROJ_MAX];
#pragma unroll
  for (int k = 0; k < 2 * NEKGPU_PROJ_MAX; ++k) acc[k] = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kThreads) {
    const double wb = w[i] * b[i];
    const double wd = C ? w[i] * d[i] : 0.0;
#pragma unroll
    for (int k = 0; k < NEKGPU_PROJ_MAX; ++k) {
      if (k < m) {
        acc[k] = fma(A[k * stride + i], wb, acc[k]);
        if (C) acc[NEKGPU_PROJ_MAX + k] = fma(C[k * stride + i], wd, acc[NEKGPU_PROJ_MAX + k]);
      }
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 2 * NEKGPU_PROJ_MAX; ++k) {
    double v = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[wid][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < nd) {
    const int k = threadIdx.x < m ? threadIdx.x : NEKGPU_PROJ_MAX + (threadIdx.x - m);
    double s = red[0][k];
    for (int q = 1; q < kThreads / 32; ++q) s += red[q][k];
    partial[(int64_t)blockIdx.x * nd + threadIdx.x] = s;
  }
}

// project1_a's Gram-Schmidt round (navier4.f:735-825): per point, in the
// reference's k order, xbar (+)= a_k x_k, bbar (+)= a_k b_k, b += (-a_k) b_k.
// first: xbar = a_1 x_1 and bbar = a_1 b_1 (cmult2) start the sums.
__global__ void __launch_bounds__(kThreads)
    combine_kernel(const double* __restrict__ xx, const double* __restrict__ bb, int64_t stride,
                   int m, Scalars a, int first, double* __restrict__ xbar,
                   double* __restrict__ bbar, double* __restrict__ b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kThreads) {
    double xs, bs;
    double bi = b[i];
    int k0 = 0;
    if (first) {
      xs = mul_rn(xx[i], a.v[0]);
      bs = mul_rn(bb[i], a.v[0]);
      bi = add_rn(bi, mul_rn(-a.v[0], bb[i]));
      k0 = 1;
    } else {
      xs = xbar[i];
      bs = bbar[i];
    }
    for (int k = k0; k < m; ++k) {
      const double xk = xx[k * stride + i], bk = bb[k * stride + i];
      xs = add_rn(xs, mul_rn(a.v[k], xk));
      bs = add_rn(bs, mul_rn(a.v[k], bk));
      bi = add_rn(bi, mul_rn(-a.v[k], bk));
    }
    xbar[i] = xs;
    bbar[i] = bs;
    b[i] = bi;
  }
}

// y1 += (-c_k) V1_k and y2 += (-c_k) V2_k for k = order[0], order[1], ...
// (add2s2 with -alpha, in the reference's order).
__global__ void __launch_bounds__(kThreads)
    subtract_kernel(double* __restrict__ y1, double* __restrict__ y2,
                    const double* __restrict__ V1, const double* __restrict__ V2, int64_t stride,
                    int nk, Scalars c, Scalars order, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kThreads) {
    double a = y1[i], b = y2[i];
    for (int q = 0; q < nk; ++q) {
      const int k = (int)order.v[q];
      a = add_rn(a, mul_rn(-c.v[q], V1[k * stride + i]));
      b = add_rn(b, mul_rn(-c.v[q], V2[k * stride + i]));
    }
    y1[i] = a;
    y2[i] = b;
  }
}

__global__ void scale2_kernel(double* __restrict__ a, double* __restrict__ b, double c,
                              int64_t n) {  // cmult (math.f): a = a * c
  for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kThreads) {
    a[i] = mul_rn(a[i], c);
    b[i] = mul_rn(b[i], c);
  }
}

// The Givens rotations of proj_ortho (navier4.f:924-940) on X and B: for
// k = m, m-1, ..., 2 (h = k-1), (v_h, v_k) <- (c v_h + s v_k, -s v_h + c v_k),
// every point independently, the rotations in sequence.  cs.v[2q], cs.v[2q+1]
// = c, s of the rotation for k = m - q.
__global__ void __launch_bounds__(kThreads)
    givens_kernel(double* __restrict__ xx, double* __restrict__ bb, int64_t stride, int m,
                  Scalars cs, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kThreads) {
    for (int q = 0; q < m - 1; ++q) {
      const int k = m - 1 - q, h = k - 1;  // 0-based vector indices
      const double c = cs.v[2 * q], s = cs.v[2 * q + 1];
      double* xh = xx + h * stride + i;
      double* xk = xx + k * stride + i;
      double* bh = bb + h * stride + i;
      double* bk = bb + k * stride + i;
      const double x1 = *xh, x2 = *xk, b1 = *bh, b2 = *bk;
      *xh = add_rn(mul_rn(c, x1), mul_rn(s, x2));
      *xk = add_rn(-mul_rn(s, x1), mul_rn(c, x2));
      *bh = add_rn(mul_rn(c, b1), mul_rn(s, b2));
      *bk = add_rn(-mul_rn(s, b1), mul_rn(c, b2));
    }
  }
}

// partial[2 blk] = max |h1 - h1old|, partial[2 blk + 1] = max |h2 - h2old|
__global__ void maxdiff_kernel(const double* __restrict__ h1, const double* __restrict__ h1o,
                               const double* __restrict__ h2, const double* __restrict__ h2o,
                               int64_t n, double* __restrict__ partial) {
  __shared__ double red[2][kThreads / 32];
  double d1 = 0.0, d2 = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kThreads) {
    d1 = fmax(d1, fabs(h1[i] - h1o[i]));
    d2 = fmax(d2, fabs(h2[i] - h2o[i]));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    d1 = fmax(d1, __shfl_xor_sync(0xffffffffu, d1, o));
    d2 = fmax(d2, __shfl_xor_sync(0xffffffffu, d2, o));
  }
  if ((threadIdx.x & 31) == 0) {
    red[0][threadIdx.x >> 5] = d1;
    red[1][threadIdx.x >> 5] = d2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < kThreads / 32; ++q) {
      d1 = fmax(d1, red[0][q]);
      d2 = fmax(d2, red[1][q]);
    }
    partial[2 * blockIdx.x] = d1;
    partial[2 * blockIdx.x + 1] = d2;
  }
}

__global__ void mask_kernel(double* __restrict__ a, const double* __restrict__ m, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kThreads)
    a[i] = mul_rn(a[i], m[i]);
}

__global__ void add_kernel(double* __restrict__ a, const double* __restrict__ b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)kThreads + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * kThreads)
    a[i] = add_rn(a[i], b[i]);
}

// hypot and givens_rotation (navier4.f:1308-1342, Nek's own hypot)
double nek_hypot(double a, double b) {
  const double c = std::fabs(a), d = std::fabs(b);
  const double x = std::max(c, d);
  const double ix = 1.0 / x;
  double t = std::min(c, d);
  t = ix * t;
  return x * std::sqrt(1.0 + t * t);
}

void givens_rotation(double a, double b, double* c, double* s, double* r) {
  if (b != 0.0) {
    const double h = nek_hypot(a, b);
    const double d = 1.0 / h;
    *c = std::fabs(a) * d;
    *s = std::copysign(d, a) * b;
    *r = std::copysign(1.0, a) * h;
  } else {
    *c = 1.0;
    *s = 0.0;
    *r = a;
  }
}

struct Ctx {
  Handle& h;
  ProjSpace& P;
  const Coef<double>& c;
  const double* msk;
  const double* w;
  int64_t n;
  cudaStream_t s;
  int nb;
  double* X(int k) { return P.xx.ptr + (size_t)k * n; }
  double* B(int k) { return P.bb.ptr + (size_t)k * n; }
};

// Sums of multidot_kernel's block partials, in block order.
int fetch_sums(Ctx& q, int nd, double* out) {
  std::vector<double> hp((size_t)q.nb * nd);
  cudaMemcpyAsync(hp.data(), q.h.red.ptr, hp.size() * sizeof(double), cudaMemcpyDeviceToHost,
                  q.s);
  if (cudaStreamSynchronize(q.s) != cudaSuccess) {
    set_error(q.h, std::string("projection: ") + cudaGetErrorString(cudaGetLastError()));
    return -3;
  }
  for (int k = 0; k < nd; ++k) {
    double t = 0.0;
    for (int b = 0; b < q.nb; ++b) t += hp[(size_t)b * nd + k];
    out[k] = t;
  }
  return 0;
}

// out[k] = (A_k, b)_w for k < m (A_k = A + k n)
int dots(Ctx& q, const double* A, int m, const double* b, double* out) {
  if (m <= 0) return 0;
  count_launch();
  multidot_kernel<<<q.nb, kThreads, 0, q.s>>>(A, nullptr, q.n, m, q.w, b, nullptr, q.n,
                                             q.h.red.ptr);
  return fetch_sums(q, m, out);
}

// out[k] = 0.5 ((X_k, bm)_w + (B_k, xm)_w) for k < m
int sym_dots(Ctx& q, const double* X0, const double* B0, int m, const double* bm,
             const double* xm, double* out) {
  if (m <= 0) return 0;
  double t[2 * NEKGPU_PROJ_MAX];
  count_launch();
  multidot_kernel<<<q.nb, kThreads, 0, q.s>>>(X0, B0, q.n, m, q.w, bm, xm, q.n, q.h.red.ptr);
  int rc = fetch_sums(q, 2 * m, t);
  for (int k = 0; k < m; ++k) out[k] = 0.5 * (t[k] + t[m + k]);
  return rc;
}

// b = mask * dssum(A x)  (proj_matvec, navier4.f:827-850)
int matvec(Ctx& q, double* b, const double* x) {
  cudaError_t e = q.h.exact
                      ? launch_axhelm<double, true>(q.h.mesh, q.h.mesh.f64, b, x, q.c, q.s)
                      : launch_axhelm<double, false>(q.h.mesh, q.h.mesh.f64, b, x, q.c, q.s);
  if (e != cudaSuccess) {
    set_error(q.h, std::string("projection matvec: ") + cudaGetErrorString(e));
    return -3;
  }
  gs_op<double>(q.h.mesh.gs, b, 0, q.s);
  count_launch();
  mask_kernel<<<q.nb, kThreads, 0, q.s>>>(b, q.msk, q.n);
  return 0;
}

void subtract(Ctx& q, double* y1, double* y2, const double* V1, const double* V2,
              const std::vector<int>& ks, const double* coef) {
  if (ks.empty()) return;
  Scalars c, o;
  for (size_t j = 0; j < ks.size(); ++j) {
    c.v[j] = coef[j];
    o.v[j] = (double)ks[j];
  }
  count_launch();
  subtract_kernel<<<q.nb, kThreads, 0, q.s>>>(y1, y2, V1, V2, q.n, (int)ks.size(), c, o, q.n);
}

void scale2(Ctx& q, double* a, double* b, double c) {
  count_launch();
  scale2_kernel<<<q.nb, kThreads, 0, q.s>>>(a, b, c, q.n);
}

constexpr double kIndepTol = 1.0e-7;  // linear-independence test, FP64 (wdsize = 8)

// proj_ortho_full_cgs2 (navier4.f:1060-1127)
int ortho_full_cgs2(Ctx& q) {
  int m = q.P.m;
  if (m <= 0) return 0;
  int flag[NEKGPU_PROJ_MAX] = {};
  for (int round = 0; round < 2; ++round) {
    for (int k = m; k >= 1; --k) {
      // alpha(j) for j = k..m: 0.5 ((x_j, b_k) + (b_j, x_k))
      double al[NEKGPU_PROJ_MAX];
      const int cnt = m - k + 1;
      int rc = sym_dots(q, q.X(k - 1), q.B(k - 1), cnt, q.B(k - 1), q.X(k - 1), al);
      if (rc) return rc;
      // x_k -= alpha(j) x_j, b_k -= alpha(j) b_j for j = m down to k+1
      std::vector<int> ks;
      std::vector<double> cf;
      for (int j = m; j >= k + 1; --j) {
        ks.push_back(j - 1);
        cf.push_back(al[j - k]);
      }
      subtract(q, q.X(k - 1), q.B(k - 1), q.P.xx.ptr, q.P.bb.ptr, ks, cf.data());
      const double normp = std::sqrt(al[0]);
      double nk = 0.0;
      rc = dots(q, q.X(k - 1), 1, q.B(k - 1), &nk);
      if (rc) return rc;
      const double normk = std::sqrt(nk);
      if (normk > kIndepTol * normp) {
        scale2(q, q.X(k - 1), q.B(k - 1), 1.0 / normk);
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
        cudaMemcpyAsync(q.X(k - 1), q.X(j - 1), q.n * sizeof(double), cudaMemcpyDeviceToDevice,
                        q.s);
        cudaMemcpyAsync(q.B(k - 1), q.B(j - 1), q.n * sizeof(double), cudaMemcpyDeviceToDevice,
                        q.s);
      }
    }
  }
  q.P.m = k;
  return 0;
}

// proj_ortho (navier4.f:852-957), after x_m, b_m were appended
int ortho(Ctx& q) {
  int m = q.P.m;
  if (m <= 0) return 0;
  double alpha[NEKGPU_PROJ_MAX], beta[NEKGPU_PROJ_MAX];
  double* xm = q.X(m - 1);
  double* bm = q.B(m - 1);
  int rc = sym_dots(q, q.P.xx.ptr, q.P.bb.ptr, m, bm, xm, alpha);
  if (rc) return rc;
  double nrm = std::sqrt(alpha[m - 1]);
  std::vector<int> ks;
  for (int k = 0; k < m - 1; ++k) ks.push_back(k);
  subtract(q, xm, bm, q.P.xx.ptr, q.P.bb.ptr, ks, alpha);
  if (m > 1) {
    rc = sym_dots(q, q.P.xx.ptr, q.P.bb.ptr, m - 1, bm, xm, beta);
    if (rc) return rc;
    subtract(q, xm, bm, q.P.xx.ptr, q.P.bb.ptr, ks, beta);
    for (int k = 0; k < m - 1; ++k) alpha[k] = alpha[k] + beta[k];
  }
  double am = 0.0;
  rc = dots(q, xm, 1, bm, &am);
  if (rc) return rc;
  alpha[m - 1] = std::sqrt(am);
  if (alpha[m - 1] > kIndepTol * nrm) {
    scale2(q, xm, bm, 1.0 / alpha[m - 1]);
    if (m > 1) {
      Scalars cs;
      for (int k = m, qq = 0; k >= 2; --k, ++qq) {
        const int hh = k - 1;
        double c, s;
        givens_rotation(alpha[hh - 1], alpha[k - 1], &c, &s, &nrm);
        alpha[hh - 1] = nrm;
        cs.v[2 * qq] = c;
        cs.v[2 * qq + 1] = s;
      }
      count_launch();
      givens_kernel<<<q.nb, kThreads, 0, q.s>>>(q.P.xx.ptr, q.P.bb.ptr, q.n, m, cs, q.n);
    }
  } else {
    q.P.m = m - 1;  // rank deficient: forget the new vector
  }
  return 0;
}

}  // namespace

int proj_space(Handle& h, int space, ProjSpace** out) {
  if (space < 0 || space >= NEKGPU_PROJ_SPACES) {
    set_error(h, "projection space index out of range");
    return -1;
  }
  if ((int)h.proj.size() <= space) h.proj.resize(space + 1);
  if (!h.proj[space]) {
    h.proj[space].reset(new ProjSpace());
    h.proj[space]->mmx = NEKGPU_PROJ_DEFAULT;
  }
  *out = h.proj[space].get();
  return 0;
}

// project1 (navier4.f:636-733): b <- b - B alpha, with xbar = X alpha kept
int proj_project1(Handle& h, ProjSpace& P, double* b, const Coef<double>& c, const double* h1,
                  const double* h2, const double* msk, const double* w) {
  const int64_t n = h.mesh.n;
  if (P.m <= 0) return 0;
  Ctx q{h, P, c, msk, w, n, h.stream, blocks(n)};
  if (h.red.ensure((size_t)q.nb * 2 * NEKGPU_PROJ_MAX)) {
    set_error(h, "projection: allocation failed");
    return -4;
  }
  // iproj_chk (:788-820): h1 / h2 changed since the space was built?
  count_launch();
  maxdiff_kernel<<<q.nb, kThreads, 0, q.s>>>(h1, P.h1old.ptr, h2, P.h2old.ptr, n, h.red.ptr);
  std::vector<double> hp(2 * (size_t)q.nb);
  cudaMemcpyAsync(hp.data(), h.red.ptr, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, q.s);
  if (cudaStreamSynchronize(q.s) != cudaSuccess) {
    set_error(h, std::string("projection: ") + cudaGetErrorString(cudaGetLastError()));
    return -3;
  }
  double dh = 0.0;
  for (double v : hp) dh = std::max(dh, v);
  int rc;
  if (dh > 0.0) {
    cudaMemcpyAsync(P.h1old.ptr, h1, n * sizeof(double), cudaMemcpyDeviceToDevice, q.s);
    cudaMemcpyAsync(P.h2old.ptr, h2, n * sizeof(double), cudaMemcpyDeviceToDevice, q.s);
    for (int j = 0; j < P.m; ++j)
      if ((rc = matvec(q, q.B(j), q.X(j)))) return rc;
    if ((rc = ortho_full_cgs2(q))) return rc;
  }
  const int m = P.m;
  if (m <= 0) return 0;
  // project1_a (:735-825): two rounds of classical Gram-Schmidt
  Scalars a;
  double al[NEKGPU_PROJ_MAX];
  for (int round = 0; round < 2; ++round) {
    if ((rc = dots(q, P.xx.ptr, m, b, al))) return rc;
    for (int k = 0; k < m; ++k) a.v[k] = al[k];
    count_launch();
    combine_kernel<<<q.nb, kThreads, 0, q.s>>>(P.xx.ptr, P.bb.ptr, n, m, a, round == 0 ? 1 : 0,
                                              P.xbar.ptr, P.bbar.ptr, b, n);
  }
  return 0;
}

// project2 (navier4.f:1129-1187): x += xbar; append (x, A x); proj_ortho
int proj_project2(Handle& h, ProjSpace& P, double* x, const Coef<double>& c, const double* msk,
                  const double* w) {
  const int64_t n = h.mesh.n;
  Ctx q{h, P, c, msk, w, n, h.stream, blocks(n)};
  if (h.red.ensure((size_t)q.nb * 2 * NEKGPU_PROJ_MAX)) {
    set_error(h, "projection: allocation failed");
    return -4;
  }
  if (P.m > 0) {
    count_launch();
    add_kernel<<<q.nb, kThreads, 0, q.s>>>(x, P.xbar.ptr, n);
  }
  P.m = std::min(P.m + 1, P.mmx);
  cudaMemcpyAsync(q.X(P.m - 1), x, n * sizeof(double), cudaMemcpyDeviceToDevice, q.s);
  int rc = matvec(q, q.B(P.m - 1), q.X(P.m - 1));
  if (rc) return rc;
  rc = ortho(q);
  if (rc) return rc;
  if (cudaStreamSynchronize(q.s) != cudaSuccess) {
    set_error(h, std::string("projection: ") + cudaGetErrorString(cudaGetLastError()));
    return -3;
  }
  return 0;
}

// Storage of a space for the current mesh (zeroed h1old / h2old, as the
// reference's approx array starts).
int proj_alloc(Handle& h, ProjSpace& P) {
  const int64_t n = h.mesh.n;
  if (P.xx.cap >= (size_t)n * P.mmx && P.bb.cap >= (size_t)n * P.mmx && P.h1old.cap >= (size_t)n)
    return 0;
  if (P.xx.ensure((size_t)n * P.mmx) || P.bb.ensure((size_t)n * P.mmx) || P.xbar.ensure(n) ||
      P.bbar.ensure(n) || P.h1old.ensure(n) || P.h2old.ensure(n)) {
    set_error(h, "projection: allocation failed");
    return -4;
  }
  P.m = 0;
  cudaMemsetAsync(P.h1old.ptr, 0, n * sizeof(double), h.stream);
  cudaMemsetAsync(P.h2old.ptr, 0, n * sizeof(double), h.stream);
  return 0;
}

}  // namespace nekgpu
