// cg_kernels.cuh -- the PCG update kernel (kernel C of an iteration) as a
// block body, shared by the single-problem and batched solvers.
//
//   x += alpha p ; r -= alpha w ; z = r d            (hmholtz.f:804-805, :730)
//   s1 = sum z r mult ; s2 = sum mult binv r r       (vlsc3 :754, vlsc32 :758)
//   (fused multiply-add form: s1 = sum (r r) md, s2 = sum (r r) mb with the
//   per-solve weights md = mult d, mb = mult binv)
//   last block: rtz1, rbn2 = sqrt(s2/vol), convergence (:778), beta (:794)
#pragma once
#include "common.cuh"

namespace nekgpu {

// FOLD (fused multiply-add form only): d and b arrive as the folded weights
// md = mult d and mb = mult binv, and z r mult = (r r) md, mult binv r r =
// (r r) mb -- the same sums with one array and three operations fewer per
// point (z is not stored: the operator recomputes it).
template <typename T, bool EXACT, bool FIRST, bool FOLD = false>
struct UpdatePoint {
  // x += alpha p ; r -= alpha w ; z = r d ; s1 += z r mult ; s2 += mult binv r r
  __device__ __forceinline__ static void run(T& x, T& r, T p, T w, T d, T m, T b, T alpha,
                                             CompAcc<T>& a1, CompAcc<T>& a2) {
    if (!FIRST) {
      x = madd<EXACT>(alpha, p, x);   // add2s2(x,p,alpha)   (hmholtz.f:804)
      r = madd<EXACT>(-alpha, w, r);  // add2s2(r,w,-alpha)  (hmholtz.f:805)
    }
    if (FOLD) {
      const T rr = r * r;
      a1.add(rr * d);  // d = mult * d
      a2.add(rr * b);  // b = mult * binv
    } else if (EXACT) {
      const T z = mul_x(r, d);                         // col3 (:730)
      a1.add(mul_x(mul_x(z, r), m));                   // vlsc3 (:754)
      a2.add(mul_x(mul_x(mul_x(m, b), r), r));         // vlsc32 (:758, :848)
    } else {
      const T z = r * d;
      a1.add(z * r * m);
      a2.add(m * b * r * r);
    }
  }
};

__device__ __forceinline__ void cg_finalize(CgScalars* cg, double s1, double s2);

// Block body of the update kernel: block `blk` of `nblk` (1-D blocks).
// VEC: 16-byte vector accesses (all seven arrays 16-byte aligned).
template <typename T, bool EXACT, bool FIRST, bool VEC, bool FOLD = false>
__device__ __forceinline__ void cg_update_body(T* __restrict__ x, T* __restrict__ r,
                                               const T* __restrict__ p, const T* __restrict__ w,
                                               const T* __restrict__ d,
                                               const T* __restrict__ mult,
                                               const T* __restrict__ binv, int64_t n,
                                               CgScalars* cg, double* __restrict__ partial,
                                               int blk, int nblk, double* red, int* am_last_s) {
  int& am_last = *am_last_s;
  const T alpha = FIRST ? T(0) : (T)cg->alpha;
  CompAcc<T> a1, a2;
  using P = UpdatePoint<T, EXACT, FIRST, FOLD>;
  const int64_t gtid = blk * (int64_t)blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)nblk * blockDim.x;
  constexpr int W = 16 / sizeof(T);
  const int64_t nv = VEC ? n / W : 0;
  const uint64_t wpol = sizeof(T) == 4 ? l2_policy_evict_first() : 0;
  int64_t iv = gtid;
  for (; iv < nv; iv += stride) {
    T xx[W], rr[W], pp[W], ww[W], dd[W], mm[W], bb[W];
    ld16(rr, r, iv);
    ld16(dd, d, iv);
    if (!FOLD) ld16(mm, mult, iv);
    ld16(bb, binv, iv);
    if (!FIRST) {
      ld16(xx, x, iv);
      ld16(pp, p, iv);
      if constexpr (sizeof(T) == 4)  // last use of the L2-resident w
        *reinterpret_cast<float4*>(ww) = ld_hint4(reinterpret_cast<const float*>(w) + 4 * iv, wpol);
      else
        ld16(ww, w, iv);
    }
#pragma unroll
    for (int q = 0; q < W; ++q) P::run(xx[q], rr[q], pp[q], ww[q], dd[q], mm[q], bb[q], alpha, a1, a2);
    if (!FIRST) {
      st16(x, xx, iv);
      st16(r, rr, iv);
    }
  }
  for (int64_t i = nv * W + gtid; i < n; i += stride) {
    T xi = FIRST ? T(0) : x[i], ri = r[i];
    P::run(xi, ri, FIRST ? T(0) : p[i], FIRST ? T(0) : w[i], d[i], FOLD ? T(0) : mult[i],
           binv[i], alpha, a1, a2);
    if (!FIRST) {
      x[i] = xi;
      r[i] = ri;
    }
  }
  const double b1 = block_sum_comp(a1, red);
  const double b2 = block_sum_comp(a2, red);
  if (threadIdx.x == 0) {
    partial[blk] = b1;
    partial[nblk + blk] = b2;
    __threadfence();
    const unsigned int ticket = atomicAdd(&cg->counter[1], 1u);
    am_last = (ticket == (unsigned int)nblk - 1);
  }
  __syncthreads();
  if (!am_last) return;
  double t1 = 0.0, t2 = 0.0;
#pragma unroll 4
  for (int q = threadIdx.x; q < nblk; q += blockDim.x) {
    t1 += __ldcg(partial + q);
    t2 += __ldcg(partial + nblk + q);
  }
  const double s1 = block_sum(t1, red);
  const double s2 = block_sum(t2, red);
  if (threadIdx.x == 0) cg_finalize(cg, s1, s2);
}

// The last block's step of the update kernel: counts the iteration, stores
// rtz1 = s1 and rbn2 = sqrt(s2/vol), tests convergence (hmholtz.f:778) and
// forms beta (:794).
__device__ __forceinline__ void cg_finalize(CgScalars* cg, double s1, double s2) {
  {
    cg->counter[1] = 0u;
    const int iter = cg->iter + 1;
    cg->iter = iter;
    if (iter > cg->maxiter) {
      // the reference's loop has ended (do iter=1,niter): no further check,
      // rbn2 stays the norm of the last checked iterate
      cg->niter = cg->maxiter;
      cg->done = 1;
      return;
    }
    cg->s1 = s1;
    cg->s2 = s2;
    cg->rtz2 = cg->rtz1;
    cg->rtz1 = s1;
    const double rbn2 = sqrt(s2 / cg->vol);
    cg->rbn2 = rbn2;
    if (iter == 1) cg->rbn0 = rbn2;
    if (cg->tin < 0) cg->tol = fabs(cg->tin) * cg->rbn0;
    if (!isfinite(rbn2) || !isfinite(s1)) {
      cg->nonfinite = 1;
      cg->niter = iter - 1;
      cg->done = 1;
    } else if (rbn2 <= cg->tol && (iter > 1 || cg->istep <= 5)) {
      cg->niter = iter - 1;
      cg->done = 1;
    }
    cg->beta = (iter == 1) ? 0.0 : s1 / cg->rtz2;
  }
}

template <typename T, bool EXACT, bool FIRST, bool VEC, bool FOLD>
__global__ void __launch_bounds__(256)
    cg_update_kernel(T* __restrict__ x, T* __restrict__ r, const T* __restrict__ p,
                     const T* __restrict__ w, const T* __restrict__ d,
                     const T* __restrict__ mult, const T* __restrict__ binv, int64_t n,
                     CgScalars* cg, double* __restrict__ partial) {
  __shared__ double red[32];
  __shared__ int am_last;
  if (cg->done) return;
  cg_update_body<T, EXACT, FIRST, VEC, FOLD>(x, r, p, w, d, mult, binv, n, cg, partial,
                                             blockIdx.x, gridDim.x, red, &am_last);
}

// The update kernel with cggo's null-space correction (no Dirichlet point
// and h2 = 0, hmholtz.f:705-720, :747-750): z = r d, then z += rmean with
// rmean = smean * sum z bm1 (smean = -1 / sum bm1), and s1 = sum z r mult
// over the corrected z, formed as sum (r d) r mult + rmean sum r mult.  The
// kernel publishes rmean (cg->zmean) for the next operator launch, which
// forms p = (r d + rmean) + beta p.
template <typename T, bool EXACT, bool FIRST>
__global__ void __launch_bounds__(256)
    cg_update_mcor_kernel(T* __restrict__ x, T* __restrict__ r, const T* __restrict__ p,
                          const T* __restrict__ w, const T* __restrict__ d,
                          const T* __restrict__ mult, const T* __restrict__ binv,
                          const T* __restrict__ bm1, int64_t n, CgScalars* cg,
                          double* __restrict__ partial) {
  __shared__ double red[32];
  __shared__ int am_last;
  if (cg->done) return;
  const T alpha = FIRST ? T(0) : (T)cg->alpha;
  double a1 = 0.0, a2 = 0.0, a3 = 0.0, a4 = 0.0;
  const int nblk = gridDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)nblk * blockDim.x) {
    T ri = r[i];
    if (!FIRST) {
      x[i] = madd<EXACT>(alpha, p[i], x[i]);
      ri = madd<EXACT>(-alpha, w[i], ri);
      r[i] = ri;
    }
    const T m = mult[i];
    const T z = EXACT ? mul_x(ri, d[i]) : ri * d[i];
    a1 += (double)(EXACT ? mul_x(mul_x(z, ri), m) : z * ri * m);
    a2 += (double)(EXACT ? mul_x(mul_x(mul_x(m, binv[i]), ri), ri) : m * binv[i] * ri * ri);
    a3 += (double)(EXACT ? mul_x(z, bm1[i]) : z * bm1[i]);
    a4 += (double)(EXACT ? mul_x(ri, m) : ri * m);
  }
  const double b1 = block_sum(a1, red), b2 = block_sum(a2, red);
  const double b3 = block_sum(a3, red), b4 = block_sum(a4, red);
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = b1;
    partial[nblk + blockIdx.x] = b2;
    partial[2 * nblk + blockIdx.x] = b3;
    partial[3 * nblk + blockIdx.x] = b4;
    __threadfence();
    const unsigned int ticket = atomicAdd(&cg->counter[1], 1u);
    am_last = (ticket == (unsigned int)nblk - 1);
  }
  __syncthreads();
  if (!am_last) return;
  double t[4] = {0.0, 0.0, 0.0, 0.0};
  for (int q = threadIdx.x; q < nblk; q += blockDim.x)
    for (int k = 0; k < 4; ++k) t[k] += __ldcg(partial + k * nblk + q);
  double s[4];
  for (int k = 0; k < 4; ++k) s[k] = block_sum(t[k], red);
  if (threadIdx.x == 0) {
    const double zmean = cg->smean * s[2];
    cg->zmean = zmean;
    cg_finalize(cg, s[0] + zmean * s[3], s[1]);
  }
}

}  // namespace nekgpu
