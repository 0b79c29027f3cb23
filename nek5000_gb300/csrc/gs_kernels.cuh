// gs_kernels.cuh -- the PCG form of the gather-scatter (kernel B of an
// iteration) as a block body, shared by the single-problem and batched
// solvers: w = mask * dssum(w) on every element-boundary group, boundary part
// of rho = sum w p mult (core/hmholtz.f:797-801; skipped when the operator
// reduced rho over every point), then alpha = rtz1 / rho.
#pragma once
#include "gs.cuh"

namespace nekgpu {

// Groups of C copies (C in 1, 2, 4, 8): each thread takes G groups of its
// class (block-strided, so index loads stay coalesced), loads every group's
// indices with one vector access, issues all gathers before any use, sums each
// group in ascending local-index order, scatters, and accumulates rho.
template <int C>
__device__ __forceinline__ void load_ids(const int* __restrict__ cidx, int s, int (&id)[C]) {
  if constexpr (C == 1) {
    id[0] = cidx[s];
  } else if constexpr (C == 2) {
    const int2 v = reinterpret_cast<const int2*>(cidx)[s];
    id[0] = v.x;
    id[1] = v.y;
  } else {
#pragma unroll
    for (int h = 0; h < C / 4; ++h) {
      const int4 v = reinterpret_cast<const int4*>(cidx)[(C / 4) * s + h];
      id[4 * h] = v.x;
      id[4 * h + 1] = v.y;
      id[4 * h + 2] = v.z;
      id[4 * h + 3] = v.w;
    }
  }
}

// FP32 w is touched with an evict-last L2 policy (it stays resident for the
// update kernel).  RHO = false skips the rho accumulation (the operator then
// reduced rho over every local point, see AxArgs::allrho).
template <typename T>
__device__ __forceinline__ T w_load(const T* w, int i, uint64_t pol) {
  if constexpr (sizeof(T) == 4) return ld_hint(w + i, pol);
  else return w[i];
}
template <typename T>
__device__ __forceinline__ void w_store(T* w, int i, T v, uint64_t pol) {
  if constexpr (sizeof(T) == 4) st_hint(w + i, v, pol);
  else w[i] = v;
}

// Sum of a[q] for q = q0, q0 + st, ... < q1 (one lane's share of a fold),
// with eight loads in flight: accumulator c takes terms c, c + 8, ... of the
// sequence, and the eight are added in order (a fixed order for fixed
// arguments).
__device__ __forceinline__ double strided_sum_cg(const double* __restrict__ a, int q0, int q1,
                                                 int st) {
  double acc[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  int q = q0;
  for (; q + 7 * st < q1; q += 8 * st) {
#pragma unroll
    for (int c = 0; c < 8; ++c) acc[c] += __ldcg(a + q + c * st);
  }
#pragma unroll
  for (int c = 0; c < 7; ++c)
    if (q + c * st < q1) acc[c] += __ldcg(a + q + c * st);
  double s = acc[0];
#pragma unroll
  for (int c = 1; c < 8; ++c) s += acc[c];
  return s;
}

template <typename T, int C, int G, bool RHO>
__device__ __forceinline__ void gs_groups(const int* __restrict__ cidx, int s0, int step, int cnt,
                                          int goff, T* __restrict__ w, const T* __restrict__ p,
                                          const T* __restrict__ segmask,
                                          const T* __restrict__ segmsum, CompAcc<T>& acc) {
  int id[G][C];
  bool on[G];
#pragma unroll
  for (int q = 0; q < G; ++q) {
    const int s = s0 + q * step;
    on[q] = s < cnt;
    if (on[q]) load_ids<C>(cidx, s, id[q]);
  }
  const uint64_t keep = sizeof(T) == 4 ? l2_policy_evict_last() : 0;
  T v[G][C], p0[G], mk[G], ms[G];
#pragma unroll
  for (int q = 0; q < G; ++q) {
    if (!on[q]) continue;
    const int s = s0 + q * step;
#pragma unroll
    for (int c = 0; c < C; ++c) v[q][c] = w_load(w, id[q][c], keep);
    if constexpr (RHO) {
      p0[q] = p[id[q][0]];
      ms[q] = segmsum[goff + s];
    }
    mk[q] = segmask[goff + s];
  }
#pragma unroll
  for (int q = 0; q < G; ++q) {
    if (!on[q]) continue;
    T t = v[q][0];
#pragma unroll
    for (int c = 1; c < C; ++c) t = t + v[q][c];
    t = t * mk[q];
#pragma unroll
    for (int c = 0; c < C; ++c) w_store(w, id[q][c], t, keep);
    if constexpr (RHO) acc.add(t * p0[q] * ms[q]);
  }
}

// Block body: block `blk` of `nblk`.  The blocks of each size class are
// contiguous (a block runs one class).  Warp 0 also folds a strided slice of
// the operator's interior partials into the block's partial; the last block
// sets rho and alpha = rtz1 / rho.
// Groups per thread of class k under a groups-per-thread shift (the host's
// gs_shape computes the same numbers for the block offsets).
__host__ __device__ constexpr int gs_groups_shifted(int k, int gshift) {
  return k >= kGsClasses - 1 ? 1
         : gshift >= 0       ? ((gs_groups_per_thread(k) << gshift) > 8 ? 8 : (gs_groups_per_thread(k) << gshift))
                             : ((gs_groups_per_thread(k) >> (-gshift)) < 1 ? 1 : (gs_groups_per_thread(k) >> (-gshift)));
}

template <typename T, int GSH = 0, bool RHO = true>
__device__ __forceinline__ void gs_cg_body(T* __restrict__ w, const T* __restrict__ p,
                                           const int* __restrict__ start,
                                           const int* __restrict__ idx, const GsClasses& cls,
                                           const T* __restrict__ segmask,
                                           const T* __restrict__ segmsum, CgScalars* cg,
                                           const double* __restrict__ partialA, int nA,
                                           double* __restrict__ partialB, int blk, int nblk,
                                           double* red, int* am_last_s) {
  constexpr bool rho = RHO;
  int& am_last = *am_last_s;
  int k = 0;
  while (k < kGsClasses - 1 && blk >= cls.boff[k + 1]) ++k;
  const int G = cls.g[k];  // = gs_groups_shifted(k, GSH)
  const int s0 = (blk - cls.boff[k]) * blockDim.x * G + threadIdx.x;
  const int* ci = idx + cls.ioff[k];
  const int goff = cls.soff[k], cnt = cls.cnt[k];
  CompAcc<T> acc;
#define NEKGPU_GS_CG(C, GG) \
  gs_groups<T, C, GG, RHO>(ci, s0, blockDim.x, cnt, goff, w, p, segmask, segmsum, acc);
  switch (k) {
    case 0: NEKGPU_GS_CG(1, gs_groups_shifted(0, GSH)) break;
    case 1: NEKGPU_GS_CG(2, gs_groups_shifted(1, GSH)) break;
    case 2: NEKGPU_GS_CG(4, gs_groups_shifted(2, GSH)) break;
    case 3: NEKGPU_GS_CG(8, gs_groups_shifted(3, GSH)) break;
#undef NEKGPU_GS_CG
    default:
      for (int q = 0; q < G; ++q) {
        const int sl = s0 + q * blockDim.x;
        if (sl >= cnt) break;
        const int g = goff + sl;
        const int a = start[g], b = start[g + 1];
        T t = w[idx[a]];
        for (int c = a + 1; c < b; ++c) t = t + w[idx[c]];
        t = t * segmask[g];
        for (int c = a; c < b; ++c) w[idx[c]] = t;
        if constexpr (RHO) acc.add(t * p[idx[a]] * segmsum[g]);
      }
  }
  if constexpr (!rho) {
    // The operator's per-element partials hold all of rho.  Warp 0 folds a
    // strided slice of them and the last block's warp 0 sums the block
    // partials in lane order; no block-wide barrier, so the other warps leave
    // as soon as their groups are done.
    // Warp 0 of block b folds the fixed chunks b, b + nblk, ... of
    // kFoldChunk partials (lane l takes every 32nd one), so that the sum does
    // not depend on the block count whenever nblk covers every chunk.
    if (threadIdx.x >= 32) return;
    constexpr int kFoldChunk = 1024;
    double pa = 0.0;
    for (int c0 = blk * kFoldChunk; c0 < nA; c0 += nblk * kFoldChunk)
      pa += strided_sum_cg(partialA, c0 + (int)threadIdx.x, min(c0 + kFoldChunk, nA), 32);
    pa = warp_sum(pa);
    unsigned int last = 0;
    if (threadIdx.x == 0) {
      partialB[blk] = pa;
      __threadfence();
      const unsigned int ticket = atomicAdd(&cg->counter[0], 1u);
      last = (ticket == (unsigned int)nblk - 1) ? 1u : 0u;
    }
    last = __shfl_sync(0xffffffffu, last, 0);
    if (!last) return;
    __threadfence();
    double pb = strided_sum_cg(partialB, threadIdx.x, nblk, 32);
    pb = warp_sum(pb);
    if (threadIdx.x == 0) {
      cg->rho = pb;
      cg->alpha = cg->rtz1 / pb;
      cg->counter[0] = 0u;
    }
    return;
  }
  double dot = block_sum_comp(acc, red);  // thread 0
  if (threadIdx.x < 32) {
    double pa = 0.0;
    for (int q = blk + nblk * threadIdx.x; q < nA; q += nblk * 32) pa += __ldcg(partialA + q);
    pa = warp_sum(pa);
    if (threadIdx.x == 0) {
      partialB[blk] = dot + pa;
      __threadfence();
      const unsigned int ticket = atomicAdd(&cg->counter[0], 1u);
      am_last = (ticket == (unsigned int)nblk - 1);
    }
  }
  __syncthreads();
  if (!am_last) return;
  double pb = 0.0;
#pragma unroll 8
  for (int q = threadIdx.x; q < nblk; q += blockDim.x) pb += __ldcg(partialB + q);
  const double rho_all = block_sum(pb, red);
  if (threadIdx.x == 0) {
    cg->rho = rho_all;
    cg->alpha = cg->rtz1 / rho_all;
    cg->counter[0] = 0u;
  }
}

template <typename T, int GSH, bool RHO>
__global__ void __launch_bounds__(kGsMaxThreads)
    gs_cg_kernel(T* __restrict__ w, const T* __restrict__ p, const int* __restrict__ start,
                 const int* __restrict__ idx, const GsClasses cls,
                 const T* __restrict__ segmask, const T* __restrict__ segmsum, CgScalars* cg,
                 const double* __restrict__ partialA, int nA, double* __restrict__ partialB) {
  __shared__ double red[32];
  __shared__ int am_last;
  if (cg->done) return;
  gs_cg_body<T, GSH, RHO>(w, p, start, idx, cls, segmask, segmsum, cg, partialA, nA, partialB,
                          blockIdx.x, gridDim.x, red, &am_last);
}

}  // namespace nekgpu
