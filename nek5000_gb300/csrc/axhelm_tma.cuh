// axhelm_tma.cuh -- the operator with TMA-staged element blocks.
//
// Same mathematics and contraction order as axhelm.cuh (core/hmholtz.f:72-259,
// 3-D deformed path), organised for HBM bandwidth:
//
//  * one block owns EPB consecutive elements (a compile-time shape the
//    autotuner picks from tma_epb_cand); since every array is
//    element-major, their u (or p, r, d), G, bm1 and coefficient slices are
//    each one contiguous range, staged into shared memory by a handful of
//    1-D bulk asynchronous copies (cp.async.bulk) completing on one mbarrier
//    -- every byte the block needs is in flight at once;
//  * thread (i,j) of an element keeps the rows D(i,:), D(j,:) and the columns
//    D(:,i), D(:,j) in registers; rows of the staged field are read as 8- or
//    16-byte vectors (warp broadcasts), columns as conflict-free scalars;
//  * the t-direction transposed contraction accumulates in registers.
//
// Valid when the arrays are 16-byte aligned.  For even lx1 a block's slices
// start and end on 16-byte boundaries (lx1^3 sizeof(T) is a multiple of 16).
// For odd lx1 (FP32, lx1 <= 9) each slice is copied as the window of whole
// 16-byte units that holds it -- up to 3 values before its first element and
// after its last, never outside the array -- and the slice pointer is offset
// into the window; a block whose window would reach past the end of an array
// (the last block) stages its slices with plain loads instead.  Otherwise
// axhelm.cuh's kernel is used.
#pragma once
#include "axhelm.cuh"
#include "tma.cuh"

namespace nekgpu {

// Built-in elements per block: about 128 threads, at least one element.
template <int NX>
__host__ __device__ constexpr int tma_epb() {
  return (128 / (NX * NX)) > 0 ? (128 / (NX * NX)) : 1;
}

// Shapes the autotuner may pick: half, once and twice the built-in count.
template <int NX>
__host__ __device__ constexpr int tma_epb_cand(int q) {
  return q == 0 ? (tma_epb<NX>() / 2 > 0 ? tma_epb<NX>() / 2 : 1)
                : (q == 1 ? tma_epb<NX>() : 2 * tma_epb<NX>());
}

// Values of a staged slice of `len` values in shared memory: len when len
// values are whole 16-byte units for every block (P sizeof(T) a multiple of
// 16), else room for the 16-byte window around them.
template <typename T>
__host__ __device__ constexpr int tma_window(int len, bool whole) {
  return whole ? len : ((len + 2 * (16 / (int)sizeof(T)) - 2) / (16 / (int)sizeof(T))) *
                           (16 / (int)sizeof(T));
}

// Number of staged field slices (of EPB*P values) besides G and the work slabs.
__host__ __device__ constexpr int tma_nslices(bool fused, int h1mode, int h2mode) {
  return 1 + (fused ? 2 : 0) + (h2mode ? 1 : 0) + (h1mode == 1 ? 1 : 0) + (h2mode == 2 ? 1 : 0);
}

// The fused form reuses the r and d slices (consumed by the p update) as the
// two work slabs; the plain form needs two more.
template <int NX, typename T, int EPB>
__host__ __device__ constexpr size_t tma_smem_bytes(bool fused, int h1mode, int h2mode) {
  constexpr int P = NX * NX * NX;
  constexpr bool whole = (P * sizeof(T)) % 16 == 0;
  return 64 /* mbarrier + pad */ + ((size_t)NX * NX * sizeof(T) + 15) / 16 * 16 /* D */ +
         sizeof(T) * ((size_t)tma_window<T>(EPB * P, whole) *
                          (tma_nslices(fused, h1mode, h2mode) + (fused ? 0 : 2)) +
                      tma_window<T>(6 * EPB * P, whole));
}

// Load NX consecutive values of T from shared memory with the widest aligned
// vector width that NX*sizeof(T) allows.
template <int NX, typename T>
__device__ __forceinline__ void load_row(const T* __restrict__ p, T (&v)[NX]) {
  if constexpr ((NX * sizeof(T)) % 16 == 0) {
    using V = typename Vec16<T>::type;
    constexpr int W = 16 / sizeof(T);
#pragma unroll
    for (int c = 0; c < NX / W; ++c) {
      const V x = reinterpret_cast<const V*>(p)[c];
      if constexpr (W == 4) {
        v[4 * c] = x.x;
        v[4 * c + 1] = x.y;
        v[4 * c + 2] = x.z;
        v[4 * c + 3] = x.w;
      } else {
        v[2 * c] = x.x;
        v[2 * c + 1] = x.y;
      }
    }
  } else if constexpr (sizeof(T) == 4 && (NX * sizeof(T)) % 8 == 0) {
#pragma unroll
    for (int c = 0; c < NX / 2; ++c) {
      const float2 x = reinterpret_cast<const float2*>(p)[c];
      v[2 * c] = x.x;
      v[2 * c + 1] = x.y;
    }
  } else {
#pragma unroll
    for (int l = 0; l < NX; ++l) v[l] = p[l];
  }
}

// Body of the kernel for element block `blk` (elements blk*EPB ...); the
// block's threads are (NX*NX, EPB); smem_raw is its dynamic shared memory.
template <int NX, typename T, bool FUSED, int EPB>
__device__ __forceinline__ void axhelm_tma_body(const AxArgs<T>& a, int blk,
                                                unsigned char* smem_raw) {
  constexpr int P = NX * NX * NX, NXY = NX * NX;
  constexpr int U = 16 / (int)sizeof(T);  // values per 16-byte unit
  constexpr bool whole = (P % U) == 0;     // every block's slices are whole units
  constexpr int SL = tma_window<T>(EPB * P, whole), SLG = tma_window<T>(6 * EPB * P, whole);
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
  T* sD = reinterpret_cast<T*>(smem_raw + 64);  // D[i][l] row-major
  // staged slices (windows of SL values, 16-byte aligned), G's of SLG
  T* base = reinterpret_cast<T*>(smem_raw + 64 + ((NX * NX * sizeof(T) + 15) / 16) * 16);
  const int hb = a.h2mode ? 1 : 0, hh1 = a.h1mode == 1 ? 1 : 0, hh2 = a.h2mode == 2 ? 1 : 0;
  const int e0 = blk * EPB;
  const int ne = min(EPB, a.nel - e0);  // elements of this block
  const size_t off = (size_t)e0 * P;
  // values of the window before the block's first element (0 when whole)
  const int du = whole ? 0 : (int)(off % U), dg = whole ? 0 : (int)((6 * off) % U);
  T* wU = base;
  T* wR = wU + SL;
  T* wDg = wR + (FUSED ? SL : 0);
  T* wB = wDg + (FUSED ? SL : 0);
  T* wH1 = wB + hb * SL;
  T* wH2 = wH1 + hh1 * SL;
  T* wG = wH2 + hh2 * SL;
  T* sU = wU + du;
  T* sR = wR + du;
  T* sDg = wDg + du;
  T* sB = wB + du;
  T* sH1 = wH1 + du;
  T* sH2 = wH2 + du;
  T* sG = wG + dg;
  T* st1 = FUSED ? sR : wG + SLG;
  T* st2 = FUSED ? sDg : wG + SLG + SL;

  if constexpr (FUSED) {
    if (a.cg->done) return;
  }
  const int tid = threadIdx.x + NXY * threadIdx.y;
  if (tid == 0) {
    mbar_init(bar, 1);
    mbar_fence_init();
  }
  for (int q = tid; q < NXY; q += NXY * EPB) sD[q] = a.D[q];
  __syncthreads();
  // window lengths (whole 16-byte units) and whether they stay inside the
  // arrays; if not (the last block of an odd order), plain loads of the same
  // slices (block-uniform)
  const int wl = whole ? ne * P : (du + ne * P + U - 1) / U * U;
  const int wlg = whole ? 6 * ne * P : (dg + 6 * ne * P + U - 1) / U * U;
  const size_t n = (size_t)a.nel * P;
  const bool bulk = whole || (off - du + wl <= n && 6 * off - dg + wlg <= 6 * n);
  if (!bulk) {
    const int nv = ne * P, nt = NXY * EPB;
    for (int q = tid; q < nv; q += nt) {
      sU[q] = a.u[off + q];
      if constexpr (FUSED) {
        sR[q] = a.r[off + q];
        sDg[q] = a.d[off + q];
      }
      if (hb) sB[q] = a.bm1[off + q];
      if (hh1) sH1[q] = a.h1[off + q];
      if (hh2) sH2[q] = a.h2[off + q];
    }
    for (int q = tid; q < 6 * nv; q += nt) sG[q] = a.G[6 * off + q];
  }
  if (tid == 0 && bulk) {
    const uint32_t fb = (uint32_t)(wl * sizeof(T)), fg = (uint32_t)(wlg * sizeof(T));
    const uint32_t total = fb * (1 + (FUSED ? 2 : 0) + hb + hh1 + hh2) + fg;
    mbar_expect_tx(bar, total);
    // every input is read once per apply: evict first, so that L2 keeps w
    // (operands shared by the fields of a multi-field solve: default policy)
    const uint64_t pol = l2_policy_evict_first();
    const uint64_t spol = a.shared_in ? l2_policy_evict_normal() : pol;
    const size_t wo = off - du;
    bulk_g2s_hint(wU, a.u + wo, fb, bar, pol);
    if constexpr (FUSED) {
      bulk_g2s_hint(wR, a.r + wo, fb, bar, pol);
      bulk_g2s_hint(wDg, a.d + wo, fb, bar, spol);
    }
    if (hb) bulk_g2s_hint(wB, a.bm1 + wo, fb, bar, spol);
    if (hh1) bulk_g2s_hint(wH1, a.h1 + wo, fb, bar, spol);
    if (hh2) bulk_g2s_hint(wH2, a.h2 + wo, fb, bar, spol);
    bulk_g2s_hint(wG, a.G + (6 * off - dg), fg, bar, spol);
  }
  // D rows / columns of this thread while the copies fly
  const int i = threadIdx.x % NX, j = threadIdx.x / NX, el = threadIdx.y;
  T Di[NX], Dj[NX], DTi[NX], DTj[NX];
#pragma unroll
  for (int l = 0; l < NX; ++l) {
    Di[l] = a.D[i * NX + l];
    Dj[l] = a.D[j * NX + l];
    DTi[l] = a.D[l * NX + i];
    DTj[l] = a.D[l * NX + j];
  }
  bool ok = true;
  if (bulk) ok = mbar_wait_bounded(bar, 0, a.err);
  else __syncthreads();
  const bool act = ok && el < ne;
  const int lo = el * P;  // element offset inside the staged slices
  const size_t eo = (size_t)(e0 + (el < ne ? el : 0)) * P;

  T beta = T(0);
  if constexpr (FUSED) beta = (T)a.cg->beta;
  T ru[NX];
  int qp[NX];  // positions of the column's points in the vectors (face order or natural)
#pragma unroll
  for (int k = 0; k < NX; ++k) {
    const int pt = k * NXY + j * NX + i;
    qp[k] = (FUSED && a.perm) ? __ldg(a.perm + pt) : pt;
  }
  if (FUSED && a.perm) {
    // face-ordered vectors: p at each position, then the slabs in natural order
#pragma unroll
    for (int k = 0; k < NX; ++k) {
      const int q = qp[k];
      T v = T(0);
      if (act) {
        v = fma(beta, sU[lo + q], sR[lo + q] * sDg[lo + q]);  // add2s1: p = beta*p + r*d
        a.p[eo + q] = v;
      }
      ru[k] = v;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NX; ++k)
      if (el < EPB) sU[lo + k * NXY + j * NX + i] = ru[k];
  } else {
#pragma unroll
    for (int k = 0; k < NX; ++k) {
      const int pt = k * NXY + j * NX + i;
      T v = act ? sU[lo + pt] : T(0);
      if constexpr (FUSED) {
        if (act) {
          v = fma(beta, v, sR[lo + pt] * sDg[lo + pt]);  // add2s1: p = beta*p + r*d
          sU[lo + pt] = v;
          a.p[eo + pt] = v;
        }
      }
      ru[k] = v;
    }
  }
  __syncthreads();

  T rau[NX];
#pragma unroll
  for (int m = 0; m < NX; ++m) rau[m] = T(0);
  const T* gE = sG + 6 * lo;
#pragma unroll
  for (int k = 0; k < NX; ++k) {
    const T* slab = sU + lo + k * NXY;
    T row[NX], dk[NX];
    load_row<NX, T>(slab + j * NX, row);
    load_row<NX, T>(sD + k * NX, dk);
    T ur = Di[0] * row[0];
#pragma unroll
    for (int l = 1; l < NX; ++l) ur = fma(Di[l], row[l], ur);
    T us = slab[i] * Dj[0];
#pragma unroll
    for (int l = 1; l < NX; ++l) us = fma(slab[l * NX + i], Dj[l], us);
    T ut = ru[0] * dk[0];
#pragma unroll
    for (int l = 1; l < NX; ++l) ut = fma(ru[l], dk[l], ut);
    const int pt = k * NXY + j * NX + i;
    const T g1 = gE[pt], g2 = gE[P + pt], g3 = gE[2 * P + pt], g4 = gE[3 * P + pt],
            g5 = gE[4 * P + pt], g6 = gE[5 * P + pt];
    const T h = hh1 ? sH1[lo + pt] : a.h1s;
    T t1 = ur * g1, t2 = us * g2, t3 = ut * g3;
    t1 = fma(us, g4, t1);
    t1 = fma(ut, g5, t1);
    t2 = fma(ur, g4, t2);
    t2 = fma(ut, g6, t2);
    t3 = fma(ur, g5, t3);
    t3 = fma(us, g6, t3);
    st1[lo + pt] = t1 * h;
    st2[lo + pt] = t2 * h;
    t3 *= h;
#pragma unroll
    for (int m = 0; m < NX; ++m) rau[m] = (k == 0) ? t3 * dk[m] : fma(t3, dk[m], rau[m]);
  }
  __syncthreads();

  T dot = T(0);
  const uint64_t keep = l2_policy_evict_last();
#pragma unroll
  for (int k = 0; k < NX; ++k) {
    const T* s1 = st1 + lo + k * NXY;
    const T* s2 = st2 + lo + k * NXY;
    T row[NX];
    load_row<NX, T>(s1 + j * NX, row);
    T tm1 = DTi[0] * row[0];
#pragma unroll
    for (int l = 1; l < NX; ++l) tm1 = fma(DTi[l], row[l], tm1);
    T tm2 = s2[i] * DTj[0];
#pragma unroll
    for (int l = 1; l < NX; ++l) tm2 = fma(s2[l * NX + i], DTj[l], tm2);
    T s = (tm1 + tm2) + rau[k];
    const int pt = k * NXY + j * NX + i;
    if (act) {
      if (hb) {
        const T hv = hh2 ? sH2[lo + pt] : a.h2s;
        s = fma(hv * sB[lo + pt], ru[k], s);
      }
      if constexpr (FUSED && sizeof(T) == 4) st_hint(a.au + eo + qp[k], s, keep);
      else a.au[eo + pt] = s;
      if constexpr (FUSED) {
        if (a.allrho || (i > 0 && i < NX - 1 && j > 0 && j < NX - 1 && k > 0 && k < NX - 1 &&
                         (!a.skip || !a.skip[eo + pt])))
          dot = fma(s, ru[k], dot);
      }
    }
  }
  if constexpr (FUSED) {
    // one partial per element, summed as axhelm.cuh's kernel does; the
    // element's staged G (read only before the second barrier) holds the
    // sum's NX^2 values and NX doubles: 6 NX^3 sizeof(T) is enough
    element_sum<NX, T>(dot, sG + 6 * lo, threadIdx.x, true, el < ne ? a.partial + e0 + el : nullptr);
  }
  if (tid == 0 && ok) mbar_inval(bar);
}

template <int NX, typename T, bool FUSED, int EPB>
__global__ void __launch_bounds__(NX* NX* EPB) axhelm_tma_kernel(const AxArgs<T> a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  axhelm_tma_body<NX, T, FUSED, EPB>(a, blockIdx.x, smem_raw);
}

// lx1 = 10 with one element per block: at least 5 resident blocks (96
// registers, 20 warps per SM) instead of the 4 that the 128 registers of the
// kernel above allow.  (A minimum-blocks bound on every shape is not
// neutral: with a minimum of 1 ptxas gives the lx1 = 8 kernel 191 registers
// instead of 96.)
template <typename T, bool FUSED>
__global__ void __launch_bounds__(100, 5) axhelm_tma_kernel_10x1(const AxArgs<T> a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  axhelm_tma_body<10, T, FUSED, 1>(a, blockIdx.x, smem_raw);
}

}  // namespace nekgpu
