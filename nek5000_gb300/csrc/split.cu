// split.cu -- the FP32 inner PCG of the mixed solve in the assembled-boundary
// layout.
//
// The reference keeps every vector element-local: a point on a face, edge or
// corner exists once per element that holds it, and dssum (core/dssum.f:79)
// makes the copies agree after each operator apply.  Inside the FP32 inner
// solve nothing outside sees the vectors, so they are stored the way the
// PCG needs them instead:
//
//   interior points   vI[e * NIp + q]   the (NX-2)^3 points of element e that
//                                       no other element holds, x fastest
//                                       (NIp: rounded up to 4 values)
//   boundary points   vB[g]             once per gather-scatter group g (one
//                                       global node on element boundaries),
//                                       in the order of the PCG-form maps
//
// r, p, x, the Jacobi diagonal d and the norm weight binv live in this
// layout; their copies are equal in the reference's arithmetic (d, binv and
// the masks are assembled; r, p, x stay continuous), so nothing is lost, and
// the multiplicity weights of the dot products (vlsc3 with vmult,
// core/hmholtz.f:754-758) become 1: each global node is summed once.
//
// One iteration is two kernels:
//   K1  the operator.  Element blocks stage G, bm1, h1, h2 and the interior
//       slices of r, d, p_old with 1-D bulk copies (TMA) and gather the
//       element's boundary values of r, d, p_old through gmap; p = r d +
//       beta p_old is formed in shared memory, w = A p element-locally
//       (core/hmholtz.f:191-217) and written out, interior part to wI and the
//       boundary copies to wBc[e * NBp + b]; rho = sum over local points of
//       p w (equal to p^T A p), reduced in fixed order, and alpha = rtz1 / rho
//       by the last block.
//   K2  the update.  Interior points stream; for each boundary group the
//       copies of w are summed from wBc (the direct-stiffness sum,
//       core/dssum.f:33-98) and masked; then p = r d + beta p_old (the same
//       rounding as K1), x += alpha p, r -= alpha w and the sums of r^2 d and
//       r^2 binv; the last block forms rtz, the norm, the convergence test and
//       beta (cg_finalize).
//
// Against the element-local form this drops the separate boundary-group
// pass, whose scattered loads and stores of single values were bound by L2
// latency, and reads r, p, x, d and binv once per global node: 71 against 80
// bytes per point and iteration.  Measured on GB300 at E=32^3, N=7 it is
// nevertheless slower (0.356 against 0.283 ms per iteration): the gathers
// through gmap in K1 and through cpos in K2 are scattered single values
// again, now in kernels with fewer warps in flight (K1: 18 warps per SM,
// bound by its shared memory), so their latency is exposed.  It stays an
// option (NEKGPU_OPT_SPLIT), off by default.
#include <algorithm>
#include <cmath>
#include <vector>

#include "axhelm_tma.cuh"
#include "cg_kernels.cuh"
#include "impl.cuh"

namespace nekgpu {

struct SplitLayout {
  int nx = 0, nel = 0, NI = 0, NB = 0, NIp = 0, NBp = 0;
  int nb = 0;      // boundary groups (global boundary nodes)
  int nbp = 0;     // nb rounded up to 4
  int epb = 1;     // elements per operator block
  int nblk1 = 0;   // operator blocks
  int nchunk = 0;  // reduction chunks of the operator's block partials
  int nblk2 = 0, nblkI = 0;  // update blocks: total, interior part
  GsClasses cls{};  // group classes of the PCG-form maps (counts and offsets)
  DevBuf<int> gmap, cpos, bfirst;
  DevBuf<unsigned short> bpt;
  DevBuf<float> rI, pI, xI, wI, dI, bI;
  DevBuf<float> rB, pB, xB, dB, bB, mB;
  DevBuf<float> wBc;
  DevBuf<double> part1, cpart1, part2;
  DevBuf<unsigned int> ccount;
  bool ready = false;
};

void SplitLayoutDeleter::operator()(SplitLayout* p) const { delete p; }

namespace {

constexpr int kUpdThreads = 256;
constexpr int kChunk = 256;  // operator block partials per reduction chunk

// Interior points of an element that come before natural point (i, j, k) in
// the x-fastest order; for an interior point this is its interior index, for
// a boundary point pt - this is its boundary index.
__host__ __device__ __forceinline__ int interior_before(int nx, int i, int j, int k) {
  const int m = nx - 2;
  auto clamp = [](int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); };
  int c = clamp(k - 1, 0, m) * m * m;
  if (k >= 1 && k <= m) {
    c += clamp(j - 1, 0, m) * m;
    if (j >= 1 && j <= m) c += clamp(i - 1, 0, m);
  }
  return c;
}

__host__ __device__ __forceinline__ bool is_interior(int nx, int i, int j, int k) {
  return i > 0 && i < nx - 1 && j > 0 && j < nx - 1 && k > 0 && k < nx - 1;
}

struct SplitArgs {
  const float* G;
  const float* bm1;
  const float* h1;
  const float* h2;
  float h1s, h2s;
  int h1mode, h2mode;
  const float* D;
  int nel;
  const int* gmap;
  const unsigned short* bpt;
  float *rI, *pI, *xI, *wI;
  const float *dI, *bI;
  float *rB, *pB, *xB;
  const float *dB, *bB, *mB;
  float* wBc;
  const int* bstart;  // PCG-form map starts (the "other" class)
  const int* cpos;    // wBc position of every copy, parallel to the map's idx
  GsClasses cls;
  int nb, nI4, nblkI;
  CgScalars* cg;
  double* part1;
  double* cpart1;
  unsigned int* ccount;
  int nchunk;
  double* part2;
  int* err;
};

__device__ __forceinline__ float form_p(float beta, float pold, float r, float d) {
  return __fmaf_rn(beta, pold, __fmul_rn(r, d));  // add2s1 (hmholtz.f:802)
}

template <int NX>
__host__ __device__ constexpr int split_ni() {
  return (NX - 2) * (NX - 2) * (NX - 2);
}
template <int NX>
__host__ __device__ constexpr int split_nip() {
  return (split_ni<NX>() + 3) / 4 * 4;
}
template <int NX>
__host__ __device__ constexpr int split_nb() {
  return NX * NX * NX - split_ni<NX>();
}
template <int NX>
__host__ __device__ constexpr int split_nbp() {
  return (split_nb<NX>() + 3) / 4 * 4;
}

template <int NX, int EPB>
__host__ __device__ constexpr size_t split_smem_bytes(int hb, int hh1, int hh2) {
  constexpr int P = NX * NX * NX;
  return 64 + (size_t)((NX * NX * 4 + 15) / 16) * 16 +
         (size_t)EPB * 4 * ((6 + hb + hh1 + hh2 + 3) * P + 3 * split_nip<NX>());
}

// K1: see the file comment.  Threads (NX*NX, EPB); thread (i, j) of element
// slot el walks the z-column of its element.
template <int NX, int EPB>
__global__ void __launch_bounds__(NX* NX* EPB) split_ax_kernel(const SplitArgs a) {
  constexpr int P = NX * NX * NX, NXY = NX * NX, NI = split_ni<NX>(), NB = split_nb<NX>();
  constexpr int NIp = split_nip<NX>(), NBp = split_nbp<NX>(), M = NX - 2;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ double red[32];
  __shared__ int am_last;
  if (a.cg->done) return;
  const int hb = a.h2mode ? 1 : 0, hh1 = a.h1mode == 1 ? 1 : 0, hh2 = a.h2mode == 2 ? 1 : 0;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem_raw);
  float* sD = reinterpret_cast<float*>(smem_raw + 64);
  float* sG = reinterpret_cast<float*>(smem_raw + 64 + ((NX * NX * 4 + 15) / 16) * 16);
  float* sB = sG + 6 * EPB * P;
  float* sH1 = sB + hb * EPB * P;
  float* sH2 = sH1 + hh1 * EPB * P;
  float* sU = sH2 + hh2 * EPB * P;
  float* st1 = sU + EPB * P;
  float* st2 = st1 + EPB * P;
  float* sRI = st2 + EPB * P;
  float* sDI = sRI + EPB * NIp;
  float* sPI = sDI + EPB * NIp;

  const int nthr = NXY * EPB;
  const int tid = threadIdx.x + NXY * threadIdx.y;
  const int e0 = blockIdx.x * EPB;
  const int ne = min(EPB, a.nel - e0);
  if (tid == 0) {
    mbar_init(bar, 1);
    mbar_fence_init();
  }
  for (int q = tid; q < NXY; q += nthr) sD[q] = a.D[q];
  __syncthreads();
  if (tid == 0) {
    const uint32_t fb = (uint32_t)(ne * P * 4), ib = (uint32_t)(ne * NIp * 4);
    const uint32_t total = fb * (6 + hb + hh1 + hh2) + 3 * ib;
    mbar_expect_tx(bar, total);
    const uint64_t pol = l2_policy_evict_first();
    const size_t off = (size_t)e0 * P, ioff = (size_t)e0 * NIp;
    bulk_g2s_hint(sG, a.G + 6 * off, 6 * fb, bar, pol);
    if (hb) bulk_g2s_hint(sB, a.bm1 + off, fb, bar, pol);
    if (hh1) bulk_g2s_hint(sH1, a.h1 + off, fb, bar, pol);
    if (hh2) bulk_g2s_hint(sH2, a.h2 + off, fb, bar, pol);
    bulk_g2s_hint(sRI, a.rI + ioff, ib, bar, pol);
    bulk_g2s_hint(sDI, a.dI + ioff, ib, bar, pol);
    bulk_g2s_hint(sPI, a.pI + ioff, ib, bar, pol);
  }
  const float beta = (float)a.cg->beta;
  // boundary values of the block's elements, gathered while the copies fly:
  // every index load first, then every value load, so that all of them are
  // in flight together
  {
    constexpr int NG = (NB * EPB + NXY * EPB - 1) / (NXY * EPB);
    int gq[NG], pq[NG];
#pragma unroll
    for (int u = 0; u < NG; ++u) {
      const int q = tid + u * nthr;
      gq[u] = -1;
      if (q < ne * NB) {
        const int el = q / NB, b = q - el * NB;
        gq[u] = __ldg(a.gmap + (size_t)(e0 + el) * NBp + b);
        pq[u] = el * P + __ldg(a.bpt + b);
      }
    }
    float pv[NG], rv[NG], dv[NG];
#pragma unroll
    for (int u = 0; u < NG; ++u) {
      if (gq[u] >= 0) {
        pv[u] = a.pB[gq[u]];
        rv[u] = a.rB[gq[u]];
        dv[u] = __ldg(a.dB + gq[u]);
      }
    }
#pragma unroll
    for (int u = 0; u < NG; ++u)
      if (gq[u] >= 0) sU[pq[u]] = form_p(beta, pv[u], rv[u], dv[u]);
  }
  const int i = threadIdx.x % NX, j = threadIdx.x / NX, el = threadIdx.y;
  float Di[NX], Dj[NX], DTi[NX], DTj[NX];
#pragma unroll
  for (int l = 0; l < NX; ++l) {
    Di[l] = a.D[i * NX + l];
    Dj[l] = a.D[j * NX + l];
    DTi[l] = a.D[l * NX + i];
    DTj[l] = a.D[l * NX + j];
  }
  const bool ok = mbar_wait_bounded(bar, 0, a.err);
  if (ok) {
    for (int q = tid; q < ne * NI; q += nthr) {
      const int e = q / NI, c = q - e * NI;
      const int ii = 1 + c % M, jj = 1 + (c / M) % M, kk = 1 + c / (M * M);
      sU[e * P + kk * NXY + jj * NX + ii] =
          form_p(beta, sPI[e * NIp + c], sRI[e * NIp + c], sDI[e * NIp + c]);
    }
  }
  __syncthreads();
  const bool act = ok && el < ne;
  const int lo = el * P;
  const int e = e0 + (el < ne ? el : 0);

  float ru[NX];
#pragma unroll
  for (int k = 0; k < NX; ++k) ru[k] = act ? sU[lo + k * NXY + j * NX + i] : 0.f;
  float rau[NX];
#pragma unroll
  for (int m = 0; m < NX; ++m) rau[m] = 0.f;
  const float* gE = sG + 6 * lo;
#pragma unroll
  for (int k = 0; k < NX; ++k) {
    const float* slab = sU + lo + k * NXY;
    float row[NX], dk[NX];
    load_row<NX, float>(slab + j * NX, row);
    load_row<NX, float>(sD + k * NX, dk);
    float ur = Di[0] * row[0];
#pragma unroll
    for (int l = 1; l < NX; ++l) ur = fmaf(Di[l], row[l], ur);
    float us = slab[i] * Dj[0];
#pragma unroll
    for (int l = 1; l < NX; ++l) us = fmaf(slab[l * NX + i], Dj[l], us);
    float ut = ru[0] * dk[0];
#pragma unroll
    for (int l = 1; l < NX; ++l) ut = fmaf(ru[l], dk[l], ut);
    const int pt = k * NXY + j * NX + i;
    const float g1 = gE[pt], g2 = gE[P + pt], g3 = gE[2 * P + pt], g4 = gE[3 * P + pt],
                g5 = gE[4 * P + pt], g6 = gE[5 * P + pt];
    const float h = hh1 ? sH1[lo + pt] : a.h1s;
    float t1 = ur * g1, t2 = us * g2, t3 = ut * g3;
    t1 = fmaf(us, g4, t1);
    t1 = fmaf(ut, g5, t1);
    t2 = fmaf(ur, g4, t2);
    t2 = fmaf(ut, g6, t2);
    t3 = fmaf(ur, g5, t3);
    t3 = fmaf(us, g6, t3);
    st1[lo + pt] = t1 * h;
    st2[lo + pt] = t2 * h;
    t3 *= h;
#pragma unroll
    for (int m = 0; m < NX; ++m) rau[m] = (k == 0) ? t3 * dk[m] : fmaf(t3, dk[m], rau[m]);
  }
  __syncthreads();

  float dot = 0.f;
  const uint64_t keep = l2_policy_evict_last();
#pragma unroll
  for (int k = 0; k < NX; ++k) {
    const float* s1 = st1 + lo + k * NXY;
    const float* s2 = st2 + lo + k * NXY;
    float row[NX];
    load_row<NX, float>(s1 + j * NX, row);
    float tm1 = DTi[0] * row[0];
#pragma unroll
    for (int l = 1; l < NX; ++l) tm1 = fmaf(DTi[l], row[l], tm1);
    float tm2 = s2[i] * DTj[0];
#pragma unroll
    for (int l = 1; l < NX; ++l) tm2 = fmaf(s2[l * NX + i], DTj[l], tm2);
    float s = (tm1 + tm2) + rau[k];
    const int pt = k * NXY + j * NX + i;
    if (act) {
      if (hb) {
        const float hv = hh2 ? sH2[lo + pt] : a.h2s;
        s = fmaf(hv * sB[lo + pt], ru[k], s);
      }
      const int rank = interior_before(NX, i, j, k);
      if (is_interior(NX, i, j, k)) st_hint(a.wI + (size_t)e * NIp + rank, s, keep);
      else st_hint(a.wBc + (size_t)e * NBp + (pt - rank), s, keep);
      dot = fmaf(s, ru[k], dot);
    }
  }
  // rho: element sums in a fixed order (sG is free again), then the block's
  // partial, then two-level fixed-order reduction over the blocks
  element_sum<NX, float>(dot, sG + 6 * lo, threadIdx.x, true, nullptr);
  // element_sum leaves the element's row sums in sG + 6 lo + rows offset
  if (tid == 0) {
    double bsum = 0.0;
    for (int q = 0; q < ne; ++q) {
      const double* rows = reinterpret_cast<const double*>(
          reinterpret_cast<const unsigned char*>(sG + 6 * q * P) + element_sum_rows_offset<NX, float>());
      double s = rows[0];
#pragma unroll
      for (int r = 1; r < NX; ++r) s += rows[r];
      bsum += s;
    }
    a.part1[blockIdx.x] = bsum;
    __threadfence();
    const int chunk = blockIdx.x / kChunk;
    const int nin = min(kChunk, (int)gridDim.x - chunk * kChunk);
    const unsigned int t = atomicAdd(&a.ccount[chunk], 1u);
    am_last = (t == (unsigned int)nin - 1) ? 1 : 0;
  }
  __syncthreads();
  if (am_last) {  // last block of its chunk: the chunk's partial
    __threadfence();
    const int chunk = blockIdx.x / kChunk;
    const int b0 = chunk * kChunk, nin = min(kChunk, (int)gridDim.x - b0);
    double v = 0.0;
    for (int q = tid; q < nin; q += nthr) v += __ldcg(a.part1 + b0 + q);
    v = block_sum(v, red);
    if (tid == 0) {
      a.cpart1[chunk] = v;
      a.ccount[chunk] = 0u;
      __threadfence();
      const unsigned int t = atomicAdd(&a.cg->counter[0], 1u);
      am_last = (t == (unsigned int)a.nchunk - 1) ? 2 : 0;
    }
    __syncthreads();
    if (am_last == 2) {  // last chunk: rho and alpha
      __threadfence();
      double w = 0.0;
      for (int q = tid; q < a.nchunk; q += nthr) w += __ldcg(a.cpart1 + q);
      w = block_sum(w, red);
      if (tid == 0) {
        a.cg->rho = w;
        a.cg->alpha = a.cg->rtz1 / w;
        a.cg->counter[0] = 0u;
      }
    }
  }
  if (tid == 0 && ok) mbar_inval(bar);
}

// One unique point of the update: p = r d + beta p_old, x += alpha p,
// r -= alpha w, then the sums of r^2 d and r^2 binv.
template <bool FIRST>
__device__ __forceinline__ void upd_point(float& x, float& r, float& p, float w, float d, float b,
                                          float alpha, float beta, CompAcc<float>& a1,
                                          CompAcc<float>& a2) {
  if (!FIRST) {
    p = form_p(beta, p, r, d);
    x = fmaf(alpha, p, x);
    r = fmaf(-alpha, w, r);
  }
  const float rr = r * r;
  a1.add(rr * d);
  a2.add(rr * b);
}

// G boundary groups of C copies per thread (C = 0: the class of other sizes,
// through the map's starts), block-strided: every index and value load of
// the G groups is issued before the first use, then the sums (ascending copy
// order), the mask and the point updates.
template <bool FIRST, int C, int G>
__device__ __forceinline__ void upd_groups(const SplitArgs& a, const GsClasses& cls, int k,
                                           int s0, float alpha, float beta, CompAcc<float>& a1,
                                           CompAcc<float>& a2) {
  constexpr int CC = C > 0 ? C : 1;
  const int cnt = cls.cnt[k], soff = cls.soff[k];
  int cp[G][CC];
  bool on[G];
#pragma unroll
  for (int q = 0; q < G; ++q) {
    const int s = s0 + q * kUpdThreads;
    on[q] = s < cnt;
    if (!FIRST && on[q]) {
      if constexpr (C == 1) {
        cp[q][0] = __ldg(a.cpos + cls.ioff[k] + s);
      } else if constexpr (C == 2) {
        const int2 v = __ldg(reinterpret_cast<const int2*>(a.cpos + cls.ioff[k]) + s);
        cp[q][0] = v.x;
        cp[q][1] = v.y;
      } else if constexpr (C >= 4) {
#pragma unroll
        for (int h = 0; h < C / 4; ++h) {
          const int4 v = __ldg(reinterpret_cast<const int4*>(a.cpos + cls.ioff[k]) + (C / 4) * s + h);
          cp[q][4 * h] = v.x;
          cp[q][4 * h + 1] = v.y;
          cp[q][4 * h + 2] = v.z;
          cp[q][4 * h + 3] = v.w;
        }
      }
    }
  }
  const uint64_t pol = l2_policy_evict_first();
  float w[G], x[G], r[G], p[G], d[G], b[G], m[G];
#pragma unroll
  for (int q = 0; q < G; ++q) {
    if (!on[q]) continue;
    const int g = soff + s0 + q * kUpdThreads;
    w[q] = 0.f;
    if (!FIRST) {
      if constexpr (C > 0) {
        float v[CC];
#pragma unroll
        for (int c = 0; c < CC; ++c) v[c] = ld_hint(a.wBc + cp[q][c], pol);
        float t = v[0];
#pragma unroll
        for (int c = 1; c < CC; ++c) t = t + v[c];
        w[q] = t;
      } else {
        const int c0 = __ldg(a.bstart + g), c1 = __ldg(a.bstart + g + 1);
        float t = ld_hint(a.wBc + __ldg(a.cpos + c0), pol);
        for (int c = c0 + 1; c < c1; ++c) t = t + ld_hint(a.wBc + __ldg(a.cpos + c), pol);
        w[q] = t;
      }
      m[q] = __ldg(a.mB + g);
      x[q] = a.xB[g];
      p[q] = a.pB[g];
    } else {
      x[q] = p[q] = 0.f;
    }
    r[q] = a.rB[g];
    d[q] = __ldg(a.dB + g);
    b[q] = __ldg(a.bB + g);
  }
#pragma unroll
  for (int q = 0; q < G; ++q) {
    if (!on[q]) continue;
    const int g = soff + s0 + q * kUpdThreads;
    float ww = FIRST ? 0.f : w[q] * m[q];
    upd_point<FIRST>(x[q], r[q], p[q], ww, d[q], b[q], alpha, beta, a1, a2);
    if (!FIRST) {
      a.xB[g] = x[q];
      a.rB[g] = r[q];
      a.pB[g] = p[q];
    }
  }
}

// K2: blocks [0, nblkI) stream the interior (one float4 per thread), the rest
// take the boundary groups by class (upd_groups).
template <bool FIRST>
__global__ void __launch_bounds__(kUpdThreads) split_update_kernel(const SplitArgs a) {
  __shared__ double red[32];
  __shared__ int am_last;
  if (a.cg->done) return;
  const float alpha = FIRST ? 0.f : (float)a.cg->alpha;
  const float beta = FIRST ? 0.f : (float)a.cg->beta;
  CompAcc<float> a1, a2;
  const int blk = blockIdx.x;
  if (blk < a.nblkI) {
    const int iv = blk * kUpdThreads + threadIdx.x;
    if (iv < a.nI4) {
      float4 r = reinterpret_cast<const float4*>(a.rI)[iv];
      const float4 d = reinterpret_cast<const float4*>(a.dI)[iv];
      const float4 b = reinterpret_cast<const float4*>(a.bI)[iv];
      float4 x = make_float4(0.f, 0.f, 0.f, 0.f), p = x, w = x;
      if (!FIRST) {
        x = reinterpret_cast<const float4*>(a.xI)[iv];
        p = reinterpret_cast<const float4*>(a.pI)[iv];
        w = ld_hint4(a.wI + 4 * (size_t)iv, l2_policy_evict_first());
      }
      upd_point<FIRST>(x.x, r.x, p.x, w.x, d.x, b.x, alpha, beta, a1, a2);
      upd_point<FIRST>(x.y, r.y, p.y, w.y, d.y, b.y, alpha, beta, a1, a2);
      upd_point<FIRST>(x.z, r.z, p.z, w.z, d.z, b.z, alpha, beta, a1, a2);
      upd_point<FIRST>(x.w, r.w, p.w, w.w, d.w, b.w, alpha, beta, a1, a2);
      if (!FIRST) {
        reinterpret_cast<float4*>(a.xI)[iv] = x;
        reinterpret_cast<float4*>(a.rI)[iv] = r;
        reinterpret_cast<float4*>(a.pI)[iv] = p;
      }
    }
  } else {
    const int bb = blk - a.nblkI;
    const GsClasses& C = a.cls;
    int k = 0;
    while (k < kGsClasses - 1 && bb >= C.boff[k + 1]) ++k;
    const int s0 = (bb - C.boff[k]) * kUpdThreads * C.g[k] + threadIdx.x;
    switch (k) {
      case 0: upd_groups<FIRST, 1, 4>(a, C, 0, s0, alpha, beta, a1, a2); break;
      case 1: upd_groups<FIRST, 2, 4>(a, C, 1, s0, alpha, beta, a1, a2); break;
      case 2: upd_groups<FIRST, 4, 2>(a, C, 2, s0, alpha, beta, a1, a2); break;
      case 3: upd_groups<FIRST, 8, 1>(a, C, 3, s0, alpha, beta, a1, a2); break;
      default: upd_groups<FIRST, 0, 1>(a, C, 4, s0, alpha, beta, a1, a2); break;
    }
  }
  const double b1 = block_sum_comp(a1, red);
  const double b2 = block_sum_comp(a2, red);
  const int nblk = gridDim.x;
  if (threadIdx.x == 0) {
    a.part2[blk] = b1;
    a.part2[nblk + blk] = b2;
    __threadfence();
    const unsigned int t = atomicAdd(&a.cg->counter[1], 1u);
    am_last = (t == (unsigned int)nblk - 1);
  }
  __syncthreads();
  if (!am_last) return;
  __threadfence();
  double t1 = 0.0, t2 = 0.0;
  for (int q = threadIdx.x; q < nblk; q += kUpdThreads) {
    t1 += __ldcg(a.part2 + q);
    t2 += __ldcg(a.part2 + nblk + q);
  }
  const double s1 = block_sum(t1, red);
  const double s2 = block_sum(t2, red);
  if (threadIdx.x == 0) cg_finalize(a.cg, s1, s2);
}

// ---- layout conversions (once per outer step, not per iteration) ----------

// Interior and boundary slots of the split layout from an element-local FP64
// vector, times sc; the padding slots get 0.
__global__ void split_from_local_kernel(float* __restrict__ vI, float* __restrict__ vB,
                                        const double* __restrict__ src, double sc, int nx,
                                        int NI, int NIp, int64_t nI, const int* __restrict__ bfirst,
                                        int nb, int nbp) {
  const int P = nx * nx * nx, m = nx - 2;
  const int64_t tot = nI + nbp;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < tot;
       t += (int64_t)gridDim.x * blockDim.x) {
    if (t < nI) {
      const int64_t e = t / NIp;
      const int c = (int)(t - e * NIp);
      float v = 0.f;
      if (c < NI) {
        const int i = 1 + c % m, j = 1 + (c / m) % m, k = 1 + c / (m * m);
        v = (float)(src[e * P + (k * nx + j) * nx + i] * sc);
      }
      vI[t] = v;
    } else {
      const int g = (int)(t - nI);
      vB[g] = g < nb ? (float)(src[bfirst[g]] * sc) : 0.f;
    }
  }
}

// x64 += sc * x32 at every element-local point.
__global__ void split_axpy_kernel(double* __restrict__ x, const float* __restrict__ xI,
                                  const float* __restrict__ xB, const int* __restrict__ gmap,
                                  double sc, int nx, int NIp, int NBp, int64_t n) {
  const int P = nx * nx * nx;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = t / P;
    const int pt = (int)(t - e * P);
    const int i = pt % nx, j = (pt / nx) % nx, k = pt / (nx * nx);
    const int rank = interior_before(nx, i, j, k);
    const float v = is_interior(nx, i, j, k) ? xI[e * NIp + rank]
                                             : xB[gmap[e * NBp + (pt - rank)]];
    x[t] = fma(sc, (double)v, x[t]);
  }
}

// Sums of r^2 d and r^2 binv over the split layout (block partials).
__global__ void split_rz_kernel(const float* __restrict__ rI, const float* __restrict__ dI,
                                const float* __restrict__ bI, int64_t nI,
                                const float* __restrict__ rB, const float* __restrict__ dB,
                                const float* __restrict__ bB, int nb, double* __restrict__ part) {
  __shared__ double red[32];
  CompAcc<float> a1, a2;
  const int64_t tot = nI + nb;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < tot;
       t += (int64_t)gridDim.x * blockDim.x) {
    float r, d, b;
    if (t < nI) {
      r = rI[t];
      d = dI[t];
      b = bI[t];
    } else {
      r = rB[t - nI];
      d = dB[t - nI];
      b = bB[t - nI];
    }
    const float rr = r * r;
    a1.add(rr * d);
    a2.add(rr * b);
  }
  const double b1 = block_sum_comp(a1, red);
  const double b2 = block_sum_comp(a2, red);
  if (threadIdx.x == 0) {
    part[blockIdx.x] = b1;
    part[gridDim.x + blockIdx.x] = b2;
  }
}

__global__ void scale_f32_kernel(float* __restrict__ a, float f, int64_t n) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x)
    a[t] *= f;
}

inline int grid_for(int64_t n) {
  return (int)std::min<int64_t>(std::max<int64_t>((n + 255) / 256, 1), 152 * 8);
}

template <int NX, int EPB>
cudaError_t launch_k1_nx(const SplitArgs& a, int nblk, cudaStream_t s) {
  const int hb = a.h2mode ? 1 : 0, hh1 = a.h1mode == 1 ? 1 : 0, hh2 = a.h2mode == 2 ? 1 : 0;
  static std::atomic<uint32_t> configured{0};  // per device
  if (first_on_device(configured)) {
    const int maxb = (int)split_smem_bytes<NX, EPB>(1, 1, 1);
    cudaError_t e = cudaFuncSetAttribute(split_ax_kernel<NX, EPB>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, maxb);
    if (e != cudaSuccess) return e;
    cudaFuncSetAttribute(split_ax_kernel<NX, EPB>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         100);
    mark_device(configured);
  }
  count_launch();
  split_ax_kernel<NX, EPB><<<nblk, dim3(NX * NX, EPB), split_smem_bytes<NX, EPB>(hb, hh1, hh2), s>>>(a);
  return cudaGetLastError();
}

// Elements per operator block by lx1: about 128 threads for the small orders,
// one element (lx1^2 threads) from lx1 = 8 on.
int split_epb(int nx) { return nx == 4 ? 8 : nx == 6 ? 2 : 1; }

cudaError_t launch_k1(int nx, const SplitArgs& a, int nblk, cudaStream_t s) {
  switch (nx) {
    case 4: return launch_k1_nx<4, 8>(a, nblk, s);
    case 6: return launch_k1_nx<6, 2>(a, nblk, s);
    case 8: return launch_k1_nx<8, 1>(a, nblk, s);
    case 10: return launch_k1_nx<10, 1>(a, nblk, s);
    case 12: return launch_k1_nx<12, 1>(a, nblk, s);
    default: return cudaErrorInvalidValue;
  }
}

SplitArgs make_args(Handle& h, SplitLayout& L, const Coef<float>& c) {
  SplitArgs a{};
  const Mesh& m = h.mesh;
  a.G = m.f32.G;
  a.bm1 = m.f32.bm1;
  a.h1 = c.h1;
  a.h2 = c.h2;
  a.h1s = c.h1s;
  a.h2s = c.h2s;
  a.h1mode = c.h1mode;
  a.h2mode = c.h2mode;
  a.D = m.f32.D;
  a.nel = m.nel;
  a.gmap = L.gmap.ptr;
  a.bpt = L.bpt.ptr;
  a.rI = L.rI.ptr;
  a.pI = L.pI.ptr;
  a.xI = L.xI.ptr;
  a.wI = L.wI.ptr;
  a.dI = L.dI.ptr;
  a.bI = L.bI.ptr;
  a.rB = L.rB.ptr;
  a.pB = L.pB.ptr;
  a.xB = L.xB.ptr;
  a.dB = L.dB.ptr;
  a.bB = L.bB.ptr;
  a.mB = L.mB.ptr;
  a.wBc = L.wBc.ptr;
  a.bstart = m.gs.bstart;
  a.cpos = L.cpos.ptr;
  a.cls = L.cls;
  a.nb = L.nb;
  a.nI4 = (int)((int64_t)L.nel * L.NIp / 4);
  a.nblkI = L.nblkI;
  a.cg = h.cg;
  a.part1 = L.part1.ptr;
  a.cpart1 = L.cpart1.ptr;
  a.ccount = L.ccount.ptr;
  a.nchunk = L.nchunk;
  a.part2 = L.part2.ptr;
  a.err = m.dev_err;
  return a;
}

}  // namespace

bool split_eligible(const Handle& h) {
  const Mesh& m = h.mesh;
  const int nx = m.nx1;
  if (!h.use_split) return false;
  if (nx != 4 && nx != 6 && nx != 8 && nx != 10 && nx != 12) return false;
  if (m.gs.skip) return false;  // an interior point shared through the numbering
  if (!m.use_tma) return false;
  // 16-byte alignment of every staged slice (cudaMalloc'ed arrays are)
  auto al = [](const void* p) { return ((uintptr_t)p & 15u) == 0; };
  return al(m.f32.G) && al(m.f32.bm1);
}

// Maps of the layout from the PCG-form gather-scatter maps (host, once per
// mesh): gmap (group of each local boundary point), cpos (wBc position of
// each copy, parallel to the map's idx), bfirst (first copy of each group),
// bpt (natural point of each boundary index).
int split_setup(Handle& h) {
  Mesh& m = h.mesh;
  if (!h.split) h.split.reset(new SplitLayout());
  SplitLayout& L = *h.split;
  if (L.ready && L.nx == m.nx1 && L.nel == m.nel) return 0;
  L.ready = false;
  const int nx = m.nx1, P = nx * nx * nx;
  L.nx = nx;
  L.nel = m.nel;
  L.NI = (nx - 2) * (nx - 2) * (nx - 2);
  L.NB = P - L.NI;
  L.NIp = (L.NI + 3) / 4 * 4;
  L.NBp = (L.NB + 3) / 4 * 4;
  L.nb = m.gs.nbseg;
  L.nbp = (L.nb + 3) / 4 * 4;
  L.cls = m.gs.cls;
  L.epb = split_epb(nx);
  L.nblk1 = (m.nel + L.epb - 1) / L.epb;
  L.nchunk = (L.nblk1 + kChunk - 1) / kChunk;
  const int64_t nI = (int64_t)m.nel * L.NIp;
  L.nblkI = (int)((nI / 4 + kUpdThreads - 1) / kUpdThreads);
  int nblkB = 0;
  const int gpt[kGsClasses] = {4, 4, 2, 1, 1};  // groups per thread (upd_groups)
  for (int k = 0; k < kGsClasses; ++k) {
    L.cls.g[k] = gpt[k];
    L.cls.boff[k] = nblkB;
    nblkB += (L.cls.cnt[k] + kUpdThreads * gpt[k] - 1) / (kUpdThreads * gpt[k]);
  }
  L.cls.boff[kGsClasses] = nblkB;
  L.nblk2 = std::max(L.nblkI + nblkB, 1);
  // host copies of the PCG-form maps
  std::vector<int> bst((size_t)m.gs.nbseg + 1), bix((size_t)m.gs.nbidx);
  if (cudaMemcpy(bst.data(), m.gs.bstart, bst.size() * sizeof(int), cudaMemcpyDeviceToHost) !=
          cudaSuccess ||
      (!bix.empty() && cudaMemcpy(bix.data(), m.gs.bidx, bix.size() * sizeof(int),
                                  cudaMemcpyDeviceToHost) != cudaSuccess)) {
    set_error(h, "split layout: map download failed");
    return -3;
  }
  std::vector<int> gmap((size_t)m.nel * L.NBp, 0), cpos(bix.size(), 0), bfirst((size_t)L.nbp, 0);
  std::vector<unsigned short> bpt((size_t)L.NB);
  for (int pt = 0; pt < P; ++pt) {
    const int i = pt % nx, j = (pt / nx) % nx, k = pt / (nx * nx);
    if (!is_interior(nx, i, j, k)) bpt[(size_t)(pt - interior_before(nx, i, j, k))] = (unsigned short)pt;
  }
  std::vector<int> seen((size_t)m.nel * L.NBp, 0);
  auto copies = [&](int g, int& a, int& b) {  // copies of group g in the map's idx
    int k = 0;
    while (k < kGsClasses - 1 && g >= m.gs.cls.soff[k] + m.gs.cls.cnt[k]) ++k;
    a = bst[(size_t)g];
    b = k < kGsClasses - 1 ? a + (1 << k) : bst[(size_t)g + 1];
  };
  for (int g = 0; g < L.nb; ++g) {
    int a, b;
    copies(g, a, b);
    bfirst[(size_t)g] = bix[(size_t)a];
    for (int c = a; c < b; ++c) {
      const int li = bix[(size_t)c];
      const int e = li / P, pt = li % P;
      const int i = pt % nx, j = (pt / nx) % nx, k = pt / (nx * nx);
      if (is_interior(nx, i, j, k)) {
        set_error(h, "split layout: an interior point in a boundary group");
        return -1;
      }
      const int bidx = pt - interior_before(nx, i, j, k);
      const size_t pos = (size_t)e * L.NBp + bidx;
      gmap[pos] = g;
      seen[pos] = 1;
      cpos[(size_t)c] = (int)pos;
    }
  }
  for (int e = 0; e < m.nel; ++e)
    for (int b = 0; b < L.NB; ++b)
      if (!seen[(size_t)e * L.NBp + b]) {
        set_error(h, "split layout: an element-boundary point outside every group");
        return -1;
      }
  const size_t nB = (size_t)std::max(L.nbp, 4);
  if (L.gmap.ensure(gmap.size()) || L.cpos.ensure(std::max<size_t>(cpos.size(), 1)) ||
      L.bfirst.ensure(nB) || L.bpt.ensure(bpt.size()) || L.rI.ensure(nI) || L.pI.ensure(nI) ||
      L.xI.ensure(nI) || L.wI.ensure(nI) || L.dI.ensure(nI) || L.bI.ensure(nI) || L.rB.ensure(nB) ||
      L.pB.ensure(nB) || L.xB.ensure(nB) || L.dB.ensure(nB) || L.bB.ensure(nB) ||
      L.mB.ensure(nB) || L.wBc.ensure((size_t)m.nel * L.NBp) || L.part1.ensure(L.nblk1) ||
      L.cpart1.ensure(L.nchunk) || L.ccount.ensure(L.nchunk) || L.part2.ensure(2 * (size_t)L.nblk2)) {
    set_error(h, "split layout: device allocation failed");
    return -4;
  }
  cudaStream_t s = h.stream;
  cudaMemcpyAsync(L.gmap.ptr, gmap.data(), gmap.size() * sizeof(int), cudaMemcpyHostToDevice, s);
  if (!cpos.empty())
    cudaMemcpyAsync(L.cpos.ptr, cpos.data(), cpos.size() * sizeof(int), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(L.bfirst.ptr, bfirst.data(), bfirst.size() * sizeof(int), cudaMemcpyHostToDevice,
                  s);
  cudaMemcpyAsync(L.bpt.ptr, bpt.data(), bpt.size() * sizeof(unsigned short),
                  cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(L.ccount.ptr, 0, L.nchunk * sizeof(unsigned int), s);
  cudaMemsetAsync(L.wBc.ptr, 0, (size_t)m.nel * L.NBp * sizeof(float), s);
  cudaMemsetAsync(L.wI.ptr, 0, nI * sizeof(float), s);
  if (cudaStreamSynchronize(s) != cudaSuccess) {
    set_error(h, std::string("split layout: ") + cudaGetErrorString(cudaGetLastError()));
    return -3;
  }
  L.ready = true;
  return 0;
}

// Operator data of one inner solve in the layout: d and binv from the FP64
// element-local arrays, the mask per group.  r from r64 / scale; x, p = 0.
int split_load(Handle& h, const double* r64, double inv_scale, const double* d64,
               const double* binv64, const double* mask64) {
  SplitLayout& L = *h.split;
  cudaStream_t s = h.stream;
  const int64_t nI = (int64_t)L.nel * L.NIp;
  const int gr = grid_for(nI + L.nbp);
  auto conv = [&](float* vI, float* vB, const double* src, double sc) {
    count_launch();
    split_from_local_kernel<<<gr, 256, 0, s>>>(vI, vB, src, sc, L.nx, L.NI, L.NIp, nI,
                                               L.bfirst.ptr, L.nb, L.nbp);
  };
  conv(L.dI.ptr, L.dB.ptr, d64, 1.0);
  conv(L.bI.ptr, L.bB.ptr, binv64, 1.0);
  conv(L.rI.ptr, L.rB.ptr, r64, inv_scale);
  // mask per group (the interior check of the solve guarantees 1 inside)
  count_launch();
  split_from_local_kernel<<<gr, 256, 0, s>>>(L.xI.ptr, L.mB.ptr, mask64, 1.0, L.nx, L.NI, L.NIp,
                                             nI, L.bfirst.ptr, L.nb, L.nbp);
  cudaMemsetAsync(L.xI.ptr, 0, nI * sizeof(float), s);
  cudaMemsetAsync(L.xB.ptr, 0, (size_t)L.nbp * sizeof(float), s);
  cudaMemsetAsync(L.pI.ptr, 0, nI * sizeof(float), s);
  cudaMemsetAsync(L.pB.ptr, 0, (size_t)L.nbp * sizeof(float), s);
  return cuda_pending(h, "split load") ? -3 : 0;
}

// The iteration-1 check of the inner solve (no update): rtz, norm, beta = 0.
int split_first_check(Handle& h, const Coef<float>& c) {
  SplitLayout& L = *h.split;
  const SplitArgs a = make_args(h, L, c);
  count_launch();
  split_update_kernel<true><<<L.nblk2, kUpdThreads, 0, h.stream>>>(a);
  return cuda_pending(h, "split first check") ? -3 : 0;
}

// Iterations until the device flags the solve done (as pcg_iterate).
PcgResult split_iterate(Handle& h, const Coef<float>& c) {
  PcgResult res;
  SplitLayout& L = *h.split;
  cudaStream_t s = h.stream;
  const SplitArgs a = make_args(h, L, c);
  const int chunk = std::max(1, h.graph_chunk);
  if (h.timing && h.ax_ev.size() < 4 * (size_t)chunk) {
    for (cudaEvent_t e : h.ax_ev) cudaEventDestroy(e);
    h.ax_ev.assign(4 * (size_t)chunk, nullptr);
    for (auto& e : h.ax_ev) cudaEventCreate(&e);
  }
  auto enqueue_chunk = [&](int k) -> cudaError_t {
    for (int q = 0; q < k; ++q) {
      if (h.timing) cudaEventRecord(h.ax_ev[4 * q], s);
      cudaError_t e = launch_k1(L.nx, a, L.nblk1, s);
      if (e != cudaSuccess) return e;
      if (h.timing) cudaEventRecord(h.ax_ev[4 * q + 1], s);
      count_launch();
      split_update_kernel<false><<<L.nblk2, kUpdThreads, 0, s>>>(a);
      if (h.timing) cudaEventRecord(h.ax_ev[4 * q + 2], s);
    }
    return cudaGetLastError();
  };
  bool graph = h.use_graph && !h.timing;
  if (graph) {
    Handle::GraphKey key;
    const void* ptrs[15] = {L.rI.ptr, L.pI.ptr, L.xI.ptr, L.wI.ptr, L.rB.ptr, L.pB.ptr,
                            L.xB.ptr, L.wBc.ptr, c.h1,    c.h2,     h.mesh.f32.G, L.gmap.ptr,
                            L.dI.ptr, L.mB.ptr, nullptr};
    for (int i = 0; i < 15; ++i) key.ptr[i] = ptrs[i];
    key.ints[0] = 100;  // split form
    key.ints[1] = c.h1mode;
    key.ints[2] = c.h2mode;
    key.ints[3] = L.nblk1;
    key.ints[4] = chunk;
    key.ints[5] = h.mesh.nel;
    key.dbl[0] = (double)c.h1s;
    key.dbl[1] = (double)c.h2s;
    if (!h.gexec || !(key == h.gkey)) {
      if (h.gexec) cudaGraphExecDestroy(h.gexec);
      h.gexec = nullptr;
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed);
      capturing() = true;
      if (e == cudaSuccess) e = enqueue_chunk(chunk);
      capturing() = false;
      cudaError_t e2 = cudaStreamEndCapture(s, &g);
      if (e == cudaSuccess) e = e2;
      if (e == cudaSuccess) e = cudaGraphInstantiate(&h.gexec, g, 0);
      if (g) cudaGraphDestroy(g);
      if (e != cudaSuccess) {
        cudaGetLastError();
        h.gexec = nullptr;
        graph = false;
      } else {
        h.gkey = key;
        h.gchunk = chunk;
      }
    }
  }
  int launched = 0, iter_before = 0;
  for (;;) {
    cudaMemcpyAsync(h.cg_host, h.cg, sizeof(CgScalars), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) {
      res.status = -3;
      set_error(h, std::string("split pcg: ") + cudaGetErrorString(cudaGetLastError()));
      return res;
    }
    if (h.timing && launched) {
      const int live = std::min(launched, h.cg_host->iter - iter_before);
      auto span = [&](int x, int y) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, h.ax_ev[x], h.ax_ev[y]) != cudaSuccess) {
          cudaGetLastError();
          ms = 0.f;
        }
        return (double)ms;
      };
      for (int q = 0; q < live; ++q) {
        h.ms_axhelm += span(4 * q, 4 * q + 1);
        h.ms_update += span(4 * q + 1, 4 * q + 2);
      }
      h.n_axhelm += live;
    }
    if (h.cg_host->done) break;
    iter_before = h.cg_host->iter;
    cudaError_t e;
    int k;
    if (graph) {
      k = chunk;
      count_launch(2LL * chunk);
      e = cudaGraphLaunch(h.gexec, s);
    } else {
      const int left = h.cg_host->maxiter - h.cg_host->iter + 1;
      k = std::min(chunk, std::max(left, 1));
      e = enqueue_chunk(k);
    }
    if (e != cudaSuccess) {
      res.status = -3;
      set_error(h, std::string("split pcg launch: ") + cudaGetErrorString(e));
      return res;
    }
    launched = k;
  }
  int derr = 0;
  if (h.mesh.dev_err) {
    cudaMemcpyAsync(&derr, h.mesh.dev_err, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    if (derr) {
      res.status = -3;
      set_error(h, "split pcg: a bounded wait for a bulk copy expired");
      return res;
    }
  }
  const CgScalars& fin = *h.cg_host;
  res.niter = fin.niter;
  res.rbn0 = fin.rbn0;
  res.rbn2 = fin.rbn2;
  if (fin.nonfinite) {
    res.status = -7;
    set_error(h, "split pcg: non-finite residual norm");
  } else if (!(fin.rbn2 <= fin.tol) && fin.iter > fin.maxiter) {
    res.status = -5;
  }
  return res;
}

void split_axpy(Handle& h, double* x64, double scale) {
  SplitLayout& L = *h.split;
  const int64_t n = h.mesh.n;
  count_launch();
  split_axpy_kernel<<<grid_for(n), 256, 0, h.stream>>>(x64, L.xI.ptr, L.xB.ptr, L.gmap.ptr, scale,
                                                      L.nx, L.NIp, L.NBp, n);
}

// Residual replacement in the layout (see mixed_replace_into): r = r64 /
// s_new, p rescaled by scale / s_new (exact: powers of two), x = 0, and the
// host scalars of the last check updated for the new r.
int split_replace(Handle& h, const double* r64, double& scale, double inner_tol, int* restarts) {
  SplitLayout& L = *h.split;
  const Mesh& m = h.mesh;
  cudaStream_t s = h.stream;
  int st = 0;
  const double amax = device_absmax<double>(h, r64, m.n, &st);
  if (st) return -3;
  if (amax == 0.0) return 1;
  const double s_new = std::ldexp(1.0, std::ilogb(amax));
  const double ratio = scale / s_new;
  const int64_t nI = (int64_t)L.nel * L.NIp;
  const int gr = grid_for(nI + L.nbp);
  count_launch(4);
  split_from_local_kernel<<<gr, 256, 0, s>>>(L.rI.ptr, L.rB.ptr, r64, 1.0 / s_new, L.nx, L.NI,
                                             L.NIp, nI, L.bfirst.ptr, L.nb, L.nbp);
  scale_f32_kernel<<<grid_for(nI), 256, 0, s>>>(L.pI.ptr, (float)ratio, nI);
  scale_f32_kernel<<<grid_for(L.nbp), 256, 0, s>>>(L.pB.ptr, (float)ratio, L.nbp);
  cudaMemsetAsync(L.xI.ptr, 0, nI * sizeof(float), s);
  cudaMemsetAsync(L.xB.ptr, 0, (size_t)L.nbp * sizeof(float), s);
  const int nb = grid_for(nI + L.nb);
  if (h.red.ensure(2 * (size_t)nb)) return -4;
  split_rz_kernel<<<nb, 256, 0, s>>>(L.rI.ptr, L.dI.ptr, L.bI.ptr, nI, L.rB.ptr, L.dB.ptr,
                                     L.bB.ptr, L.nb, h.red.ptr);
  std::vector<double> hp(2 * (size_t)nb);
  cudaMemcpyAsync(hp.data(), h.red.ptr, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) {
    set_error(h, std::string("split replace: ") + cudaGetErrorString(cudaGetLastError()));
    return -3;
  }
  double s1 = 0.0, s2 = 0.0;
  for (int b = 0; b < nb; ++b) {
    s1 += hp[(size_t)b];
    s2 += hp[(size_t)nb + b];
  }
  CgScalars& c = *h.cg_host;
  const double rec = c.rbn2 * ratio;
  c.rtz2 = c.rtz2 * ratio * ratio;
  c.rtz1 = s1;
  c.rbn0 = std::sqrt(s2 / m.vol);
  c.beta = (c.rbn0 <= 2.0 * rec) ? s1 / c.rtz2 : 0.0;
  if (c.beta == 0.0 && restarts) ++*restarts;
  c.rbn2 = c.rbn0;
  c.tol = inner_tol * c.rbn0;
  c.done = 0;
  c.counter[0] = c.counter[1] = c.counter[2] = c.counter[3] = 0u;
  cudaMemcpyAsync(h.cg, &c, sizeof(CgScalars), cudaMemcpyHostToDevice, s);
  scale = s_new;
  return 0;
}

}  // namespace nekgpu
