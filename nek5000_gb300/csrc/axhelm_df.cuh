// axhelm_df.cuh -- the FP64 operator with its tensor contractions in
// double-float arithmetic on the FP32 pipe.
//
// GB300 issues FP32 fused multiply-adds at about 64 times its FP64 rate, and
// the FP64 operator (axhelm.cuh) is bound by the FP64 pipe at a tenth of the
// HBM bandwidth.  Here the mathematics and contraction order of
// core/hmholtz.f:191-217 stay, but every value inside the contractions is a
// pair (hi, lo) of FP32 numbers whose sum carries 48 significant bits:
//
//   * the FP64 input p is split once per point, hi = fl32(p),
//     lo = fl32(p - hi); the geometric factors G1..G6 and D come split from
//     setup (OpData::Gdf, the D pairs in shared memory);
//   * each product-accumulate is Dekker's TwoProduct (the exact error of
//     hi*hi from one fused multiply-add) plus the two cross products, added
//     into a running (sum, error) pair by Knuth's TwoSum -- the compensated
//     dot product of Ogita, Rump and Oishi (SIAM J. Sci. Comput. 26, 2005),
//     whose result is as accurate as if computed with twice the working
//     precision and then rounded;
//   * the element-local result hi + lo is formed in FP64, where the mass
//     term h2 B p, the PCG's p update and its rho dot product stay.
//
// Per point this leaves about six FP64 operations (the p update, the
// recombination, the mass term, the rho dot) against 121 in the FP64 kernel;
// the conversions of the split and the recombination are integer operations
// (df_split_int, df_widen), the rest runs on the FP32 pipe.  The result differs from the FP64 operator by a few
// units in 2^-48 of the magnitude of the summed terms.
#pragma once
#include "axhelm.cuh"

namespace nekgpu {

struct DfPair {
  float h, l;
};

__device__ __forceinline__ DfPair df_split(double v) {
  const float h = __double2float_rn(v);
  return {h, __double2float_rn(v - (double)h)};
}

__device__ __forceinline__ double df_join(float h, float l) { return (double)h + (double)l; }

// The same split and join with the conversions done by integer operations.
// On GB300 FP32 <-> FP64 conversions issue on the FP64 pipe (2 results per
// clock per SM); split and join took about five of them per point, more pipe
// time than the operator's FP64 arithmetic.
//
// Split: |v|'s bit pattern rounded at bit 29 (half away from zero; a carry
// runs into the exponent, as the value does) is hi's significand and
// exponent; |v| - |hi| is the integer difference of the two patterns in units
// of ulp(v) (at most 2^28 in magnitude), so lo = fl32(that integer) * ulp(v)
// is fl32(v - hi) exactly.  hi equals fl32(v) except at exact ties, where it
// is the other neighbour and lo keeps the pair exact.  Outside
// 2^-74 <= |v| < 2^126 (ulp(v) or hi out of the FP32 normal range), and for
// infinities and NaN, the FP64 form runs.
__device__ __forceinline__ DfPair df_split_int(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const unsigned long long a = b & 0x7FFFFFFFFFFFFFFFull;
  const float sgn = (b >> 63) ? -1.0f : 1.0f;
  if (a == 0ull) return {sgn * 0.0f, 0.0f};
  const int E = (int)(a >> 52);
  if (E < 949 || E > 1149) return df_split(v);
  const unsigned long long r = (a + (1ull << 28)) & ~((1ull << 29) - 1ull);
  const float h = __uint_as_float((unsigned int)((r >> 29) - (896ull << 23)));
  const int rem = (int)(long long)(a - r);
  const float l = __int2float_rn(rem) * __int_as_float((E - 948) << 23);
  return {sgn * h, sgn * l};
}

// (double)f by assembling the FP64 bit pattern (normal f and zeros; others
// convert).
__device__ __forceinline__ double df_widen(float f) {
  const unsigned int u = __float_as_uint(f);
  const unsigned int e = (u >> 23) & 0xFFu;
  if (e == 0u && (u & 0x7FFFFFu) == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
  if (e == 0u || e == 0xFFu) return (double)f;
  const unsigned int hi = (u & 0x80000000u) | ((e + 896u) << 20) | ((u >> 3) & 0xFFFFFu);
  return __hiloint2double((int)hi, (int)(u << 29));
}

__device__ __forceinline__ double df_join_int(float h, float l) {
  return df_widen(h) + df_widen(l);
}

// (sh, sl) += (ah, al) * (bh, bl): TwoProduct of the high parts, the cross
// products into its error, TwoSum into the running sum; sl gathers the
// errors (normalised once at the end by df_norm).
__device__ __forceinline__ void df_mac(float& sh, float& sl, float ah, float al, float bh,
                                       float bl) {
  const float p = ah * bh;
  float e = fmaf(ah, bh, -p);
  e = fmaf(ah, bl, e);
  e = fmaf(al, bh, e);
  const float s = sh + p;
  const float bb = s - sh;
  const float t = (sh - (s - bb)) + (p - bb);
  sh = s;
  sl += t + e;
}

// First term of a sum: (sh, sl) = (ah, al) * (bh, bl).
__device__ __forceinline__ void df_mul(float& sh, float& sl, float ah, float al, float bh,
                                       float bl) {
  const float p = ah * bh;
  float e = fmaf(ah, bh, -p);
  e = fmaf(ah, bl, e);
  sl = fmaf(al, bh, e);
  sh = p;
}

// Renormalise (|sl| small against |sh|): FastTwoSum.
__device__ __forceinline__ void df_norm(float& sh, float& sl) {
  const float s = sh + sl;
  sl = sl - (s - sh);
  sh = s;
}

// (sh, sl) += (ah, al): TwoSum of the high parts.
__device__ __forceinline__ void df_add(float& sh, float& sl, float ah, float al) {
  const float s = sh + ah;
  const float bb = s - sh;
  const float t = (sh - (s - bb)) + (ah - bb);
  sh = s;
  sl += t + al;
}

// Shared memory of the kernel: D and D^T pairs (padded rows), then three
// padded slabs of pairs per element.  (Staging the block's G pairs in shared
// memory as well, by one bulk copy, measured slower on GB300: 1.25 against
// 0.87 ms per launch at E=32^3 N=7, the larger blocks halving the resident
// warps.)
template <int NX>
__host__ __device__ constexpr size_t axhelm_df_smem_bytes(int epb) {
  return (size_t)(2 * NX * (NX + 1) + epb * 3 * AxShape<NX>::LP) * sizeof(float2);
}

// Arguments beyond AxArgs<double>: the split geometric factors.
struct DfArgs {
  AxArgs<double> a;
  const float2* Gdf;  // [e][6][P] (hi, lo) pairs of G1..G6
  const float2* Ddf;  // [NX][NX] (hi, lo) pairs of D, row-major
};

// Block body (threads (NX*NX, epb), as axhelm_body).
template <int NX, bool FUSED>
__device__ __forceinline__ void axhelm_df_body(const DfArgs& A, int blk, int tx, int ty, int epb,
                                               unsigned char* smem_raw) {
  constexpr int R = AxShape<NX>::R, LP = AxShape<NX>::LP, P = AxShape<NX>::P;
  constexpr int NXY = NX * NX;
  const AxArgs<double>& a = A.a;
  float2* sD = reinterpret_cast<float2*>(smem_raw);  // sD[i*R+l]  = D[i][l]
  float2* sDT = sD + NX * R;                         // sDT[i*R+l] = D[l][i]
  const int tyc = ty < epb ? ty : 0;
  float2* su = sDT + NX * R + tyc * 3 * LP;
  float2* st1 = su + LP;
  float2* st2 = st1 + LP;

  const int i = tx % NX, j = tx / NX;
  const int ft = tx + NXY * ty, nthr = NXY * epb;
  if (ty < epb)
    for (int q = ft; q < NXY; q += nthr) {
      const int r = q / NX, c = q % NX;
      const float2 v = A.Ddf[q];
      sD[r * R + c] = v;
      sDT[c * R + r] = v;
    }
  const int e = blk * epb + ty;
  const bool act = ty < epb && e < a.nel;
  const size_t eo = (size_t)(act ? e : 0) * P;

  double beta = 0.0, zmean = 0.0;
  bool mcor = false;
  if constexpr (FUSED) {
    beta = a.cg->beta;
    mcor = a.cg->mcor != 0;
    if (mcor) zmean = a.cg->zmean;
  }
  const bool unit_h1 = a.h1mode == 0 && a.h1s == 1.0;
  const DfPair h1c = df_split(a.h1s);

  double ru64[NX];
  float ruh[NX], rul[NX];
#pragma unroll
  for (int k = 0; k < NX; ++k) {
    const int pt = k * NXY + j * NX + i;
    double v = 0.0;
    if (act) {
      if constexpr (FUSED) {
        double z = a.r[eo + pt] * a.d[eo + pt];
        if (mcor) z = z + zmean;       // cadd(z,rmean) (hmholtz.f:749)
        v = fma(beta, a.u[eo + pt], z);  // add2s1: p = beta*p + z
        a.p[eo + pt] = v;
      } else {
        v = a.u[eo + pt];
      }
    }
    ru64[k] = v;
    const DfPair s = df_split_int(v);
    ruh[k] = s.h;
    rul[k] = s.l;
    if (ty < epb) su[k * NX * R + j * R + i] = make_float2(s.h, s.l);
  }
  __syncthreads();

  float rauh[NX], raul[NX];
  const float2* __restrict__ g = A.Gdf + (size_t)(act ? e : 0) * 6 * P;
  // G pairs of plane k are loaded one plane ahead, so that their latency
  // hides behind plane k - 1's contractions
  float2 gn[6];
  auto load_g = [&](int k) {
    const int pt = k * NXY + j * NX + i;
#pragma unroll
    for (int q = 0; q < 6; ++q) gn[q] = act ? __ldg(g + q * P + pt) : make_float2(0.f, 0.f);
  };
  load_g(0);
#pragma unroll
  for (int k = 0; k < NX; ++k) {
    const float2 g1 = gn[0], g2 = gn[1], g3 = gn[2], g4 = gn[3], g5 = gn[4], g6 = gn[5];
    if (k + 1 < NX) load_g(k + 1);
    const float2* slab = su + k * NX * R;
    float urh, url, ush, usl, uth, utl;
    {
      float2 dd = sD[i * R], uu = slab[j * R];
      df_mul(urh, url, dd.x, dd.y, uu.x, uu.y);
#pragma unroll 2
      for (int l = 1; l < NX; ++l) {
        dd = sD[i * R + l];
        uu = slab[j * R + l];
        df_mac(urh, url, dd.x, dd.y, uu.x, uu.y);
      }
      df_norm(urh, url);
    }
    {
      float2 uu = slab[i], dd = sD[j * R];
      df_mul(ush, usl, uu.x, uu.y, dd.x, dd.y);
#pragma unroll 2
      for (int l = 1; l < NX; ++l) {
        uu = slab[l * R + i];
        dd = sD[j * R + l];
        df_mac(ush, usl, uu.x, uu.y, dd.x, dd.y);
      }
      df_norm(ush, usl);
    }
    {
      float2 dd = sD[k * R];
      df_mul(uth, utl, ruh[0], rul[0], dd.x, dd.y);
#pragma unroll
      for (int l = 1; l < NX; ++l) {
        dd = sD[k * R + l];
        df_mac(uth, utl, ruh[l], rul[l], dd.x, dd.y);
      }
      df_norm(uth, utl);
    }
    const int pt = k * NXY + j * NX + i;
    DfPair h = h1c;
    if (act && a.h1mode) h = df_split_int(__ldg(a.h1 + eo + pt));
    // col3 / addcol3 order of hmholtz.f:199-206
    float t1h, t1l, t2h, t2l, t3h, t3l;
    df_mul(t1h, t1l, urh, url, g1.x, g1.y);
    df_mul(t2h, t2l, ush, usl, g2.x, g2.y);
    df_mul(t3h, t3l, uth, utl, g3.x, g3.y);
    df_mac(t1h, t1l, ush, usl, g4.x, g4.y);
    df_mac(t1h, t1l, uth, utl, g5.x, g5.y);
    df_mac(t2h, t2l, urh, url, g4.x, g4.y);
    df_mac(t2h, t2l, uth, utl, g6.x, g6.y);
    df_mac(t3h, t3l, urh, url, g5.x, g5.y);
    df_mac(t3h, t3l, ush, usl, g6.x, g6.y);
    df_norm(t1h, t1l);
    df_norm(t2h, t2l);
    df_norm(t3h, t3l);
    if (!unit_h1) {  // col2 by h1 (:207-209)
      df_mul(t1h, t1l, t1h, t1l, h.h, h.l);
      df_mul(t2h, t2l, t2h, t2l, h.h, h.l);
      df_mul(t3h, t3l, t3h, t3l, h.h, h.l);
      df_norm(t1h, t1l);
      df_norm(t2h, t2l);
      df_norm(t3h, t3l);
    }
    if (ty < epb) {
      st1[k * NX * R + j * R + i] = make_float2(t1h, t1l);
      st2[k * NX * R + j * R + i] = make_float2(t2h, t2l);
    }
    // tm3(ij,m) = sum_k tmp3(ij,k) D(k,m)
#pragma unroll
    for (int m = 0; m < NX; ++m) {
      const float2 dd = sD[k * R + m];
      if (k == 0) df_mul(rauh[m], raul[m], t3h, t3l, dd.x, dd.y);
      else df_mac(rauh[m], raul[m], t3h, t3l, dd.x, dd.y);
    }
  }
  __syncthreads();

  double dot = 0.0;  // interior w*p of this column
#pragma unroll
  for (int k = 0; k < NX; ++k) {
    const float2* s1 = st1 + k * NX * R;
    const float2* s2 = st2 + k * NX * R;
    float ah, al, bh, bl;
    {  // tm1(i,jk) = sum_l D(l,i) tmp1(l,jk)
      float2 dd = sDT[i * R], tt = s1[j * R];
      df_mul(ah, al, dd.x, dd.y, tt.x, tt.y);
#pragma unroll 2
      for (int l = 1; l < NX; ++l) {
        dd = sDT[i * R + l];
        tt = s1[j * R + l];
        df_mac(ah, al, dd.x, dd.y, tt.x, tt.y);
      }
    }
    {  // tm2(i,j,k) = sum_l tmp2(i,l,k) D(l,j)
      float2 tt = s2[i], dd = sDT[j * R];
      df_mul(bh, bl, tt.x, tt.y, dd.x, dd.y);
#pragma unroll 2
      for (int l = 1; l < NX; ++l) {
        tt = s2[l * R + i];
        dd = sDT[j * R + l];
        df_mac(bh, bl, tt.x, tt.y, dd.x, dd.y);
      }
    }
    // au = (tm1 + tm2) + tm3  (:215-217)
    df_add(ah, al, bh, bl);
    df_add(ah, al, rauh[k], raul[k]);
    double s = df_join_int(ah, al);
    const int pt = k * NXY + j * NX + i;
    if (act) {
      if (a.h2mode) {  // addcol4(au,helm2,bm1,u) (:225), in FP64
        double hb;
        if (a.hbm) {
          hb = __ldg(a.hbm + eo + pt);
        } else {
          const double hh = (a.h2mode == 1) ? a.h2s : __ldg(a.h2 + eo + pt);
          hb = hh * __ldg(a.bm1 + eo + pt);
        }
        s = fma(hb, ru64[k], s);
      }
      a.au[eo + pt] = s;
      if constexpr (FUSED) {
        if (a.allrho || (i > 0 && i < NX - 1 && j > 0 && j < NX - 1 && k > 0 && k < NX - 1 &&
                         (!a.skip || !a.skip[eo + pt])))
          dot = fma(s, ru64[k], dot);
      }
    }
  }
  if constexpr (FUSED) {
    // the element's u slab (read only before the first barrier) holds the
    // fixed-order sum's values
    element_sum<NX, double>(dot, su, tx, ty < epb, act ? a.partial + e : nullptr);
  }
}

template <int NX, bool FUSED>
__global__ void __launch_bounds__(256) axhelm_df_kernel(const DfArgs A) {
  extern __shared__ __align__(16) unsigned char smem_df[];
  if constexpr (FUSED) {
    if (A.a.cg->done) return;
  }
  axhelm_df_body<NX, FUSED>(A, blockIdx.x, threadIdx.x, threadIdx.y, blockDim.y, smem_df);
}

}  // namespace nekgpu
