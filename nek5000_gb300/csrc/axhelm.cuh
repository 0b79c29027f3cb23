// axhelm.cuh -- matrix-free Helmholtz operator, 3-D deformed elements.
//
//   au = h1 * sum_ij D_i^T (G_ij D_j u) + h2 * B u           (per element)
//
// Restates core/hmholtz.f:72-259 (3-D deformed branch :191-217, h2 term :225)
// for one element per thread-slab: an lx1 x lx1 slab of threads owns the
// element, thread (i,j) walks the z-column k = 0..lx1-1.  The element's field
// is staged once in shared memory (row-padded against bank conflicts); D and
// D^T live in shared memory and are read as warp broadcasts; the t-direction
// transposed contraction accumulates in registers, so only the r and s
// intermediates go through shared memory.  G is read once, coalesced
// (consecutive i are consecutive addresses inside G[e][m][:]).
//
// Contraction order is the reference's mxm -> mxf<n> order
// (core/mxm_std.f:139-230): sum over the inner index l = 0..lx1-1 left to
// right.  With EXACT = true every product and sum is rounded separately, in
// the reference's order, so FP64 results equal an unfused evaluation of the
// Fortran bit for bit; EXACT = false uses fused multiply-adds.
//
// FUSED = true is the PCG form (hmholtz.f:795-801 folded together): the load
// stage forms p <- r*d + beta*p (col3 + add2s1, :730, :795) and stores it,
// the operator is applied to the new p, and the element-interior part of
// rho = sum w*p*mult (glsc3 :801; interior points have mult = 1 and are not
// touched by dssum/mask) is reduced into one FP64 partial per element, in an
// order fixed by the element's own point indices, so that the number of
// elements a block holds changes the speed and never the result.
#pragma once
#include "common.cuh"

namespace nekgpu {

template <typename T>
struct AxArgs {
  T* au;           // out: w
  const T* u;      // in: field (plain) / old p (fused; may alias p)
  const T* G;      // G[e][6][P]
  const T* bm1;    // mass (read when h2mode != 0)
  const T* h1;     // h1 array (h1mode 1)
  const T* h2;     // h2 array (h2mode 2)
  T h1s, h2s;      // uniform h1 (h1mode 0) / h2 (h2mode 1)
  int h1mode, h2mode;
  const T* hbm;    // h2 * bm1 per point, formed once per solve (h2mode != 0), or null
  const T* D;      // lx1*lx1 row-major, D[i][j]
  int nel;
  // fused PCG operands
  T* p;
  const T* r;
  const T* d;
  const CgScalars* cg;
  double* partial; // one per element
  int* err;        // device flag: set if a bounded wait expired
  const unsigned char* skip;  // interior points owned by the boundary-group kernel
  // Fused form: 0 = rho partial over element-interior points (the
  // reference's glsc3 of the assembled w, its boundary part added by the
  // boundary-group kernel); 1 = over every local point of the unassembled w,
  // which equals the same rho because p is continuous and zero where masked
  // (sum_g w_g p_g = sum_i w_local_i p_i), and spares the boundary-group
  // kernel its p reads.  The FP32 inner solve uses 1.
  int allrho;
  // 1: G, d, bm1, h1, h2 are read by several launches of one iteration (the
  // fields of a multi-field solve): staged with the default L2 policy so that
  // the later reads hit L2; 0: every input is read once (evict first).
  int shared_in;
  // Fused form: the PCG vectors (r, d, p, w) store each element's points in
  // the face order of perm.cu; perm[pt] is the position of natural point pt
  // (G, bm1, h1, h2 stay natural).  nullptr: natural order.
  const int* perm;
};

// Orders the TMA-staged FP32 kernel (axhelm_tma.cuh) serves: every even
// lx1, and odd lx1 up to 9 in blocks of 4 elements.
__host__ __device__ constexpr bool tma_lx1(int nx) {
  return nx % 2 == 0 || (nx >= 3 && nx <= 9);
}

template <int NX>
struct AxShape {
  static constexpr int R = NX + 1;           // padded row
  static constexpr int LP = NX * NX * R;     // padded element slab
  static constexpr int P = NX * NX * NX;
};

// Sum of one value per thread (i,j) of an element's slab in a fixed order:
// each row j summed over i left to right in the field precision V, then the
// row sums over j in FP64 (so an FP32 kernel spends only 2 NX FP64
// operations per element).  `buf` holds element_sum_bytes<NX, V>() bytes
// owned by this element, 8-byte aligned; threads with own = false (no
// element in this block slot) take part in the barriers only.  The sum is
// stored to *out by thread 0 of the element when out is not null.
template <int NX, typename V>
__host__ __device__ constexpr int element_sum_rows_offset() {
  return ((NX * NX * (int)sizeof(V) + 7) / 8) * 8;  // bytes to the row sums
}
template <int NX, typename V>
__device__ __forceinline__ void element_sum(V v, void* buf, int tx, bool own, double* out) {
  V* vals = reinterpret_cast<V*>(buf);
  double* rows = reinterpret_cast<double*>(reinterpret_cast<unsigned char*>(buf) +
                                           element_sum_rows_offset<NX, V>());
  if (own) vals[tx] = v;
  __syncthreads();
  if (own && tx < NX) {
    V s = vals[tx * NX];
#pragma unroll
    for (int c = 1; c < NX; ++c) s += vals[tx * NX + c];
    rows[tx] = (double)s;
  }
  __syncthreads();
  if (own && tx == 0 && out) {
    double s = rows[0];
#pragma unroll
    for (int r = 1; r < NX; ++r) s += rows[r];
    *out = s;
  }
}

// D and D^T (padded rows), the even-odd blocks of both (4 (NX/2)^2 values),
// then three slabs per element.
template <int NX, typename T>
__host__ __device__ constexpr size_t axhelm_smem_bytes(int epb) {
  return (size_t)(2 * NX * (NX + 1) + 4 * (NX / 2) * (NX / 2) + epb * 3 * AxShape<NX>::LP) *
         sizeof(T);
}

// Even-odd form of a t-direction contraction v = M u with M centro-
// antisymmetric (M[n-1-i][n-1-j] = -M[i][j], true of the GLL derivative
// matrix and of its transpose), n = NX even, H = NX/2 (Solomonoff's even-odd
// decomposition): with e_l = u_l + u_{n-1-l}, o_l = u_l - u_{n-1-l},
// E_il = (M_il + M_i,n-1-l)/2 and O_il = (M_il - M_i,n-1-l)/2 (i, l < H),
// v_i = E e + O o and v_{n-1-i} = O o - E e: 6 operations per output
// instead of 8 at NX = 8.
template <int NX, typename T>
__device__ __forceinline__ void even_odd_apply(const T (&u)[NX], const T* __restrict__ sE,
                                               const T* __restrict__ sO, T (&v)[NX]) {
  constexpr int H = NX / 2;
  T ev[H], od[H];
#pragma unroll
  for (int l = 0; l < H; ++l) {
    ev[l] = u[l] + u[NX - 1 - l];
    od[l] = u[l] - u[NX - 1 - l];
  }
#pragma unroll
  for (int k = 0; k < H; ++k) {
    T ae = sE[k * H] * ev[0], bo = sO[k * H] * od[0];
#pragma unroll
    for (int l = 1; l < H; ++l) {
      ae = fma(sE[k * H + l], ev[l], ae);
      bo = fma(sO[k * H + l], od[l], bo);
    }
    v[k] = ae + bo;
    v[NX - 1 - k] = bo - ae;
  }
}

// Block body: `blk` is the element-block index, thread (tx = i + NX*j, ty)
// works on element blk*epb + ty; threads with ty >= epb take part in the
// barriers only.  `smem_raw` holds axhelm_smem_bytes<NX,T>(epb) bytes.
template <int NX, typename T, bool EXACT, bool FUSED>
__device__ __forceinline__ void axhelm_body(const AxArgs<T>& a, int blk, int tx, int ty, int epb,
                                            unsigned char* smem_raw, double* red) {
  constexpr int R = AxShape<NX>::R, LP = AxShape<NX>::LP, P = AxShape<NX>::P;
  constexpr int NXY = NX * NX;
  // even-odd t-direction contractions: the fused multiply-add FP64 form
  // (the FP64 pipe bounds it), even lx1
  constexpr bool EO = !EXACT && sizeof(T) == 8 && NX % 2 == 0;
  constexpr int H = NX / 2;
  T* sD = reinterpret_cast<T*>(smem_raw);  // sD[i*R+l]  = D[i][l]
  T* sDT = sD + NX * R;                    // sDT[i*R+l] = D[l][i]
  T* sE = sDT + NX * R;                    // even-odd blocks of D (t forward)
  T* sO = sE + H * H;
  T* sET = sO + H * H;                     // and of D^T (t transposed)
  T* sOT = sET + H * H;
  const int tyc = ty < epb ? ty : 0;
  T* su = sOT + H * H + tyc * 3 * LP;
  T* st1 = su + LP;
  T* st2 = st1 + LP;

  const int tid = tx;
  const int i = tid % NX, j = tid / NX;
  const int ft = tx + NXY * ty, nthr = NXY * epb;
  if (ty < epb)
    for (int q = ft; q < NXY; q += nthr) {
      const int r = q / NX, c = q % NX;
      const T v = a.D[q];
      sD[r * R + c] = v;
      sDT[c * R + r] = v;
    }
  if constexpr (EO) {
    if (ty < epb)
      for (int q = ft; q < H * H; q += nthr) {
        const int k = q / H, l = q % H;
        // ut_k = sum_l D[k][l] ru_l ;  rau_m = sum_k D[k][m] t3_k
        sE[q] = T(0.5) * (a.D[k * NX + l] + a.D[k * NX + NX - 1 - l]);
        sO[q] = T(0.5) * (a.D[k * NX + l] - a.D[k * NX + NX - 1 - l]);
        sET[q] = T(0.5) * (a.D[l * NX + k] + a.D[(NX - 1 - l) * NX + k]);
        sOT[q] = T(0.5) * (a.D[l * NX + k] - a.D[(NX - 1 - l) * NX + k]);
      }
  }
  const int e = blk * epb + ty;
  const bool act = ty < epb && e < a.nel;
  const size_t eo = (size_t)(act ? e : 0) * P;

  T beta = T(0), zmean = T(0);
  bool mcor = false;
  if constexpr (FUSED) {
    beta = (T)a.cg->beta;
    mcor = a.cg->mcor != 0;
    if (mcor) zmean = (T)a.cg->zmean;
  }
  const bool unit_h1 = a.h1mode == 0 && a.h1s == T(1);

  T ru[NX];
#pragma unroll
  for (int k = 0; k < NX; ++k) {
    const int pt = k * NXY + j * NX + i;
    T v = T(0);
    if (act) {
      if constexpr (FUSED) {
        const int q = a.perm ? __ldg(a.perm + pt) : pt;  // position in the vectors
        T z = EXACT ? mul_x(a.r[eo + q], a.d[eo + q]) : a.r[eo + q] * a.d[eo + q];
        if (mcor) z = EXACT ? add_x(z, zmean) : z + zmean;  // cadd(z,rmean) (hmholtz.f:749)
        v = madd<EXACT>(beta, a.u[eo + q], z);  // add2s1: p = beta*p + z
        a.p[eo + q] = v;
      } else {
        v = a.u[eo + pt];
      }
    }
    ru[k] = v;
    if (ty < epb) su[k * NX * R + j * R + i] = v;
  }
  __syncthreads();

  T rau[NX];
#pragma unroll
  for (int m = 0; m < NX; ++m) rau[m] = T(0);
  T utv[NX], t3v[NX];  // even-odd form: all ut before the planes, t3 of every plane
  if constexpr (EO) even_odd_apply<NX, T>(ru, sE, sO, utv);

  const T* __restrict__ g = a.G + (size_t)(act ? e : 0) * 6 * P;
#pragma unroll
  for (int k = 0; k < NX; ++k) {
    const T* slab = su + k * NX * R;
    // dudr(i,jk) = sum_l D(i,l) u(l,jk)      (mxm(dxm1,lx1,u,lx1,dudr,nyz))
    T ur = EXACT ? mul_x(sD[i * R], slab[j * R]) : sD[i * R] * slab[j * R];
#pragma unroll
    for (int l = 1; l < NX; ++l) ur = madd<EXACT>(sD[i * R + l], slab[j * R + l], ur);
    // duds(i,j,k) = sum_l u(i,l,k) D(j,l)     (mxm(u(1,1,iz),lx1,dytm1,ly1,duds,ly1))
    T us = EXACT ? mul_x(slab[i], sD[j * R]) : slab[i] * sD[j * R];
#pragma unroll
    for (int l = 1; l < NX; ++l) us = madd<EXACT>(slab[l * R + i], sD[j * R + l], us);
    // dudt(ij,k) = sum_l u(ij,l) D(k,l)       (mxm(u,nxy,dztm1,lz1,dudt,lz1))
    T ut;
    if constexpr (EO) {
      ut = utv[k];
    } else {
      ut = EXACT ? mul_x(ru[0], sD[k * R]) : ru[0] * sD[k * R];
#pragma unroll
      for (int l = 1; l < NX; ++l) ut = madd<EXACT>(ru[l], sD[k * R + l], ut);
    }

    const int pt = k * NXY + j * NX + i;
    T g1 = 0, g2 = 0, g3 = 0, g4 = 0, g5 = 0, g6 = 0, h = a.h1s;
    if (act) {
      g1 = __ldg(g + pt);
      g2 = __ldg(g + P + pt);
      g3 = __ldg(g + 2 * P + pt);
      g4 = __ldg(g + 3 * P + pt);
      g5 = __ldg(g + 4 * P + pt);
      g6 = __ldg(g + 5 * P + pt);
      if (a.h1mode) h = __ldg(a.h1 + eo + pt);
    }
    // col3 / addcol3 order of hmholtz.f:199-206, then col2 by h1 (:207-209)
    T t1 = EXACT ? mul_x(ur, g1) : ur * g1;
    T t2 = EXACT ? mul_x(us, g2) : us * g2;
    T t3 = EXACT ? mul_x(ut, g3) : ut * g3;
    t1 = madd<EXACT>(us, g4, t1);
    t1 = madd<EXACT>(ut, g5, t1);
    t2 = madd<EXACT>(ur, g4, t2);
    t2 = madd<EXACT>(ut, g6, t2);
    t3 = madd<EXACT>(ur, g5, t3);
    t3 = madd<EXACT>(us, g6, t3);
    if (!unit_h1) {  // h1 = 1: the products are exact, skip them
      if (EXACT) {
        t1 = mul_x(t1, h);
        t2 = mul_x(t2, h);
        t3 = mul_x(t3, h);
      } else {
        t1 *= h;
        t2 *= h;
        t3 *= h;
      }
    }
    if (ty < epb) {
      st1[k * NX * R + j * R + i] = t1;
      st2[k * NX * R + j * R + i] = t2;
    }
    // tm3(ij,m) = sum_k tmp3(ij,k) D(k,m)      (mxm(tmp3,nxy,dzm1,lz1,tm3,lz1))
    if constexpr (EO) {
      t3v[k] = t3;
    } else {
#pragma unroll
      for (int m = 0; m < NX; ++m) {
        if (k == 0) rau[m] = EXACT ? mul_x(t3, sD[m]) : t3 * sD[m];
        else rau[m] = madd<EXACT>(t3, sD[k * R + m], rau[m]);
      }
    }
  }
  if constexpr (EO) even_odd_apply<NX, T>(t3v, sET, sOT, rau);
  __syncthreads();

  T dot = T(0);  // interior w*p of this column, in field precision
#pragma unroll
  for (int k = 0; k < NX; ++k) {
    const T* s1 = st1 + k * NX * R;
    const T* s2 = st2 + k * NX * R;
    // tm1(i,jk) = sum_l D(l,i) tmp1(l,jk)     (mxm(dxtm1,lx1,tmp1,lx1,tm1,nyz))
    T tm1 = EXACT ? mul_x(sDT[i * R], s1[j * R]) : sDT[i * R] * s1[j * R];
#pragma unroll
    for (int l = 1; l < NX; ++l) tm1 = madd<EXACT>(sDT[i * R + l], s1[j * R + l], tm1);
    // tm2(i,j,k) = sum_l tmp2(i,l,k) D(l,j)   (mxm(tmp2(1,1,iz),lx1,dym1,ly1,tm2,ly1))
    T tm2 = EXACT ? mul_x(s2[i], sDT[j * R]) : s2[i] * sDT[j * R];
#pragma unroll
    for (int l = 1; l < NX; ++l) tm2 = madd<EXACT>(s2[l * R + i], sDT[j * R + l], tm2);
    // au = ((0 + tm1) + tm2) + tm3   (rzero + add2 x3, :125, :215-217)
    T s = EXACT ? add_x(add_x(tm1, tm2), rau[k]) : (tm1 + tm2) + rau[k];
    const int pt = k * NXY + j * NX + i;
    if (act) {
      if (a.h2mode) {  // addcol4(au,helm2,bm1,u): au + helm2*bm1*u  (:225)
        T hb;
        if (a.hbm) {
          hb = __ldg(a.hbm + eo + pt);  // = helm2*bm1, rounded as below
        } else {
          const T hh = (a.h2mode == 1) ? a.h2s : __ldg(a.h2 + eo + pt);
          const T bm = __ldg(a.bm1 + eo + pt);
          hb = EXACT ? mul_x(hh, bm) : hh * bm;
        }
        s = EXACT ? add_x(s, mul_x(hb, ru[k])) : fma(hb, ru[k], s);
      }
      if constexpr (FUSED && sizeof(T) == 4) {
        const int q = a.perm ? __ldg(a.perm + pt) : pt;
        st_hint(a.au + eo + q, s, l2_policy_evict_last());
      } else {
        a.au[eo + pt] = s;
      }
      if constexpr (FUSED) {
        if (a.allrho || (i > 0 && i < NX - 1 && j > 0 && j < NX - 1 && k > 0 && k < NX - 1 &&
                         (!a.skip || !a.skip[eo + pt])))
          dot = fma(s, ru[k], dot);
      }
    }
  }
  if constexpr (FUSED) {
    // The element's u slab (read only before the first barrier) holds the
    // sum's NX^2 values and NX doubles: NX^2 (NX+1) sizeof(T) is enough.
    (void)red;
    element_sum<NX, T>(dot, su, tid, ty < epb, act ? a.partial + e : nullptr);
  }
}

template <int NX, typename T, bool EXACT, bool FUSED>
__global__ void __launch_bounds__(256) axhelm_kernel(const AxArgs<T> a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  __shared__ double red[32];
  if constexpr (FUSED) {
    if (a.cg->done) return;  // uniform over the grid: nothing to do after convergence
  }
  axhelm_body<NX, T, EXACT, FUSED>(a, blockIdx.x, threadIdx.x, threadIdx.y, blockDim.y, smem_raw,
                                   red);
}

// Elements per block for a given lx1 (about 256 threads, at least one element).
__host__ __device__ constexpr int axhelm_epb(int nx) {
  return (256 / (nx * nx)) > 0 ? (256 / (nx * nx)) : 1;
}

}  // namespace nekgpu
