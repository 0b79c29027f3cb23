// pcg.cu -- Jacobi preconditioner (setprec), vector kernels and the fused
// Jacobi-PCG driver (cggo).
//
// One PCG iteration of core/hmholtz.f:726-815 runs as three kernels with all
// scalars kept on the device:
//   A  axhelm_kernel<FUSED>   p = r*d + beta*p ; w = A p ; interior rho partials
//   B  gs_cg_kernel           w = mask*dssum(w) on boundary groups ; rho, alpha
//   C  cg_update_kernel       x += alpha p ; r -= alpha w ; z = r*d ;
//                             s1 = sum z r mult ; s2 = sum r^2 mult binv ;
//                             last block: rtz1, rbn2, convergence, beta
// C's finalisation is the convergence test at the top of the next reference
// iteration (:754-793), so the iteration counts match cggo's.
#include <algorithm>
#include <cmath>

#include "cg_kernels.cuh"
#include "impl.cuh"

namespace nekgpu {

void set_error(Handle& h, const std::string& msg) { h.err = msg; }

namespace {

constexpr int kVecThreads = 256;
constexpr int NEKGPU_ENOMEM_ = -4;

inline int vec_blocks(int64_t n) {
  int64_t b = (n + kVecThreads - 1) / kVecThreads;
  return (int)std::min<int64_t>(std::max<int64_t>(b, 1), 152 * 6);
}

// ---- min/max of h1 and h2 (uniformity detection) ---------------------------
template <typename T>
__global__ void minmax_kernel(const T* __restrict__ a, int64_t n, double* out) {
  __shared__ double smn[32], smx[32];
  double mn = INFINITY, mx = -INFINITY;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double v = (double)a[i];
    mn = fmin(mn, v);
    mx = fmax(mx, v);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    mn = fmin(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    smn[wid] = mn;
    smx[wid] = mx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < (int)(blockDim.x + 31) / 32; ++q) {
      mn = fmin(mn, smn[q]);
      mx = fmax(mx, smx[q]);
    }
    out[2 * blockIdx.x] = mn;
    out[2 * blockIdx.x + 1] = mx;
  }
}

// ---- setprec: one thread per point, exact reference order ------------------
// hmholtz.f:400-486 (3-D deformed), then col2 by h1 (:504) and addcol3
// h2*bm1 (:505).  dssum and the reciprocal follow in separate kernels.
template <int NX>
__global__ void setprec_kernel(double* __restrict__ dp, const double* __restrict__ G,
                               const double* __restrict__ D, const double* __restrict__ bm1,
                               const double* __restrict__ h1, const double* __restrict__ h2,
                               double h1s, double h2s, int h1mode, int h2mode, int nel) {
  constexpr int P = NX * NX * NX;
  __shared__ double sDT[NX][NX];  // DT(i,q) = D(q,i): dxtm1(i,q)
  for (int q = threadIdx.x; q < NX * NX; q += blockDim.x) {
    const int r = q / NX, c = q % NX;
    sDT[c][r] = D[q];
  }
  __syncthreads();
  const int64_t gid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (gid >= (int64_t)nel * P) return;
  const int64_t e = gid / P;
  const int pt = (int)(gid % P);
  const int ix = pt % NX, iy = (pt / NX) % NX, iz = pt / (NX * NX);
  const double* g = G + e * 6 * P;
  const double *g1 = g, *g2 = g + P, *g3 = g + 2 * P, *g4 = g + 3 * P, *g5 = g + 4 * P,
               *g6 = g + 5 * P;
  auto I = [](int x, int y, int z) { return x + NX * (y + NX * z); };
  double v = 0.0;
  for (int q = 0; q < NX; ++q)
    v = __dadd_rn(v, __dmul_rn(g1[I(q, iy, iz)], __dmul_rn(sDT[ix][q], sDT[ix][q])));
  for (int q = 0; q < NX; ++q)
    v = __dadd_rn(v, __dmul_rn(g2[I(ix, q, iz)], __dmul_rn(sDT[iy][q], sDT[iy][q])));
  for (int q = 0; q < NX; ++q)
    v = __dadd_rn(v, __dmul_rn(g3[I(ix, iy, q)], __dmul_rn(sDT[iz][q], sDT[iz][q])));
  // Cross terms, loops 600/700/800 (:440-467): with IY,IZ (resp. IX,IZ and
  // IX,IY) ranging over {1, lx1}, they touch the 8 element corners only.
  const int L = NX - 1;
  if ((ix == 0 || ix == L) && (iy == 0 || iy == L) && (iz == 0 || iz == L)) {
    const double dx = sDT[ix][ix], dy = sDT[iy][iy], dz = sDT[iz][iz];
    v = __dadd_rn(__dadd_rn(v, __dmul_rn(__dmul_rn(g4[pt], dx), dy)),
                  __dmul_rn(__dmul_rn(g5[pt], dx), dz));  // 600
    v = __dadd_rn(__dadd_rn(v, __dmul_rn(__dmul_rn(g4[pt], dy), dx)),
                  __dmul_rn(__dmul_rn(g6[pt], dy), dz));  // 700
    v = __dadd_rn(__dadd_rn(v, __dmul_rn(__dmul_rn(g5[pt], dz), dx)),
                  __dmul_rn(__dmul_rn(g6[pt], dz), dy));  // 800
  }
  const double hv = h1mode ? h1[gid] : h1s;
  v = __dmul_rn(v, hv);
  if (h2mode) {
    const double h2v = (h2mode == 1) ? h2s : h2[gid];
    v = __dadd_rn(v, __dmul_rn(h2v, bm1[gid]));
  }
  dp[gid] = v;
}

__global__ void invert_kernel(double* __restrict__ a, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    a[i] = 1.0 / a[i];
}

template <typename TO, typename TI>
__global__ void cast_kernel(TO* __restrict__ o, const TI* __restrict__ a, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    o[i] = (TO)a[i];
}

// ---- generic FP64 reductions for setup-time scalars --------------------------
// kind 0: sum a            1: sum (a*b)*c        2: sum (a*a)*b
//      3: max |a|          4: sum ((a*b)*b)*c    5: sum a*b        6: min a
__global__ void sum_kernel(int kind, const double* __restrict__ a, const double* __restrict__ b,
                           const double* __restrict__ c, int64_t n, double* out) {
  __shared__ double red[32];
  const bool ismax = (kind == 3), ismin = (kind == 6);
  double acc = ismin ? INFINITY : 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    switch (kind) {
      case 0: acc += a[i]; break;
      case 1: acc += __dmul_rn(__dmul_rn(a[i], b[i]), c[i]); break;
      case 2: acc += __dmul_rn(__dmul_rn(a[i], a[i]), b[i]); break;
      case 3: acc = fmax(acc, fabs(a[i])); break;
      case 4: acc += __dmul_rn(__dmul_rn(__dmul_rn(a[i], b[i]), b[i]), c[i]); break;
      case 5: acc += __dmul_rn(a[i], b[i]); break;
      default: acc = fmin(acc, a[i]); break;
    }
  }
  if (ismax || ismin) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double v = __shfl_xor_sync(0xffffffffu, acc, o);
      acc = ismax ? fmax(acc, v) : fmin(acc, v);
    }
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
      for (int q = 1; q < (int)(blockDim.x + 31) / 32; ++q)
        acc = ismax ? fmax(acc, red[q]) : fmin(acc, red[q]);
      out[blockIdx.x] = acc;
    }
    return;
  }
  acc = block_sum(acc, red);
  if (threadIdx.x == 0) out[blockIdx.x] = acc;
}

// ---- PCG update / convergence kernel ---------------------------------------
// Element-interior points handled by the fused operator must carry mask 1 and
// multiplicity 1 (the reference's masks live on faces; interiors are unshared).
template <typename T>
__global__ void interior_check_kernel(const T* __restrict__ mask, const T* __restrict__ mult,
                                      const unsigned char* __restrict__ skip, int nx1, int64_t n,
                                      int* bad, bool face_order = false) {
  const int P = nx1 * nx1 * nx1, m = nx1 - 2;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int p = (int)(i % P), x = p % nx1, y = (p / nx1) % nx1, z = p / (nx1 * nx1);
    // face order (perm.cu): the element's interior points come last
    const bool in = face_order ? (m > 0 && p >= P - m * m * m)
                               : (x > 0 && x < nx1 - 1 && y > 0 && y < nx1 - 1 && z > 0 &&
                                  z < nx1 - 1);
    if (in && !(skip && skip[i]) && (mask[i] != T(1) || mult[i] != T(1))) atomicOr(bad, 1);
  }
}

// add2s2 (math.f:689): a = a + c b, rounded as the reference
__global__ void axpy_exact_kernel(double* __restrict__ a, const double* __restrict__ b, double c,
                                  int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    a[i] = __dadd_rn(a[i], __dmul_rn(c, b[i]));
}

template <typename T>
__global__ void zero_kernel(T* __restrict__ a, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    a[i] = T(0);
}

}  // namespace

// ---- host helpers ------------------------------------------------------------
int pcg_vec_blocks(int64_t n) { return vec_blocks(n); }

void launch_interior_check(Handle& h, const float* mask, const float* mult, int* bad) {
  count_launch();
  interior_check_kernel<float><<<vec_blocks(h.mesh.n), kVecThreads, 0, h.stream>>>(
      mask, mult, h.mesh.gs.skip, h.mesh.nx1, h.mesh.n, bad);
}

template <typename T>
int detect_coef(Handle& h, const T* h1, const T* h2, int64_t n, Coef<T>& c) {
  const int nb = vec_blocks(n);
  if (h.red.ensure(4 * (size_t)nb) != cudaSuccess) return NEKGPU_ENOMEM_;
  count_launch();
  minmax_kernel<T><<<nb, kVecThreads, 0, h.stream>>>(h1, n, h.red.ptr);
  count_launch();
  minmax_kernel<T><<<nb, kVecThreads, 0, h.stream>>>(h2, n, h.red.ptr + 2 * nb);
  std::vector<double> hm(4 * (size_t)nb);
  if (cudaMemcpyAsync(hm.data(), h.red.ptr, hm.size() * sizeof(double), cudaMemcpyDeviceToHost,
                      h.stream) != cudaSuccess ||
      cudaStreamSynchronize(h.stream) != cudaSuccess)
    return -3;
  double mn1 = INFINITY, mx1 = -INFINITY, mn2 = INFINITY, mx2 = -INFINITY;
  for (int b = 0; b < nb; ++b) {
    mn1 = std::min(mn1, hm[2 * b]);
    mx1 = std::max(mx1, hm[2 * b + 1]);
    mn2 = std::min(mn2, hm[2 * nb + 2 * b]);
    mx2 = std::max(mx2, hm[2 * nb + 2 * b + 1]);
  }
  c.h1 = h1;
  c.h2 = h2;
  if (mn1 == mx1) {
    c.h1mode = 0;
    c.h1s = (T)mn1;
  } else {
    c.h1mode = 1;
  }
  // ifh2 = vlamax(h2) > 0 (hmholtz.f:302-304)
  if (std::max(std::fabs(mn2), std::fabs(mx2)) == 0.0) {
    c.h2mode = 0;
    c.h2s = T(0);
  } else if (mn2 == mx2) {
    c.h2mode = 1;
    c.h2s = (T)mn2;
  } else {
    c.h2mode = 2;
  }
  return 0;
}
template int detect_coef<double>(Handle&, const double*, const double*, int64_t, Coef<double>&);
template int detect_coef<float>(Handle&, const float*, const float*, int64_t, Coef<float>&);

double device_sum(Handle& h, int kind, const double* a, const double* b, const double* c,
                  int64_t n, int* status) {
  const int nb = vec_blocks(n);
  *status = 0;
  if (h.red.ensure((size_t)nb) != cudaSuccess) {
    *status = -4;
    return 0.0;
  }
  count_launch();
  sum_kernel<<<nb, kVecThreads, 0, h.stream>>>(kind, a, b, c, n, h.red.ptr);
  std::vector<double> hp((size_t)nb);
  if (cudaMemcpyAsync(hp.data(), h.red.ptr, nb * sizeof(double), cudaMemcpyDeviceToHost,
                      h.stream) != cudaSuccess ||
      cudaStreamSynchronize(h.stream) != cudaSuccess) {
    *status = -3;
    return 0.0;
  }
  double s = (kind == 6) ? INFINITY : 0.0;
  for (int q = 0; q < nb; ++q)
    s = (kind == 3) ? std::max(s, hp[q]) : (kind == 6) ? std::min(s, hp[q]) : s + hp[q];
  return s;
}

template <int NX>
static void launch_setprec_nx(Handle& h, double* d, const Coef<double>& c) {
  const Mesh& m = h.mesh;
  const int64_t n = m.n;
  const int nb = (int)((n + 255) / 256);
  count_launch();
  setprec_kernel<NX><<<nb, 256, 0, h.stream>>>(d, m.f64.G, m.f64.D, m.f64.bm1, c.h1, c.h2, c.h1s,
                                              c.h2s, c.h1mode, c.h2mode, m.nel);
}

// d = 1/dssum(diag)  (setprec, hmholtz.f:380-524), FP64
// The element-local diagonal alone (before dssum and the reciprocal): what a
// sharded solve sums across its shards' interfaces first.
int setprec_local_f64(Handle& h, double* d, const Coef<double>& c) {
  cudaError_t pre = cudaGetLastError();
  if (pre != cudaSuccess) {
    set_error(h, std::string("setprec: error pending from an earlier call: ") +
                     cudaGetErrorString(pre));
    return -3;
  }
  switch (h.mesh.nx1) {
    case 2: launch_setprec_nx<2>(h, d, c); break;
    case 3: launch_setprec_nx<3>(h, d, c); break;
    case 4: launch_setprec_nx<4>(h, d, c); break;
    case 5: launch_setprec_nx<5>(h, d, c); break;
    case 6: launch_setprec_nx<6>(h, d, c); break;
    case 7: launch_setprec_nx<7>(h, d, c); break;
    case 8: launch_setprec_nx<8>(h, d, c); break;
    case 9: launch_setprec_nx<9>(h, d, c); break;
    case 10: launch_setprec_nx<10>(h, d, c); break;
    case 11: launch_setprec_nx<11>(h, d, c); break;
    case 12: launch_setprec_nx<12>(h, d, c); break;
    default: return -1;
  }
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(h, std::string("setprec kernel: ") + cudaGetErrorString(e));
    return -3;
  }
  return 0;
}

int setprec_f64(Handle& h, double* d, const Coef<double>& c) {
  cudaError_t pre = cudaGetLastError();
  if (pre != cudaSuccess) {
    set_error(h, std::string("setprec: error pending from an earlier call: ") +
                     cudaGetErrorString(pre));
    return -3;
  }
  switch (h.mesh.nx1) {
    case 2: launch_setprec_nx<2>(h, d, c); break;
    case 3: launch_setprec_nx<3>(h, d, c); break;
    case 4: launch_setprec_nx<4>(h, d, c); break;
    case 5: launch_setprec_nx<5>(h, d, c); break;
    case 6: launch_setprec_nx<6>(h, d, c); break;
    case 7: launch_setprec_nx<7>(h, d, c); break;
    case 8: launch_setprec_nx<8>(h, d, c); break;
    case 9: launch_setprec_nx<9>(h, d, c); break;
    case 10: launch_setprec_nx<10>(h, d, c); break;
    case 11: launch_setprec_nx<11>(h, d, c); break;
    case 12: launch_setprec_nx<12>(h, d, c); break;
    default: return -1;
  }
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(h, std::string("setprec kernel: ") + cudaGetErrorString(e));
    return -3;
  }
  gs_op<double>(h.mesh.gs, d, 0, h.stream);
  if ((e = cudaGetLastError()) != cudaSuccess) {
    set_error(h, std::string("setprec dssum: ") + cudaGetErrorString(e));
    return -3;
  }
  count_launch();
  invert_kernel<<<vec_blocks(h.mesh.n), kVecThreads, 0, h.stream>>>(d, h.mesh.n);
  if ((e = cudaGetLastError()) != cudaSuccess) {
    set_error(h, std::string("setprec invert: ") + cudaGetErrorString(e));
    return -3;
  }
  return 0;
}

// ---- PCG driver ------------------------------------------------------------
template <typename T>
static cudaError_t launch_A(Handle& h, const OpData<T>& op, PcgWork<T>& wk, const Coef<T>& c,
                            bool exact, int* nA) {
  if constexpr (std::is_same<T, double>::value) {
    if (exact)
      return launch_axhelm_cg<double, true>(h.mesh, op, wk.w.ptr, wk.p.ptr, wk.r.ptr, wk.d.ptr, c,
                                            h.cg, h.partialA.ptr, nA, h.stream);
    return launch_axhelm_cg<double, false>(h.mesh, op, wk.w.ptr, wk.p.ptr, wk.r.ptr, wk.d.ptr, c,
                                           h.cg, h.partialA.ptr, nA, h.stream);
  } else {
    (void)exact;
    return launch_axhelm_cg<float, false>(h.mesh, op, wk.w.ptr, wk.p.ptr, wk.r.ptr, wk.d.ptr, c,
                                          h.cg, h.partialA.ptr, nA, h.stream);
  }
}

// The fused multiply-add form reads the folded weights wk.md = mult d and
// wk.mb = mult binv (pcg_prepare); the exact form the reference's arrays.
template <typename T>
static void launch_C(Handle& h, PcgWork<T>& wk, T* x, const T* mult, const T* binv, bool exact,
                     bool first) {
  const int64_t n = h.mesh.n;
  const int nb = vec_blocks(n);
  if constexpr (std::is_same<T, double>::value) {
    if (h.mcor) {  // null-space correction: the reference's z, unfolded
      auto k = exact ? (first ? cg_update_mcor_kernel<double, true, true>
                              : cg_update_mcor_kernel<double, true, false>)
                     : (first ? cg_update_mcor_kernel<double, false, true>
                              : cg_update_mcor_kernel<double, false, false>);
      count_launch();
      k<<<nb, kVecThreads, 0, h.stream>>>(x, wk.r.ptr, wk.p.ptr, wk.w.ptr, wk.d.ptr, mult, binv,
                                          h.mesh.f64.bm1, n, h.cg, h.partialC.ptr);
      return;
    }
  }
  auto al = [](const void* q) { return ((uintptr_t)q & 15u) == 0; };
  const T* dd = exact ? wk.d.ptr : wk.md.ptr;
  const T* bb = exact ? binv : wk.mb.ptr;
  const bool vec = al(x) && al(wk.r.ptr) && al(wk.p.ptr) && al(wk.w.ptr) && al(dd) &&
                   al(mult) && al(bb);
  auto kern = vec ? (exact ? (first ? cg_update_kernel<T, true, true, true, false>
                                    : cg_update_kernel<T, true, false, true, false>)
                           : (first ? cg_update_kernel<T, false, true, true, true>
                                    : cg_update_kernel<T, false, false, true, true>))
                  : (exact ? (first ? cg_update_kernel<T, true, true, false, false>
                                    : cg_update_kernel<T, true, false, false, false>)
                           : (first ? cg_update_kernel<T, false, true, false, true>
                                    : cg_update_kernel<T, false, false, false, true>));
  count_launch();
  kern<<<nb, kVecThreads, 0, h.stream>>>(x, wk.r.ptr, wk.p.ptr, wk.w.ptr, dd, mult, bb, n, h.cg,
                                         h.partialC.ptr);
}

template <typename T, bool EXACT>
__global__ void hbm_kernel(T* __restrict__ hbm, const T* __restrict__ h2, T h2s, int h2mode,
                           const T* __restrict__ bm1, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const T hh = h2mode == 1 ? h2s : h2[i];
    hbm[i] = EXACT ? mul_x(hh, bm1[i]) : hh * bm1[i];
  }
}

template <typename T>
__global__ void fold_weights_kernel(T* __restrict__ md, T* __restrict__ mb,
                                    const T* __restrict__ d, const T* __restrict__ mult,
                                    const T* __restrict__ binv, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    md[i] = mult[i] * d[i];
    mb[i] = mult[i] * binv[i];
  }
}

template <typename T>
double device_absmax(Handle& h, const T* a, int64_t n, int* status) {
  const int nb = vec_blocks(n);
  *status = 0;
  if (h.red.ensure(2 * (size_t)nb) != cudaSuccess) {
    *status = -4;
    return 0.0;
  }
  count_launch();
  minmax_kernel<T><<<nb, kVecThreads, 0, h.stream>>>(a, n, h.red.ptr);
  std::vector<double> hm(2 * (size_t)nb);
  if (cudaMemcpyAsync(hm.data(), h.red.ptr, hm.size() * sizeof(double), cudaMemcpyDeviceToHost,
                      h.stream) != cudaSuccess ||
      cudaStreamSynchronize(h.stream) != cudaSuccess) {
    *status = -3;
    return 0.0;
  }
  double m = 0.0;
  for (int b = 0; b < nb; ++b) m = std::max(m, std::max(std::fabs(hm[2 * b]), std::fabs(hm[2 * b + 1])));
  return m;
}
template double device_absmax<double>(Handle&, const double*, int64_t, int*);
template double device_absmax<float>(Handle&, const float*, int64_t, int*);

// Everything of one solve before its first iteration (hmholtz.f:683-701 and
// the iteration-1 state): buffers, max|f| (an all-zero rhs returns x = 0,
// res.niter = 0 and *trivial = true), Jacobi diagonal, boundary-group
// weights and checks, r = f, p = 0, scalars.  The iteration-1 check kernel
// is not launched.
template <typename T>
PcgResult pcg_prepare(Handle& h, PcgWork<T>& wk, T* x, const T* f, const Coef<T>& c,
                      const T* mask, const T* mult, double tin, int maxiter, int istep,
                      const T* dpre, bool* trivial) {
  PcgResult res;
  *trivial = false;
  Mesh& m = h.mesh;
  const int64_t n = m.n;
  cudaStream_t s = h.stream;
  const int nA = axhelm_blocks(m.nx1, m.nel);
  // the FP32 solve in the face-ordered layout uses that layout's maps
  const GsMaps& gs = (sizeof(T) == 4 && h.gs32) ? *h.gs32 : m.gs;
  const int nB = std::max(
      std::max(gs_cg_blocks(gs), gs_cg_blocks(gs.cls_tuned[sizeof(T) == 4 ? 1 : 0])), 1);
  const int nC = vec_blocks(n);
  if (wk.r.ensure(n) || wk.w.ensure(n) || wk.p.ensure(n) || wk.d.ensure(n) ||
      wk.segmask.ensure(gs.nbseg) || wk.segmsum.ensure(gs.nbseg) ||
      h.partialA.ensure(nA) || h.partialB.ensure(nB) || h.partialC.ensure(4 * (size_t)nC)) {
    res.status = -4;
    set_error(h, "pcg: device allocation failed");
    return res;
  }
  // launch shape of the fused operator (first solve of this mesh; r, p, w are
  // scratch until they are set below)
  {
    const OpData<T>* op;
    if constexpr (std::is_same<T, double>::value) op = &m.f64;
    else op = &m.f32;
    const int st = tune_operator<T>(h, *op, wk, c);
    if (st) {
      res.status = st;
      return res;
    }
  }
  // fmax = glamax(f): an all-zero rhs returns x = 0 at once (hmholtz.f:699-701)
  if (cuda_pending(h, "pcg: before the solve")) {
    res.status = -3;
    return res;
  }
  int st = 0;
  const double fmax = device_absmax<T>(h, f, n, &st);
  if (cuda_pending(h, "pcg: max|f|")) {
    res.status = -3;
    return res;
  }
  if (st) {
    res.status = st;
    set_error(h, "pcg: reduction failed");
    return res;
  }
  count_launch();
  zero_kernel<T><<<vec_blocks(n), kVecThreads, 0, s>>>(x, n);
  if (cuda_pending(h, "pcg: zero x")) {
    res.status = -3;
    return res;
  }
  if (fmax == 0.0) {
    *trivial = true;
    return res;
  }

  // Jacobi diagonal: given by the caller (FP32 inner solves get the FP64
  // diagonal cast once), or setprec in FP64 here.
  if (dpre) {
    if (dpre != wk.d.ptr)
      cudaMemcpyAsync(wk.d.ptr, dpre, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
  } else if constexpr (std::is_same<T, double>::value) {
    st = setprec_f64(h, wk.d.ptr, c);
  } else {
    st = -1;
  }
  if (st) {
    res.status = st;
    if (h.err.empty()) set_error(h, "pcg: setprec failed");
    return res;
  }
  // boundary-group mask / multiplicity weights
  cudaMemsetAsync(h.flag, 0, 2 * sizeof(int), s);
  gs_cg_weights<T>(gs, mask, mult, wk.segmask.ptr, wk.segmsum.ptr, h.flag, s);
  count_launch();
  interior_check_kernel<T><<<vec_blocks(n), kVecThreads, 0, s>>>(mask, mult, gs.skip, m.nx1, n,
                                                                 h.flag + 1, &gs != &m.gs);
  int flags[2] = {0, 0};
  cudaMemcpyAsync(flags, h.flag, 2 * sizeof(int), cudaMemcpyDeviceToHost, s);
  // r = f, p = 0
  cudaMemcpyAsync(wk.r.ptr, f, n * sizeof(T), cudaMemcpyDeviceToDevice, s);
  count_launch();
  zero_kernel<T><<<vec_blocks(n), kVecThreads, 0, s>>>(wk.p.ptr, n);
  // non-trivial null space (no Dirichlet point, h2 = 0; hmholtz.f:703-720):
  // r += rmean dssum(bm1), rmean = smean sum r mult, smean = -1 / sum bm1
  h.mcor = false;
  double smean = 0.0;
  if constexpr (std::is_same<T, double>::value) {
    if (c.h2mode == 0) {
      const double skmin = device_sum(h, 6, mask, nullptr, nullptr, n, &st);  // glmin(mask)
      if (!st && skmin > 0.0) {
        h.mcor = true;
        smean = -1.0 / device_sum(h, 0, m.f64.bm1, nullptr, nullptr, n, &st);
        const double rmean = smean * device_sum(h, 5, wk.r.ptr, mult, nullptr, n, &st);
        cudaMemcpyAsync(wk.w.ptr, m.f64.bm1, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
        gs_op<double>(m.gs, wk.w.ptr, 0, s);
        count_launch();
        axpy_exact_kernel<<<vec_blocks(n), kVecThreads, 0, s>>>(wk.r.ptr, wk.w.ptr, rmean, n);
      }
      if (st) {
        res.status = st;
        set_error(h, "pcg: reduction failed");
        return res;
      }
    }
  }
  CgScalars& hc = *h.cg_host;
  memset(&hc, 0, sizeof(CgScalars));
  hc.mcor = h.mcor ? 1 : 0;
  hc.smean = smean;
  hc.rtz1 = 1.0;
  hc.tin = tin;
  hc.tol = std::fabs(tin);
  hc.vol = m.vol;
  hc.maxiter = maxiter;
  hc.istep = istep;
  if (maxiter < 1) {
    hc.done = 1;
    hc.niter = 0;
  }
  cudaMemcpyAsync(h.cg, &hc, sizeof(CgScalars), cudaMemcpyHostToDevice, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) {
    res.status = -3;
    set_error(h, std::string("pcg: ") + cudaGetErrorString(cudaGetLastError()));
    return res;
  }
  if (flags[0]) {
    res.status = -1;
    set_error(h, "pcg: mask differs between copies of a shared node (apply dsop '*' first)");
    return res;
  }
  if (flags[1]) {
    res.status = -1;
    set_error(h, "pcg: an element-interior point has mask or multiplicity other than 1");
    return res;
  }
  return res;
}
template PcgResult pcg_prepare<double>(Handle&, PcgWork<double>&, double*, const double*,
                                       const Coef<double>&, const double*, const double*, double,
                                       int, int, const double*, bool*);
template PcgResult pcg_prepare<float>(Handle&, PcgWork<float>&, float*, const float*,
                                      const Coef<float>&, const float*, const float*, double, int,
                                      int, const float*, bool*);

template <typename T>
PcgResult pcg_iterate(Handle& h, const OpData<T>& op, PcgWork<T>& wk, T* x, const Coef<T>& c,
                      const T* mult, const T* binv, bool exact);

// Folded update weights of a prepared solve (fused multiply-add form).
template <typename T>
static int prepare_weights(Handle& h, PcgWork<T>& wk, const T* mult, const T* binv, bool exact) {
  if (exact) return 0;
  const int64_t n = h.mesh.n;
  if (wk.md.ensure(n) || wk.mb.ensure(n)) {
    set_error(h, "pcg: device allocation failed");
    return -4;
  }
  count_launch();
  fold_weights_kernel<T><<<vec_blocks(n), kVecThreads, 0, h.stream>>>(wk.md.ptr, wk.mb.ptr,
                                                                      wk.d.ptr, mult, binv, n);
  return 0;
}

template <typename T>
int pcg_solve_extras(Handle& h, const OpData<T>& op, PcgWork<T>& wk, const T* mult, const T* binv,
                     Coef<T>& c, bool exact) {
  int st = prepare_weights<T>(h, wk, mult, binv, exact);
  if (st) return st;
  // FP64: h2 * bm1 once per solve, for the operator's mass term (the same
  // rounded product the operator would form per point and iteration)
  if constexpr (std::is_same<T, double>::value) {
    if (c.h2mode) {
      const int64_t n = h.mesh.n;
      if (wk.hbm.ensure(n)) {
        set_error(h, "pcg: device allocation failed");
        return -4;
      }
      count_launch();
      if (exact)
        hbm_kernel<T, true><<<vec_blocks(n), kVecThreads, 0, h.stream>>>(
            wk.hbm.ptr, c.h2, c.h2s, c.h2mode, op.bm1, n);
      else
        hbm_kernel<T, false><<<vec_blocks(n), kVecThreads, 0, h.stream>>>(
            wk.hbm.ptr, c.h2, c.h2s, c.h2mode, op.bm1, n);
      c.hbm = wk.hbm.ptr;
    }
  }
  return 0;
}
template int pcg_solve_extras<double>(Handle&, const OpData<double>&, PcgWork<double>&,
                                      const double*, const double*, Coef<double>&, bool);
template int pcg_solve_extras<float>(Handle&, const OpData<float>&, PcgWork<float>&,
                                     const float*, const float*, Coef<float>&, bool);

template <typename T>
int pcg_first_check(Handle& h, PcgWork<T>& wk, T* x, const T* mult, const T* binv, bool exact) {
  const int st = prepare_weights<T>(h, wk, mult, binv, exact);
  if (st) return st;
  launch_C<T>(h, wk, x, mult, binv, exact, true);
  return 0;
}
template int pcg_first_check<double>(Handle&, PcgWork<double>&, double*, const double*,
                                      const double*, bool);
template int pcg_first_check<float>(Handle&, PcgWork<float>&, float*, const float*, const float*,
                                     bool);

template <typename T>
PcgResult pcg_solve(Handle& h, const OpData<T>& op, PcgWork<T>& wk, T* x, const T* f,
                    const Coef<T>& c, const T* mask, const T* mult, const T* binv, double tin,
                    int maxiter, int istep, bool exact, const T* dpre) {
  bool trivial = false;
  PcgResult res = pcg_prepare<T>(h, wk, x, f, c, mask, mult, tin, maxiter, istep, dpre, &trivial);
  if (res.status || trivial) return res;
  Coef<T> cc = c;
  if ((res.status = pcg_solve_extras<T>(h, op, wk, mult, binv, cc, exact))) return res;
  // iteration 1 check (z, s1, s2) -- no update
  launch_C<T>(h, wk, x, mult, binv, exact, true);
  return pcg_iterate<T>(h, op, wk, x, cc, mult, binv, exact);
}

// Iterations of a prepared solve (after its iteration-1 check) until the
// device flags it done; then the reference's outputs.
template <typename T>
PcgResult pcg_iterate(Handle& h, const OpData<T>& op, PcgWork<T>& wk, T* x, const Coef<T>& c,
                      const T* mult, const T* binv, bool exact) {
  PcgResult res;
  Mesh& m = h.mesh;
  cudaStream_t s = h.stream;
  const T* f = wk.r.ptr;  // graph key only
  const T* mask = wk.segmask.ptr;
  const GsMaps& gsm = (sizeof(T) == 4 && h.gs32) ? *h.gs32 : m.gs;
  // main loop: chunks of iterations, one host check per chunk.  With kernel
  // timing on, every fused-axhelm launch is bracketed by events; after the
  // chunk's check, the first (iterations completed in the chunk) of them are
  // the live launches and are summed (later ones found the solve converged
  // and returned at once).
  const int chunk = std::max(1, h.graph_chunk);
  // four events per iteration: before the operator, after it, after the
  // boundary-group kernel, after the update
  if (h.timing && h.ax_ev.size() < 4 * (size_t)chunk) {
    for (cudaEvent_t e : h.ax_ev) cudaEventDestroy(e);
    h.ax_ev.assign(4 * (size_t)chunk, nullptr);
    for (auto& e : h.ax_ev) cudaEventCreate(&e);
  }
  // One chunk = `chunk` iterations of the three kernels.  With graphs on, the
  // chunk is captured once per argument set and replayed.
  auto enqueue_chunk = [&](int k) -> cudaError_t {
    for (int q = 0; q < k; ++q) {
      int nAb = 0;
      if (h.timing) cudaEventRecord(h.ax_ev[4 * q], s);
      cudaError_t e = launch_A<T>(h, op, wk, c, exact, &nAb);
      if (h.timing) cudaEventRecord(h.ax_ev[4 * q + 1], s);
      if (e != cudaSuccess) return e;
      // FP32: rho came whole from the operator (AxArgs::allrho)
      gs_cg<T>(gsm, wk.w.ptr, wk.p.ptr, wk.segmask.ptr, wk.segmsum.ptr, h.cg, h.partialA.ptr,
               nAb, h.partialB.ptr, s, sizeof(T) != 4, &gsm.cls_tuned[sizeof(T) == 4 ? 1 : 0]);
      if (h.timing) cudaEventRecord(h.ax_ev[4 * q + 2], s);
      launch_C<T>(h, wk, x, mult, binv, exact, false);
      if (h.timing) cudaEventRecord(h.ax_ev[4 * q + 3], s);
    }
    return cudaGetLastError();
  };
  // Events recorded by a graph's nodes cannot be paired for elapsed time, so
  // per-kernel timing runs the same kernels as direct launches.
  bool graph = h.use_graph && !h.timing;
  if (graph) {
    Handle::GraphKey key;
    const void* ptrs[15] = {x,        f,        mask,      mult,           binv, wk.r.ptr,
                            wk.w.ptr, wk.p.ptr, wk.d.ptr,  wk.md.ptr,      c.h1, c.h2,
                            wk.mb.ptr, c.perm ? (const void*)gsm.bidx : (const void*)c.hbm,
                            wk.segmask.ptr};
    for (int i = 0; i < 15; ++i) key.ptr[i] = ptrs[i];
    key.ints[0] = (int)sizeof(T);
    key.ints[1] = c.h1mode;
    key.ints[2] = c.h2mode + 8 * (int)h.mcor;
    const AxShapeSel& sh = m.ax_sel[sizeof(T) == 4 ? 1 : 0];
    const GsClasses& gc = gsm.cls_tuned[sizeof(T) == 4 ? 1 : 0];
    key.ints[3] = (int)exact + 4 * (int)m.use_tma + 8 * (sh.kind + 1) + 32 * sh.epb +
                  4096 * (gc.threads / 32) + 65536 * (m.gs_gshift[sizeof(T) == 4 ? 1 : 0] + 4);
    key.ints[4] = chunk;
    key.ints[5] = m.nel;
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
        graph = false;  // fall back to direct launches (same kernels)
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
      set_error(h, std::string("pcg: ") + cudaGetErrorString(cudaGetLastError()));
      return res;
    }
    if (h.timing && launched) {
      const int live = std::min(launched, h.cg_host->iter - iter_before);
      auto span = [&](int a, int b) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, h.ax_ev[a], h.ax_ev[b]) != cudaSuccess) {
          cudaGetLastError();
          ms = 0.f;
        }
        return (double)ms;
      };
      for (int q = 0; q < live; ++q) {
        h.ms_axhelm += span(4 * q, 4 * q + 1);
        h.ms_gs += span(4 * q + 1, 4 * q + 2);
        h.ms_update += span(4 * q + 2, 4 * q + 3);
      }
      h.n_axhelm += live;
    }
    if (h.cg_host->done) break;
    iter_before = h.cg_host->iter;
    cudaError_t e;
    int k;
    if (graph) {
      k = chunk;
      count_launch(3LL * chunk);
      e = cudaGraphLaunch(h.gexec, s);
    } else {
      const int left = h.cg_host->maxiter - h.cg_host->iter + 1;
      k = std::min(chunk, std::max(left, 1));
      e = enqueue_chunk(k);
    }
    if (e != cudaSuccess) {
      res.status = -3;
      set_error(h, std::string("pcg iteration launch: ") + cudaGetErrorString(e));
      return res;
    }
    launched = k;
  }
  const CgScalars& fin = *h.cg_host;
  res.niter = fin.niter;
  res.rbn0 = fin.rbn0;
  res.rbn2 = fin.rbn2;
  if (fin.nonfinite) {
    res.status = -7;
    set_error(h, "pcg: non-finite residual norm");
  } else if (!(fin.rbn2 <= fin.tol) && fin.iter > fin.maxiter) {
    res.status = -5;
    set_error(h, "pcg: iteration cap reached without convergence");
  }
  return res;
}

template PcgResult pcg_iterate<double>(Handle&, const OpData<double>&, PcgWork<double>&,
                                       double*, const Coef<double>&, const double*, const double*,
                                       bool);
template PcgResult pcg_iterate<float>(Handle&, const OpData<float>&, PcgWork<float>&, float*,
                                      const Coef<float>&, const float*, const float*, bool);
template PcgResult pcg_solve<double>(Handle&, const OpData<double>&, PcgWork<double>&, double*,
                                     const double*, const Coef<double>&, const double*,
                                     const double*, const double*, double, int, int, bool,
                                     const double*);
template PcgResult pcg_solve<float>(Handle&, const OpData<float>&, PcgWork<float>&, float*,
                                    const float*, const Coef<float>&, const float*, const float*,
                                    const float*, double, int, int, bool, const float*);

}  // namespace nekgpu
