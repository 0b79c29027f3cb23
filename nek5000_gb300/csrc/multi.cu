// multi.cu -- the mixed-precision solve of several fields of one mesh that
// share h1 and h2: the velocity components of a time step, which the
// reference solves one after another (ophinv, core/induct.f:1064-1071, one
// hmholtz per component with the same h1/h2 and per-component masks).
//
// Each field keeps its own FP32 PCG (its own scalars, iteration count,
// convergence test, residual replacements, mask), but one iteration of all of
// them is three kernels:
//
//  * one operator launch for every live field: block b runs the single-field
//    TMA kernel body on field b % nc of element b / nc, so the blocks of an
//    element's fields run side by side and its geometric factors, Jacobi
//    diagonal and mass -- more than half of an FP32 operator's traffic --
//    come from DRAM once and from L2 for the other fields;
//  * the boundary-group kernel loads each group's indices once and gathers,
//    masks and scatters every live field's w;
//  * the update kernel reads the folded weights once for all fields.
//
// The per-point arithmetic of each field is the single-field solve's
// (axhelm_tma.cuh, gs_kernels.cuh, cg_kernels.cuh, mixed.cu): rho from the
// unassembled operator output, per-element partials, residual replacement.
// A field that has converged is skipped by every kernel.  TMA staging needs
// an even lx1 and 16-byte aligned arrays; otherwise the fields are solved one
// after another by mixed_solve.
#include <cmath>
#include <cstring>

#include "axhelm_tma.cuh"
#include "cg_kernels.cuh"
#include "gs_kernels.cuh"
#include "impl.cuh"
#include "nekgpu.h"

namespace nekgpu {

constexpr int kMaxFields = NEKGPU_MULTI_MAX;

namespace {

constexpr int kThreads = 256;
constexpr int kBlocks = 152 * 6;

inline int vblocks(int64_t n) {
  return (int)std::min<int64_t>(std::max<int64_t>((n + kThreads - 1) / kThreads, 1), kBlocks);
}

// The operator of every live field, one launch: block b applies the
// single-field TMA kernel body (axhelm_tma.cuh, one element per block) to
// field b % nc of element b / nc.  The blocks of one element's fields run
// side by side, so the element's G, d, bm1 (and per-point h1, h2), staged
// with the default L2 policy, come from DRAM once and from L2 for the other
// fields; each field's arithmetic is exactly the single-field solve's.
struct MultiTmaArgs {
  AxArgs<float> base;  // shared operands and modes; per-field pointers below
  float* p[kMaxFields];
  const float* r[kMaxFields];
  float* w[kMaxFields];
  const CgScalars* cg[kMaxFields];
  double* partial[kMaxFields];
  int nc;
};

template <int NX>
__global__ void __launch_bounds__(NX* NX) multi_op_kernel(const MultiTmaArgs m) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int f = blockIdx.x % m.nc, e = blockIdx.x / m.nc;
  AxArgs<float> a = m.base;
#pragma unroll
  for (int c = 0; c < kMaxFields; ++c)
    if (f == c) {
      a.u = a.p = m.p[c];
      a.au = m.w[c];
      a.r = m.r[c];
      a.cg = m.cg[c];
      a.partial = m.partial[c];
    }
  axhelm_tma_body<NX, float, true, 1>(a, e, smem_raw);
}

// Boundary groups of C copies, G per thread: indices loaded once, every live
// field gathered, summed, masked and scattered (w kept in L2).
template <int C, int G>
__device__ __forceinline__ void multi_groups(const int* __restrict__ cidx, int s0, int step,
                                             int cnt, int goff, float* const* w,
                                             const float* const* segmask, const bool* live) {
  int id[G][C];
  bool on[G];
#pragma unroll
  for (int q = 0; q < G; ++q) {
    const int s = s0 + q * step;
    on[q] = s < cnt;
    if (on[q]) load_ids<C>(cidx, s, id[q]);
  }
  const uint64_t keep = l2_policy_evict_last();
#pragma unroll
  for (int f = 0; f < kMaxFields; ++f) {
    if (!live[f]) continue;
    float* wf = w[f];
    float v[G][C], mk[G];
#pragma unroll
    for (int q = 0; q < G; ++q) {
      if (!on[q]) continue;
#pragma unroll
      for (int c = 0; c < C; ++c) v[q][c] = ld_hint(wf + id[q][c], keep);
      mk[q] = segmask[f][goff + s0 + q * step];
    }
#pragma unroll
    for (int q = 0; q < G; ++q) {
      if (!on[q]) continue;
      float t = v[q][0];
#pragma unroll
      for (int c = 1; c < C; ++c) t = t + v[q][c];
      t = t * mk[q];
#pragma unroll
      for (int c = 0; c < C; ++c) st_hint(wf + id[q][c], t, keep);
    }
  }
}

struct MultiGsArgs {
  float* w[kMaxFields];
  const float* segmask[kMaxFields];
  CgScalars* cg[kMaxFields];
  const double* partialA[kMaxFields];  // per element rho partials
  double* partialB;                    // nc x nblk
  unsigned int* counter;
  const int* start;
  const int* idx;
  GsClasses cls;
  int nA, nc;
};

__global__ void __launch_bounds__(kGsThreads) multi_gs_kernel(const MultiGsArgs a) {
  bool live[kMaxFields];
  bool any = false;
#pragma unroll
  for (int c = 0; c < kMaxFields; ++c) {
    live[c] = c < a.nc && !a.cg[c]->done;
    any = any || live[c];
  }
  if (!any) return;
  const int blk = blockIdx.x, nblk = gridDim.x;
  const GsClasses& cls = a.cls;
  int k = 0;
  while (k < kGsClasses - 1 && blk >= cls.boff[k + 1]) ++k;
  const int G = cls.g[k];
  const int s0 = (blk - cls.boff[k]) * blockDim.x * G + threadIdx.x;
  const int* ci = a.idx + cls.ioff[k];
  const int goff = cls.soff[k], cnt = cls.cnt[k];
  switch (k) {
    case 0: multi_groups<1, gs_groups_per_thread(0)>(ci, s0, blockDim.x, cnt, goff, a.w, a.segmask, live); break;
    case 1: multi_groups<2, gs_groups_per_thread(1)>(ci, s0, blockDim.x, cnt, goff, a.w, a.segmask, live); break;
    case 2: multi_groups<4, gs_groups_per_thread(2)>(ci, s0, blockDim.x, cnt, goff, a.w, a.segmask, live); break;
    case 3: multi_groups<8, gs_groups_per_thread(3)>(ci, s0, blockDim.x, cnt, goff, a.w, a.segmask, live); break;
    default:
      for (int f = 0; f < kMaxFields; ++f) {
        if (!live[f]) continue;
        float* wf = a.w[f];
        for (int q = 0; q < G; ++q) {
          const int sl = s0 + q * blockDim.x;
          if (sl >= cnt) break;
          const int g = goff + sl;
          const int b0 = a.start[g], b1 = a.start[g + 1];
          float t = wf[a.idx[b0]];
          for (int c = b0 + 1; c < b1; ++c) t = t + wf[a.idx[c]];
          t = t * a.segmask[f][g];
          for (int c = b0; c < b1; ++c) wf[a.idx[c]] = t;
        }
      }
  }
  // rho of every live field from the operator's per-element partials, folded
  // in fixed chunks (as the single-field kernel); the last block sets rho and
  // alpha.  Warp 0 only: no block barrier.
  if (threadIdx.x >= 32) return;
  constexpr int kFold = 1024;
  for (int f = 0; f < kMaxFields; ++f) {
    if (!live[f]) continue;
    double pa = 0.0;
    for (int c0 = blk * kFold; c0 < a.nA; c0 += nblk * kFold)
      for (int q = c0 + threadIdx.x; q < min(c0 + kFold, a.nA); q += 32)
        pa += __ldcg(a.partialA[f] + q);
    pa = warp_sum(pa);
    if (threadIdx.x == 0) a.partialB[f * nblk + blk] = pa;
  }
  unsigned int last = 0;
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned int ticket = atomicAdd(a.counter, 1u);
    last = (ticket == (unsigned int)nblk - 1) ? 1u : 0u;
  }
  last = __shfl_sync(0xffffffffu, last, 0);
  if (!last) return;
  __threadfence();
  for (int f = 0; f < kMaxFields; ++f) {
    if (!live[f]) continue;
    double pb = 0.0;
    for (int q = threadIdx.x; q < nblk; q += 32) pb += __ldcg(a.partialB + f * nblk + q);
    pb = warp_sum(pb);
    if (threadIdx.x == 0) {
      a.cg[f]->rho = pb;
      a.cg[f]->alpha = a.cg[f]->rtz1 / pb;
    }
  }
  if (threadIdx.x == 0) *a.counter = 0u;
}

struct MultiUpdArgs {
  float* x;  // field c at c * n (also r, p, w)
  float* r;
  const float* p;
  const float* w;
  CgScalars* cg[kMaxFields];
  const float* md;  // mult * d
  const float* mb;  // mult * binv
  double* partial;  // 2 nc x nblk
  unsigned int* counter;
  int64_t n;
  int nc;
};

// x += alpha p, r -= alpha w; s1 = sum (r r) md, s2 = sum (r r) mb per live
// field; the last block runs each field's convergence test (cg_finalize).
template <bool FIRST>
__global__ void __launch_bounds__(kThreads) multi_update_kernel(const MultiUpdArgs a) {
  __shared__ double red[32];
  __shared__ int am_last;
  bool live[kMaxFields];
  bool any = false;
#pragma unroll
  for (int c = 0; c < kMaxFields; ++c) {
    live[c] = c < a.nc && !a.cg[c]->done;
    any = any || live[c];
  }
  if (!any) return;
  float alpha[kMaxFields];
#pragma unroll
  for (int c = 0; c < kMaxFields; ++c) alpha[c] = (FIRST || !live[c]) ? 0.f : (float)a.cg[c]->alpha;
  CompAcc<float> a1[kMaxFields], a2[kMaxFields];
  const int nblk = gridDim.x;
  const int64_t gtid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t stride = (int64_t)nblk * blockDim.x;
  const int64_t nv = a.n / 4;
  const uint64_t wpol = l2_policy_evict_first();
  for (int64_t iv = gtid; iv < nv; iv += stride) {
    float md[4], mb[4];
    ld16(md, a.md, iv);
    ld16(mb, a.mb, iv);
#pragma unroll
    for (int c = 0; c < kMaxFields; ++c) {
      if (!live[c]) continue;
      const int64_t fo = c * a.n;
      float rr[4];
      ld16(rr, a.r + fo, iv);
      if (!FIRST) {
        float xx[4], pp[4], ww[4];
        ld16(xx, a.x + fo, iv);
        ld16(pp, a.p + fo, iv);
        *reinterpret_cast<float4*>(ww) = ld_hint4(a.w + fo + 4 * iv, wpol);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          xx[q] = fma(alpha[c], pp[q], xx[q]);
          rr[q] = fma(-alpha[c], ww[q], rr[q]);
        }
        st16(a.x + fo, xx, iv);
        st16(a.r + fo, rr, iv);
      }
#pragma unroll
      for (int q = 0; q < 4; ++q) {
        const float r2 = rr[q] * rr[q];
        a1[c].add(r2 * md[q]);
        a2[c].add(r2 * mb[q]);
      }
    }
  }
  for (int64_t i = nv * 4 + gtid; i < a.n; i += stride) {
    for (int c = 0; c < kMaxFields; ++c) {
      if (!live[c]) continue;
      const int64_t fi = c * a.n + i;
      float ri = a.r[fi];
      if (!FIRST) {
        a.x[fi] = fma(alpha[c], a.p[fi], a.x[fi]);
        ri = fma(-alpha[c], a.w[fi], ri);
        a.r[fi] = ri;
      }
      const float r2 = ri * ri;
      a1[c].add(r2 * a.md[i]);
      a2[c].add(r2 * a.mb[i]);
    }
  }
  for (int c = 0; c < kMaxFields; ++c) {
    if (!live[c]) continue;  // uniform: every thread takes the same branch
    const double b1 = block_sum_comp(a1[c], red);
    const double b2 = block_sum_comp(a2[c], red);
    if (threadIdx.x == 0) {
      a.partial[(2 * c) * nblk + blockIdx.x] = b1;
      a.partial[(2 * c + 1) * nblk + blockIdx.x] = b2;
    }
  }
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned int ticket = atomicAdd(a.counter, 1u);
    am_last = (ticket == (unsigned int)nblk - 1);
  }
  __syncthreads();
  if (!am_last) return;
  for (int c = 0; c < kMaxFields; ++c) {
    if (!live[c]) continue;
    double t1 = 0.0, t2 = 0.0;
    for (int q = threadIdx.x; q < nblk; q += blockDim.x) {
      t1 += __ldcg(a.partial + (2 * c) * nblk + q);
      t2 += __ldcg(a.partial + (2 * c + 1) * nblk + q);
    }
    const double s1 = block_sum(t1, red);
    const double s2 = block_sum(t2, red);
    if (threadIdx.x == 0) cg_finalize(a.cg[c], s1, s2);
  }
  if (threadIdx.x == 0) *a.counter = 0u;
}

__global__ void fold_kernel(float* __restrict__ md, float* __restrict__ mb,
                            const float* __restrict__ d, const float* __restrict__ mult,
                            const float* __restrict__ binv, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    md[i] = mult[i] * d[i];
    mb[i] = mult[i] * binv[i];
  }
}

template <int NX>
cudaError_t launch_op_nx(const MultiTmaArgs& m, cudaStream_t s) {
  const size_t smem = tma_smem_bytes<NX, float, 1>(true, m.base.h1mode, m.base.h2mode);
  static std::atomic<uint32_t> configured{0};  // per device
  if (first_on_device(configured)) {
    const int maxb = (int)tma_smem_bytes<NX, float, 1>(true, 1, 2);
    cudaError_t e = cudaFuncSetAttribute(multi_op_kernel<NX>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, maxb);
    if (e != cudaSuccess) return e;
    cudaFuncSetAttribute(multi_op_kernel<NX>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         100);
    mark_device(configured);
  }
  count_launch();
  multi_op_kernel<NX><<<m.base.nel * m.nc, NX * NX, smem, s>>>(m);
  return cudaGetLastError();
}

cudaError_t launch_op(int nx, const MultiTmaArgs& m, cudaStream_t s) {
  switch (nx) {
    case 2: return launch_op_nx<2>(m, s);
    case 4: return launch_op_nx<4>(m, s);
    case 6: return launch_op_nx<6>(m, s);
    case 8: return launch_op_nx<8>(m, s);
    case 10: return launch_op_nx<10>(m, s);
    case 12: return launch_op_nx<12>(m, s);
    default: return cudaErrorInvalidValue;
  }
}

inline bool al16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

}  // namespace

// Mixed solve of nc fields sharing h1, h2, mult and binv (masks per field).
int mixed_multi_solve(Handle& h, int nc, double* const* x, const double* const* f,
                      const double* h1, const double* h2, const double* const* mask,
                      const double* mult, const double* binv, double tin, int maxit,
                      double inner_tol, int* nouter, int* ninner, double* rbn0, double* rbn2,
                      int* status) {
  Mesh& m = h.mesh;
  const int64_t n = m.n;
  cudaStream_t s = h.stream;
  for (int c = 0; c < nc; ++c) {
    nouter[c] = ninner[c] = 0;
    rbn0[c] = rbn2[c] = 0.0;
    status[c] = 0;
  }
  // TMA staging needs even lx1; otherwise one field after another
  if (m.nx1 % 2 != 0 || !m.use_tma) {
    for (int c = 0; c < nc; ++c) {
      MixedResult r = mixed_solve(h, x[c], f[c], h1, h2, mask[c], mult, binv, tin, maxit,
                                  inner_tol, 1);
      nouter[c] = r.outer;
      ninner[c] = r.inner;
      rbn0[c] = r.rbn0;
      rbn2[c] = r.rbn2;
      status[c] = r.status == -5 ? NEKGPU_ENOTCONV
                  : r.status == -7 ? NEKGPU_ENAN
                  : r.status == -1 ? NEKGPU_EINVAL
                  : r.status       ? NEKGPU_ECUDA
                                   : 0;
    }
    return 0;
  }
  if (ensure_f32(h)) {
    set_error(h, "multi: FP32 operator data allocation failed");
    return -4;
  }
  PcgWork<float>& w32 = h.w32;
  PcgWork<double>& w64 = h.w64;
  if ((int)h.multi.size() < nc) h.multi.resize(nc);
  for (int c = 0; c < nc; ++c)
    if (!h.multi[c]) h.multi[c].reset(new MultiField());
  const int nbB = std::max(gs_cg_blocks(m.gs), 1);
  const int nbC = vblocks(n);
  if (w32.mult.ensure(n) || w32.binv.ensure(n) || w32.d.ensure(n) || w32.md.ensure(n) ||
      w32.mb.ensure(n) || w32.h1.ensure(n) || w32.h2.ensure(n) || w32.segmsum.ensure(m.gs.nbseg) ||
      w64.d.ensure(n) || w64.w.ensure(n) || h.mpartialA.ensure((size_t)nc * m.nel) ||
      h.mpartialB.ensure((size_t)nc * nbB) || h.mpartialC.ensure((size_t)2 * nc * nbC) ||
      h.mcounter.ensure(2) || h.red.ensure((size_t)4 * 152 * 8)) {  // replacement sums
    set_error(h, "multi: device allocation failed");
    return -4;
  }
  if (h.mfr.ensure((size_t)nc * n) || h.mfp.ensure((size_t)nc * n) ||
      h.mfw.ensure((size_t)nc * n) || h.mfx.ensure((size_t)nc * n)) {
    set_error(h, "multi: device allocation failed");
    return -4;
  }
  // field c's FP32 PCG vectors
  auto fr = [&](int c) { return h.mfr.ptr + (size_t)c * n; };
  auto fp = [&](int c) { return h.mfp.ptr + (size_t)c * n; };
  auto fw = [&](int c) { return h.mfw.ptr + (size_t)c * n; };
  auto fx = [&](int c) { return h.mfx.ptr + (size_t)c * n; };
  for (int c = 0; c < nc; ++c) {
    MultiField& F = *h.multi[c];
    if (F.mask.ensure(n) || F.segmask.ensure(m.gs.nbseg) || F.r64.ensure(n) || F.cg.ensure(1)) {
      set_error(h, "multi: device allocation failed");
      return -4;
    }
    if (!F.cg_host) {
      if (cudaMallocHost(&F.cg_host, sizeof(CgScalars)) != cudaSuccess) {
        set_error(h, "multi: host allocation failed");
        return -4;
      }
    }
  }
  cudaMemsetAsync(h.mcounter.ptr, 0, 2 * sizeof(unsigned int), s);
  Coef<double> c64;
  if (detect_coef<double>(h, h1, h2, n, c64)) {
    set_error(h, "multi: coefficient scan failed");
    return -3;
  }
  Coef<float> c32;
  c32.h1mode = c64.h1mode;
  c32.h2mode = c64.h2mode;
  c32.h1s = (float)c64.h1s;
  c32.h2s = (float)c64.h2s;
  if (c64.h1mode) cast_to_f32(h, w32.h1.ptr, h1, 1.0, n);
  if (c64.h2mode == 2) cast_to_f32(h, w32.h2.ptr, h2, 1.0, n);
  cast_to_f32(h, w32.mult.ptr, mult, 1.0, n);
  cast_to_f32(h, w32.binv.ptr, binv, 1.0, n);
  if (setprec_f64(h, w64.d.ptr, c64)) {
    set_error(h, "multi: setprec failed");
    return -3;
  }
  cast_to_f32(h, w32.d.ptr, w64.d.ptr, 1.0, n);
  count_launch();
  fold_kernel<<<vblocks(n), kThreads, 0, s>>>(w32.md.ptr, w32.mb.ptr, w32.d.ptr, w32.mult.ptr,
                                              w32.binv.ptr, n);
  // per field: FP64 residual r = f, x = 0, scaled FP32 residual, scalars
  std::vector<double> tol(nc, 0.0), rbn(nc, 0.0), scale(nc, 1.0);
  std::vector<char> active(nc, 0);
  for (int c = 0; c < nc; ++c) {
    MultiField& F = *h.multi[c];
    CgScalars& hc = *F.cg_host;
    memset(&hc, 0, sizeof(hc));
    hc.done = 1;  // a refused field stays out of every kernel
    cudaMemcpyAsync(F.cg.ptr, &hc, sizeof(hc), cudaMemcpyHostToDevice, s);
    if (c64.h2mode == 0) {  // no Dirichlet point and h2 = 0: a null space
      int st0 = 0;
      const double skmin = device_sum(h, 6, mask[c], nullptr, nullptr, n, &st0);
      if (!st0 && skmin > 0.0) {
        status[c] = NEKGPU_EINVAL;
        set_error(h, "multi: singular operator (no Dirichlet point and h2 = 0)");
        continue;
      }
    }
    cast_to_f32(h, F.mask.ptr, mask[c], 1.0, n);
    cudaMemsetAsync(x[c], 0, n * sizeof(double), s);
    cudaMemcpyAsync(F.r64.ptr, f[c], n * sizeof(double), cudaMemcpyDeviceToDevice, s);
    const double r0 = norm64(h, F.r64.ptr, mult, binv);
    if (!(r0 >= 0.0) || !std::isfinite(r0)) {
      status[c] = NEKGPU_ENAN;
      continue;
    }
    rbn0[c] = rbn2[c] = rbn[c] = r0;
    tol[c] = tin < 0 ? std::fabs(tin) * r0 : std::fabs(tin);
    int st = 0;
    const double amax = device_absmax<double>(h, F.r64.ptr, n, &st);
    if (st) return -3;
    active[c] = r0 > 0.0 && amax > 0.0 && r0 > tol[c];
    scale[c] = amax > 0.0 ? std::ldexp(1.0, std::ilogb(amax)) : 1.0;
    cast_to_f32(h, fr(c), F.r64.ptr, 1.0 / scale[c], n);
    cudaMemsetAsync(fx(c), 0, n * sizeof(float), s);
    cudaMemsetAsync(fp(c), 0, n * sizeof(float), s);
    cudaMemsetAsync(h.flag, 0, 2 * sizeof(int), s);
    gs_cg_weights<float>(m.gs, F.mask.ptr, w32.mult.ptr, F.segmask.ptr, w32.segmsum.ptr, h.flag,
                         s);
    launch_interior_check(h, F.mask.ptr, w32.mult.ptr, h.flag + 1);
    int flags[2] = {0, 0};
    cudaMemcpyAsync(flags, h.flag, 2 * sizeof(int), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) {
      set_error(h, std::string("multi: ") + cudaGetErrorString(cudaGetLastError()));
      return -3;
    }
    if (flags[0] || flags[1]) {  // as pcg_prepare: the field is refused
      status[c] = NEKGPU_EINVAL;
      active[c] = 0;
      set_error(h, flags[0] ? "multi: mask differs between copies of a shared node"
                            : "multi: an element-interior point has mask or multiplicity other than 1");
      continue;
    }
    memset(&hc, 0, sizeof(hc));
    hc.rtz1 = 1.0;
    hc.tin = -inner_tol;
    hc.tol = inner_tol;
    hc.vol = m.vol;
    hc.maxiter = maxit;
    hc.done = active[c] ? 0 : 1;
    cudaMemcpyAsync(F.cg.ptr, &hc, sizeof(hc), cudaMemcpyHostToDevice, s);
  }
  if (cudaStreamSynchronize(s) != cudaSuccess) {
    set_error(h, std::string("multi: ") + cudaGetErrorString(cudaGetLastError()));
    return -3;
  }
  // kernel arguments (fixed for the whole solve)
  MultiTmaArgs oa{};
  oa.base.G = m.f32.G;
  oa.base.bm1 = m.f32.bm1;
  oa.base.h1 = c32.h1mode ? w32.h1.ptr : nullptr;
  oa.base.h2 = c32.h2mode == 2 ? w32.h2.ptr : nullptr;
  oa.base.h1s = c32.h1s;
  oa.base.h2s = c32.h2s;
  oa.base.h1mode = c32.h1mode;
  oa.base.h2mode = c32.h2mode;
  oa.base.D = m.f32.D;
  oa.base.d = w32.d.ptr;
  oa.base.nel = m.nel;
  oa.base.err = m.dev_err;
  oa.base.skip = m.gs.skip;
  oa.base.allrho = 1;
  oa.base.shared_in = 1;
  oa.nc = nc;
  MultiGsArgs ga{};
  ga.partialB = h.mpartialB.ptr;
  ga.counter = h.mcounter.ptr;
  ga.start = m.gs.bstart;
  ga.idx = m.gs.bidx;
  ga.cls = m.gs.cls;
  ga.nA = m.nel;
  ga.nc = nc;
  MultiUpdArgs ua{};
  ua.md = w32.md.ptr;
  ua.mb = w32.mb.ptr;
  ua.x = h.mfx.ptr;
  ua.r = h.mfr.ptr;
  ua.p = h.mfp.ptr;
  ua.w = h.mfw.ptr;
  ua.partial = h.mpartialC.ptr;
  ua.counter = h.mcounter.ptr + 1;
  ua.n = n;
  ua.nc = nc;
  bool aligned = al16(oa.base.G) && al16(oa.base.bm1) && al16(oa.base.d) &&
                 (!oa.base.h1 || al16(oa.base.h1)) && (!oa.base.h2 || al16(oa.base.h2)) &&
                 al16(ua.md) && al16(ua.mb);
  for (int c = 0; c < nc; ++c) {
    MultiField& F = *h.multi[c];
    oa.p[c] = fp(c);
    oa.r[c] = fr(c);
    oa.w[c] = fw(c);
    oa.cg[c] = F.cg.ptr;
    oa.partial[c] = h.mpartialA.ptr + (size_t)c * m.nel;
    ga.w[c] = fw(c);
    ga.segmask[c] = F.segmask.ptr;
    ga.cg[c] = F.cg.ptr;
    ga.partialA[c] = oa.partial[c];
    ua.cg[c] = F.cg.ptr;
    aligned = aligned && al16(fp(c)) && al16(fr(c)) && al16(fw(c)) && al16(fx(c));
  }
  if (!aligned) {
    set_error(h, "multi: arrays not 16-byte aligned");
    return -1;
  }
  const int nbG = gs_cg_blocks(m.gs);
  const int chunk = std::max(1, h.graph_chunk);
  // With timing on, four events per iteration (before the operator, after
  // it, after the boundary-group kernel, after the update); iterations in
  // which every field was live are summed into ms_axhelm / ms_gs / ms_update.
  if (h.timing && h.ax_ev.size() < 4 * (size_t)chunk) {
    for (cudaEvent_t e : h.ax_ev) cudaEventDestroy(e);
    h.ax_ev.assign(4 * (size_t)chunk, nullptr);
    for (auto& e : h.ax_ev) cudaEventCreate(&e);
  }
  auto iteration = [&](int q) -> cudaError_t {
    if (h.timing) cudaEventRecord(h.ax_ev[4 * q], s);
    cudaError_t e = launch_op(m.nx1, oa, s);
    if (e != cudaSuccess) return e;
    if (h.timing) cudaEventRecord(h.ax_ev[4 * q + 1], s);
    count_launch(2);
    multi_gs_kernel<<<nbG, m.gs.cls.threads, 0, s>>>(ga);
    if (h.timing) cudaEventRecord(h.ax_ev[4 * q + 2], s);
    multi_update_kernel<false><<<nbC, kThreads, 0, s>>>(ua);
    if (h.timing) cudaEventRecord(h.ax_ev[4 * q + 3], s);
    return cudaGetLastError();
  };
  count_launch();
  multi_update_kernel<true><<<nbC, kThreads, 0, s>>>(ua);  // iteration-1 checks
  std::vector<int> iter_before(nc, 0);
  for (int round = 0; round < 100000; ++round) {
    // iterate until every field's FP32 PCG has stopped
    int launched = 0;
    bool all_live = false;
    for (;;) {
      bool all = true;
      for (int c = 0; c < nc; ++c) {
        cudaMemcpyAsync(h.multi[c]->cg_host, h.multi[c]->cg.ptr, sizeof(CgScalars),
                        cudaMemcpyDeviceToHost, s);
      }
      if (cudaStreamSynchronize(s) != cudaSuccess) {
        set_error(h, std::string("multi: ") + cudaGetErrorString(cudaGetLastError()));
        return -3;
      }
      if (h.timing && launched && all_live) {
        int live = launched;
        for (int c = 0; c < nc; ++c)
          live = std::min(live, h.multi[c]->cg_host->iter - iter_before[c]);
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
      all_live = true;
      for (int c = 0; c < nc; ++c) {
        all = all && h.multi[c]->cg_host->done;
        all_live = all_live && !h.multi[c]->cg_host->done;
        iter_before[c] = h.multi[c]->cg_host->iter;
      }
      if (all) break;
      for (int q = 0; q < chunk; ++q) {
        cudaError_t e = iteration(q);
        if (e != cudaSuccess) {
          set_error(h, std::string("multi iteration launch: ") + cudaGetErrorString(e));
          return -3;
        }
      }
      launched = chunk;
    }
    // fold each stopped field into FP64, recompute its residual, replace
    bool more = false;
    for (int c = 0; c < nc; ++c) {
      if (!active[c] || status[c]) continue;
      MultiField& F = *h.multi[c];
      CgScalars& hc = *F.cg_host;
      ninner[c] = hc.niter;
      nouter[c] = round + 1;
      const bool capped = hc.iter > hc.maxiter;
      axpy_f32(h, x[c], fx(c), scale[c], n);
      const double rnew = outer_residual(h, F.r64.ptr, f[c], x[c], c64, mask[c], mult, binv,
                                         w64.w.ptr);
      if (!(rnew >= 0.0) || !std::isfinite(rnew)) {
        status[c] = NEKGPU_ENAN;
        active[c] = 0;
        continue;
      }
      const bool progress = rnew < rbn[c];
      rbn[c] = rbn2[c] = rnew;
      if (rnew <= tol[c] || capped || !progress) {
        active[c] = 0;
        continue;
      }
      ReplaceTarget t{fr(c), fp(c), fx(c), w32.d.ptr, w32.mult.ptr, w32.binv.ptr,
                      F.r64.ptr, F.cg.ptr, F.cg_host};
      const int rr = mixed_replace_into(h, t, scale[c], inner_tol, nullptr);
      if (rr < 0) {
        status[c] = NEKGPU_ECUDA;
        active[c] = 0;
        continue;
      }
      if (rr == 1) {
        active[c] = 0;
        continue;
      }
      more = true;
    }
    if (!more) break;
  }
  for (int c = 0; c < nc; ++c)
    if (!status[c] && rbn0[c] > 0.0 && !(rbn[c] <= tol[c])) status[c] = NEKGPU_ENOTCONV;
  return 0;
}

}  // namespace nekgpu

// ---------------------------------------------------------------------------
// C ABI
namespace nekgpu {
Handle* handle_lookup(const int64_t* h);
int handle_fail(Handle* H, int code, const std::string& msg);
}  // namespace nekgpu

using namespace nekgpu;

extern "C" int nekgpu_cggo_mixed_multi_dev(const int64_t* handle, const int* nfield,
                                           double* const* x, const double* const* f,
                                           const double* h1, const double* h2,
                                           const double* const* mask, const double* mult,
                                           const int* imsh, const double* tin, const int* maxit,
                                           const int* isd, const double* binv,
                                           const double* inner_tol, int* niter_outer,
                                           int* niter_inner, double* rbn0, double* rbn2,
                                           int* status) {
  (void)imsh;
  (void)isd;
  Handle* H = handle_lookup(handle);
  if (!H) return handle_fail(nullptr, NEKGPU_EHANDLE, "unknown handle");
  if (handle_enter(*H) != cudaSuccess)
    return handle_fail(H, NEKGPU_ECUDA, "call entry failed");
  if (!H->has_mesh) return handle_fail(H, NEKGPU_ENOSETUP, "mesh not set up (nekgpu_setup)");
  if (!nfield || !x || !f || !h1 || !h2 || !mask || !mult || !binv || !tin || !maxit ||
      !niter_outer || !niter_inner || !rbn0 || !rbn2 || !status)
    return handle_fail(H, NEKGPU_EINVAL, "null argument");
  const int nc = *nfield;
  if (nc < 1 || nc > NEKGPU_MULTI_MAX)
    return handle_fail(H, NEKGPU_EINVAL, "nfield must be in [1, NEKGPU_MULTI_MAX]");
  for (int c = 0; c < nc; ++c)
    if (!x[c] || !f[c] || !mask[c]) return handle_fail(H, NEKGPU_EINVAL, "null field array");
  const double itol = inner_tol ? *inner_tol : 1e-2;
  if (!(itol > 0.0 && itol < 1.0)) return handle_fail(H, NEKGPU_EINVAL, "inner_tol must be in (0, 1)");
  H->err.clear();
  H->ms_axhelm = H->ms_gs = H->ms_update = 0.0;
  H->n_axhelm = 0;
  if (H->timing) cudaEventRecord(H->evt0, H->stream);
  const int rc = mixed_multi_solve(*H, nc, x, f, h1, h2, mask, mult, binv, *tin, *maxit, itol,
                                   niter_outer, niter_inner, rbn0, rbn2, status);
  handle_leave(*H);  // no kernel of the call runs after it returns
  if (H->timing) {
    cudaEventRecord(H->evt1, H->stream);
    cudaEventSynchronize(H->evt1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, H->evt0, H->evt1);
    H->ms_total = ms;
  }
  if (rc) return handle_fail(H, rc == -4 ? NEKGPU_ENOMEM : rc == -1 ? NEKGPU_EINVAL : NEKGPU_ECUDA,
                             H->err.empty() ? "multi-field solve failed" : H->err);
  return NEKGPU_OK;
}
