// batch.cu -- many independent Helmholtz solves of uneven size and order,
// advanced together.
//
// Every problem keeps its own mesh, work vectors, PCG scalars and partial
// sums (one Handle each, all on the batch's stream).  One PCG iteration of
// the whole batch is the fused operator, the boundary-group gather-scatter
// and the update, each covering every problem: a per-block table maps a block
// to its problem, and the block runs that problem's body.  The operator is
// one launch per polynomial order present (the problems' blocks grouped by
// lx1), each compiled for its order alone, so that a launch holds only the
// registers its order needs (one kernel over every order would carry the
// largest order's registers, about 145 for FP32, and run one 256-thread block
// per SM).  For FP32 and even lx1 the order's launch is the TMA-staged
// operator body (axhelm_tma.cuh), as in a single solve.  A problem that has
// converged makes its blocks return at once, so each one stops at its own
// iteration count, exactly as if it were solved alone.  Chunks of iterations
// are captured once as a CUDA graph and replayed.
//
// The mixed form runs FP64 defect correction per problem around the batched
// FP32 PCG: every outer step solves all problems not yet converged together.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>

#include "axhelm_tma.cuh"
#include "cg_kernels.cuh"
#include "gs_kernels.cuh"
#include "impl.cuh"
#include "nekgpu.h"

namespace nekgpu {

template <typename T>
struct BDesc {
  AxArgs<T> ax;  // fused operator: au = w, u = p (old), p, r, d, cg, partial = rho partials
  int nx1, epb, nblkA;  // operator blocks; the rho partials are one per element (ax.nel)
  const int* bstart;
  const int* bidx;
  GsClasses cls;
  const T* segmask;
  const T* segmsum;
  double* partialB;
  int nblkB;
  T* x;
  const T* mult;
  const T* binv;
  const T* md;  // folded update weights mult*d, mult*binv (pcg_solve_extras)
  const T* mb;
  int64_t n;
  double* partialC;
  int nblkC, vec;
  CgScalars* cg;
};

namespace {

constexpr int kBatchThreads = 256;

// Every problem's PCG scalars into one array (one warp per problem), so that
// the host reads them with one copy after a chunk.
template <typename T>
__global__ void __launch_bounds__(256)
    batch_gather_cg_kernel(const BDesc<T>* __restrict__ D, int np, CgScalars* __restrict__ out) {
  const int q = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
  if (q >= np) return;
  const unsigned int* src = reinterpret_cast<const unsigned int*>(D[q].cg);
  unsigned int* dst = reinterpret_cast<unsigned int*>(out + q);
  for (int w = threadIdx.x % 32; w < (int)(sizeof(CgScalars) / 4); w += 32) dst[w] = __ldcg(src + w);
}

template <typename T, int NX>
__device__ __forceinline__ void batch_ax_nx(const AxArgs<T>& a, int blk, int epb,
                                            unsigned char* smem, double* red) {
  constexpr int NXY = NX * NX;
  axhelm_body<NX, T, false, true>(a, blk, threadIdx.x % NXY, threadIdx.x / NXY, epb, smem, red);
}

// The operator for the problems of one order: virtual blocks start ..
// start + gridDim.x - 1 of the operator table (every one of lx1 = NX).
template <typename T, int NX>
__global__ void __launch_bounds__(kBatchThreads)
    batch_axhelm_nx_kernel(const BDesc<T>* __restrict__ D, const int* __restrict__ map,
                           const int* __restrict__ base, int start) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double red[32];
  const int vb = start + (int)blockIdx.x;
  const int pi = map[vb];
  const BDesc<T>* d = D + pi;
  if (d->cg->done) return;
  const AxArgs<T> a = d->ax;
  batch_ax_nx<T, NX>(a, vb - base[pi], d->epb, smem, red);
}

// Elements per block of the batched TMA-staged FP32 operator: one for
// lx1 >= 7 (what the single-solve autotuner picks there), else the built-in
// count of about 128 threads.
template <int NX>
__host__ __device__ constexpr int batch_tma_epb() {
  return NX >= 7 ? 1 : tma_epb<NX>();
}

// The TMA-staged FP32 operator for the problems of one order (blocks of
// (NX*NX, EPB) threads; virtual blocks as batch_axhelm_nx_kernel).
template <int NX, int EPB>
__global__ void __launch_bounds__(NX* NX* EPB)
    batch_axhelm_tma_kernel(const BDesc<float>* __restrict__ D, const int* __restrict__ map,
                            const int* __restrict__ base, int start) {
  extern __shared__ __align__(128) unsigned char smem_tma[];
  const int vb = start + (int)blockIdx.x;
  const int pi = map[vb];
  const BDesc<float>* d = D + pi;
  if (d->cg->done) return;
  const AxArgs<float> a = d->ax;
  axhelm_tma_body<NX, float, true, EPB>(a, vb - base[pi], smem_tma);
}

template <typename T>
__global__ void __launch_bounds__(kGsThreads)
    batch_gs_kernel(const BDesc<T>* __restrict__ D, const int* __restrict__ map,
                    const int* __restrict__ base) {
  __shared__ double red[32];
  __shared__ int am_last;
  const int pi = map[blockIdx.x];
  const BDesc<T>* d = D + pi;
  if (d->cg->done) return;
  gs_cg_body<T>(d->ax.au, d->ax.p, d->bstart, d->bidx, d->cls, d->segmask, d->segmsum, d->cg,
                d->ax.partial, d->ax.nel, d->partialB, blockIdx.x - base[pi], d->nblkB, red,
                &am_last);
}

template <typename T, bool FIRST>
__global__ void __launch_bounds__(kBatchThreads)
    batch_update_kernel(const BDesc<T>* __restrict__ D, const int* __restrict__ map,
                        const int* __restrict__ base) {
  __shared__ double red[32];
  __shared__ int am_last;
  const int pi = map[blockIdx.x];
  const BDesc<T>* d = D + pi;
  if (d->cg->done) return;
  const int blk = blockIdx.x - base[pi];
  // the single-problem solve's fused multiply-add form: folded weights
  if (d->vec)
    cg_update_body<T, false, FIRST, true, true>(d->x, const_cast<T*>(d->ax.r), d->ax.p, d->ax.au,
                                                d->md, d->mult, d->mb, d->n, d->cg, d->partialC,
                                                blk, d->nblkC, red, &am_last);
  else
    cg_update_body<T, false, FIRST, false, true>(d->x, const_cast<T*>(d->ax.r), d->ax.p,
                                                 d->ax.au, d->md, d->mult, d->mb, d->n, d->cg,
                                                 d->partialC, blk, d->nblkC, red, &am_last);
}

// ---- the persistent form: one cooperative launch runs whole iterations ----
//
// Every block of the launch stays resident (cudaLaunchCooperativeKernel
// checks that they all fit at once) and walks the virtual blocks of the three
// phases of an iteration -- the operator blocks of every problem, their
// boundary-group blocks, their update blocks, with the same tables as the
// three-launch form -- separated by grid-wide barriers.  It keeps iterating
// until every problem has stopped or `kmax` iterations have run.  The
// barrier is a counter and a generation word in global memory; its wait is
// bounded (kBarrierLimit polls with a short sleep, seconds in all), after
// which the block raises bit 2 of *err and every block leaves at the next
// barrier, so that a lost block can never hold the GPU.
constexpr unsigned int kBarrierLimit = 1u << 24;

__device__ __forceinline__ bool grid_barrier(unsigned int* bar, unsigned int nblocks, int* err) {
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* gen = bar + 1;
    const unsigned int g = *gen;
    __threadfence();
    const unsigned int t = atomicAdd(bar, 1u);
    if (t == nblocks - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      unsigned int it = 0;
      while (*gen == g) {
        if (++it > kBarrierLimit) {
          atomicOr(err, 2);
          break;
        }
        __nanosleep(100);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return *reinterpret_cast<volatile int*>(err) == 0;
}

template <typename T>
__global__ void __launch_bounds__(kBatchThreads, 2)
    batch_persistent_kernel(const BDesc<T>* __restrict__ D, int np, const int* __restrict__ mapA,
                            const int* __restrict__ baseA, int gridA, const int* __restrict__ mapB,
                            const int* __restrict__ baseB, int gridB,
                            const int* __restrict__ mapC, const int* __restrict__ baseC,
                            int gridC, int kmax, unsigned int* bar, int* err) {
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ double red[32];
  __shared__ int am_last;
  __shared__ int all_done;
  const unsigned int nb = gridDim.x;
  for (int it = 0; it < kmax; ++it) {
    for (int v = blockIdx.x; v < gridA; v += nb) {  // the operator
      const int pi = mapA[v];
      const BDesc<T>* d = D + pi;
      if (d->cg->done) continue;
      const AxArgs<T> a = d->ax;
      const int blk = v - baseA[pi], epb = d->epb;
      switch (d->nx1) {
        case 2: batch_ax_nx<T, 2>(a, blk, epb, smem, red); break;
        case 3: batch_ax_nx<T, 3>(a, blk, epb, smem, red); break;
        case 4: batch_ax_nx<T, 4>(a, blk, epb, smem, red); break;
        case 5: batch_ax_nx<T, 5>(a, blk, epb, smem, red); break;
        case 6: batch_ax_nx<T, 6>(a, blk, epb, smem, red); break;
        case 7: batch_ax_nx<T, 7>(a, blk, epb, smem, red); break;
        case 8: batch_ax_nx<T, 8>(a, blk, epb, smem, red); break;
        case 9: batch_ax_nx<T, 9>(a, blk, epb, smem, red); break;
        case 10: batch_ax_nx<T, 10>(a, blk, epb, smem, red); break;
        case 11: batch_ax_nx<T, 11>(a, blk, epb, smem, red); break;
        default: batch_ax_nx<T, 12>(a, blk, epb, smem, red); break;
      }
      __syncthreads();  // the next virtual block reuses the shared memory
    }
    if (!grid_barrier(bar, nb, err)) return;
    for (int v = blockIdx.x; v < gridB; v += nb) {  // the boundary groups
      const int pi = mapB[v];
      const BDesc<T>* d = D + pi;
      if (d->cg->done) continue;
      gs_cg_body<T>(d->ax.au, d->ax.p, d->bstart, d->bidx, d->cls, d->segmask, d->segmsum, d->cg,
                    d->ax.partial, d->ax.nel, d->partialB, v - baseB[pi], d->nblkB, red,
                    &am_last);
      __syncthreads();
    }
    if (!grid_barrier(bar, nb, err)) return;
    for (int v = blockIdx.x; v < gridC; v += nb) {  // the update
      const int pi = mapC[v];
      const BDesc<T>* d = D + pi;
      if (d->cg->done) continue;
      const int blk = v - baseC[pi];
      if (d->vec)
        cg_update_body<T, false, false, true, true>(d->x, const_cast<T*>(d->ax.r), d->ax.p,
                                                    d->ax.au, d->md, d->mult, d->mb, d->n, d->cg,
                                                    d->partialC, blk, d->nblkC, red, &am_last);
      else
        cg_update_body<T, false, false, false, true>(d->x, const_cast<T*>(d->ax.r), d->ax.p,
                                                     d->ax.au, d->md, d->mult, d->mb, d->n,
                                                     d->cg, d->partialC, blk, d->nblkC, red,
                                                     &am_last);
      __syncthreads();
    }
    if (!grid_barrier(bar, nb, err)) return;
    if (threadIdx.x == 0) {  // every problem stopped: leave (the same answer in every block)
      int all = 1;
      for (int q = 0; q < np; ++q) all &= (*reinterpret_cast<volatile int*>(&D[q].cg->done) != 0);
      all_done = all;
    }
    __syncthreads();
    if (all_done) return;
  }
}

// Shared memory of one operator block: epb elements of lx1 = nx.
template <typename T>
size_t batch_smem(int nx, int epb) {
  switch (nx) {
    case 2: return axhelm_smem_bytes<2, T>(epb);
    case 3: return axhelm_smem_bytes<3, T>(epb);
    case 4: return axhelm_smem_bytes<4, T>(epb);
    case 5: return axhelm_smem_bytes<5, T>(epb);
    case 6: return axhelm_smem_bytes<6, T>(epb);
    case 7: return axhelm_smem_bytes<7, T>(epb);
    case 8: return axhelm_smem_bytes<8, T>(epb);
    case 9: return axhelm_smem_bytes<9, T>(epb);
    case 10: return axhelm_smem_bytes<10, T>(epb);
    case 11: return axhelm_smem_bytes<11, T>(epb);
    default: return axhelm_smem_bytes<12, T>(epb);
  }
}

// Elements per operator block of lx1 = nx in a block of `threads` threads.
inline int batch_epb(int nx, int threads) { return std::max(1, threads / (nx * nx)); }

// Largest operator-block shared memory over every lx1 at up to kBatchThreads.
template <typename T>
size_t batch_smem_max() {
  size_t b = 0;
  for (int nx = 2; nx <= NEKGPU_MAX_LX1; ++nx)
    b = std::max(b, batch_smem<T>(nx, batch_epb(nx, kBatchThreads)));
  return b;
}

// Elements per block and shared memory of the batched TMA operator
// (tma_lx1(nx)).
int batch_tma_epb_rt(int nx) {
  switch (nx) {
    case 2: return batch_tma_epb<2>();
    case 3: return batch_tma_epb<3>();
    case 4: return batch_tma_epb<4>();
    case 5: return batch_tma_epb<5>();
    case 7: return batch_tma_epb<7>();
    case 9: return batch_tma_epb<9>();
    case 6: return batch_tma_epb<6>();
    case 8: return batch_tma_epb<8>();
    case 10: return batch_tma_epb<10>();
    default: return batch_tma_epb<12>();
  }
}

size_t batch_tma_smem(int nx, int h1m, int h2m) {
  switch (nx) {
    case 2: return tma_smem_bytes<2, float, batch_tma_epb<2>()>(true, h1m, h2m);
    case 3: return tma_smem_bytes<3, float, batch_tma_epb<3>()>(true, h1m, h2m);
    case 4: return tma_smem_bytes<4, float, batch_tma_epb<4>()>(true, h1m, h2m);
    case 5: return tma_smem_bytes<5, float, batch_tma_epb<5>()>(true, h1m, h2m);
    case 7: return tma_smem_bytes<7, float, batch_tma_epb<7>()>(true, h1m, h2m);
    case 9: return tma_smem_bytes<9, float, batch_tma_epb<9>()>(true, h1m, h2m);
    case 6: return tma_smem_bytes<6, float, batch_tma_epb<6>()>(true, h1m, h2m);
    case 8: return tma_smem_bytes<8, float, batch_tma_epb<8>()>(true, h1m, h2m);
    case 10: return tma_smem_bytes<10, float, batch_tma_epb<10>()>(true, h1m, h2m);
    default: return tma_smem_bytes<12, float, batch_tma_epb<12>()>(true, h1m, h2m);
  }
}

// Every array the TMA body stages is 16-byte aligned.
template <typename T>
bool batch_tma_aligned(const AxArgs<T>& a) {
  auto al = [](const void* p) { return ((uintptr_t)p & 15u) == 0; };
  bool ok = al(a.u) && al(a.G) && al(a.D) && al(a.r) && al(a.d);
  if (a.h2mode) ok = ok && al(a.bm1);
  if (a.h1mode == 1) ok = ok && al(a.h1);
  if (a.h2mode == 2) ok = ok && al(a.h2);
  return ok;
}

}  // namespace

// ---------------------------------------------------------------------------
struct Batch {
  int device = 0;
  cudaStream_t stream = nullptr;
  std::vector<std::unique_ptr<Handle>> probs;
  std::string err;
  CgScalars* cg_host_all = nullptr;  // pinned, one per problem
  size_t cg_host_cap = 0;
  DevBuf<unsigned char> desc;
  DevBuf<int> map, base;
  cudaGraphExec_t gexec = nullptr;
  std::vector<int64_t> gkey;
  int chunk = 16;
  bool use_graph = true;
  // one cooperative launch per batch segment (batch_persistent_kernel)
  // instead of three graph-replayed launches per iteration.  Off by default:
  // on GB300 the fused kernel holds every phase's registers (one or two
  // blocks per SM), and its memory-bound phases run slower than the separate
  // launches (nekgpu_batch_set_persistent)
  bool persistent = false;
  DevBuf<unsigned int> bar;  // the persistent launch's barrier words
  DevBuf<int> perr;          // and its error flag
  DevBuf<CgScalars> cg_all;  // the problems' scalars gathered after a chunk
  // operator block size per precision ([0] FP64, [1] FP32): picked by
  // batch_tune for the problem set in tkey, or pinned (pinned[prec] != 0)
  int threads[2] = {0, 0};
  int pinned[2] = {0, 0};
  std::vector<int64_t> tkey[2];
  float tune_ms[2] = {0.f, 0.f};
  // FP32 orders (bit lx1) whose operator launch keeps the plain body although
  // the TMA-staged one applies: batch_tune found it faster there.  tma_pick
  // keeps each order's verdict (-1 not timed yet, 0 plain, 1 TMA) for the
  // life of the batch, so that the subsets of problems a mixed solve runs as
  // others converge do not re-decide it on fewer blocks.
  unsigned tma_off = 0u;
  int tma_pick[NEKGPU_MAX_LX1 + 1];
  Batch() { std::fill(tma_pick, tma_pick + NEKGPU_MAX_LX1 + 1, -1); }
};

namespace {

struct BatchLaunch {
  int gridA = 0, gridB = 0, gridC = 0;
  int threadsA = kBatchThreads;  // operator block size
  size_t smem = 0;               // largest operator block's shared memory
  // operator launches, one per order present: lx1, first virtual block,
  // blocks, shared memory per block
  int ngrp = 0;
  int gnx[NEKGPU_MAX_LX1 + 1] = {}, gstart[NEKGPU_MAX_LX1 + 1] = {},
      gcount[NEKGPU_MAX_LX1 + 1] = {}, gtma[NEKGPU_MAX_LX1 + 1] = {};
  size_t gsmem[NEKGPU_MAX_LX1 + 1] = {};
  const void* desc = nullptr;
  const int *mapA, *mapB, *mapC, *baseA, *baseB, *baseC;
};

// Builds descriptors and block maps for the listed problems, uploads them.
template <typename T>
int batch_tables(Batch& B, const std::vector<int>& ids, const std::vector<Coef<T>>& coef,
                 const std::vector<T*>& xs, const std::vector<const T*>& mults,
                 const std::vector<const T*>& binvs, BatchLaunch& L, int threads = 0) {
  if (threads <= 0) threads = B.threads[sizeof(T) == 4 ? 1 : 0];
  if (threads <= 0) threads = kBatchThreads;
  const int np = (int)ids.size();
  std::vector<BDesc<T>> hd(np);
  std::vector<int> mapA, mapB, mapC, baseA(np), baseB(np), baseC(np);
  size_t smem = 0;
  for (int q = 0; q < np; ++q) {
    Handle& h = *B.probs[ids[q]];
    Mesh& m = h.mesh;
    PcgWork<T>& wk = [&]() -> PcgWork<T>& {
      if constexpr (std::is_same<T, double>::value) return h.w64;
      else return h.w32;
    }();
    const OpData<T>& op = [&]() -> const OpData<T>& {
      if constexpr (std::is_same<T, double>::value) return m.f64;
      else return m.f32;
    }();
    BDesc<T>& d = hd[q];
    memset(&d, 0, sizeof(d));
    AxArgs<T>& a = d.ax;
    a.au = wk.w.ptr;
    a.u = wk.p.ptr;
    a.G = op.G;
    a.bm1 = op.bm1;
    a.h1 = coef[q].h1;
    a.h2 = coef[q].h2;
    a.h1s = coef[q].h1s;
    a.h2s = coef[q].h2s;
    a.h1mode = coef[q].h1mode;
    a.h2mode = coef[q].h2mode;
    a.D = op.D;
    a.nel = m.nel;
    a.p = wk.p.ptr;
    a.r = wk.r.ptr;
    a.d = wk.d.ptr;
    a.cg = h.cg;
    a.partial = h.partialA.ptr;
    a.err = m.dev_err;
    a.skip = m.gs.skip;
    d.nx1 = m.nx1;
    d.epb = batch_epb(m.nx1, threads);
    d.nblkA = (m.nel + d.epb - 1) / d.epb;
    d.bstart = m.gs.bstart;
    d.bidx = m.gs.bidx;
    d.cls = m.gs.cls;
    d.segmask = wk.segmask.ptr;
    d.segmsum = wk.segmsum.ptr;
    d.partialB = h.partialB.ptr;
    d.nblkB = gs_cg_blocks(m.gs);
    a.hbm = coef[q].h2mode ? coef[q].hbm : nullptr;
    d.x = xs[q];
    d.mult = mults[q];
    d.binv = binvs[q];
    d.md = wk.md.ptr;
    d.mb = wk.mb.ptr;
    d.n = m.n;
    d.partialC = h.partialC.ptr;
    // FP64: the single solve's block count (the same FP64 sums, so that a
    // batched FP64 problem returns exactly what its solve alone returns);
    // FP32: at least 8 vector steps per thread, so that the small problems'
    // blocks are not mostly reduction
    d.nblkC = std::is_same<T, double>::value
                  ? pcg_vec_blocks(m.n)
                  : (int)std::min<int64_t>(std::max<int64_t>((m.n + 8191) / 8192, 1),
                                           pcg_vec_blocks(m.n));
    auto al = [](const void* p) { return ((uintptr_t)p & 15u) == 0; };
    d.vec = al(d.x) && al(wk.r.ptr) && al(wk.p.ptr) && al(wk.w.ptr) && al(d.md) &&
            al(d.mult) && al(d.mb);
    d.cg = h.cg;
    smem = std::max(smem, batch_smem<T>(m.nx1, d.epb));
    baseB[q] = (int)mapB.size();
    mapB.insert(mapB.end(), d.nblkB, q);
    baseC[q] = (int)mapC.size();
    mapC.insert(mapC.end(), d.nblkC, q);
  }
  // operator blocks grouped by order (ascending lx1, problems in list order
  // inside an order): one launch per group
  // (FP32, an order the TMA-staged body serves, every array aligned and the
  // order not in tma_off: that body, as in a single solve; the persistent
  // form keeps the plain body in every phase)
  L.ngrp = 0;
  for (int nx = 2; nx <= NEKGPU_MAX_LX1; ++nx) {
    bool any = false;
    bool tma = std::is_same<T, float>::value && !B.persistent && tma_lx1(nx) &&
               !((B.tma_off >> nx) & 1u);
    for (int q = 0; q < np; ++q) {
      if (hd[q].nx1 != nx) continue;
      any = true;
      tma = tma && B.probs[ids[q]]->mesh.use_tma && batch_tma_aligned(hd[q].ax);
    }
    if (!any) continue;
    const int g0 = (int)mapA.size();
    size_t gs = 0;
    for (int q = 0; q < np; ++q) {
      BDesc<T>& d = hd[q];
      if (d.nx1 != nx) continue;
      if (tma) {
        d.epb = batch_tma_epb_rt(nx);
        d.nblkA = (d.ax.nel + d.epb - 1) / d.epb;
        gs = std::max(gs, batch_tma_smem(nx, d.ax.h1mode, d.ax.h2mode));
      } else {
        gs = std::max(gs, batch_smem<T>(nx, d.epb));
      }
      baseA[q] = (int)mapA.size();
      mapA.insert(mapA.end(), d.nblkA, q);
    }
    L.gnx[L.ngrp] = nx;
    L.gstart[L.ngrp] = g0;
    L.gcount[L.ngrp] = (int)mapA.size() - g0;
    L.gsmem[L.ngrp] = gs;
    L.gtma[L.ngrp] = tma ? 1 : 0;
    ++L.ngrp;
  }
  const size_t dbytes = sizeof(BDesc<T>) * np;
  const size_t nmap = mapA.size() + mapB.size() + mapC.size();
  if (B.desc.ensure(dbytes) || B.map.ensure(nmap) || B.base.ensure(3 * (size_t)np)) return -4;
  std::vector<int> maps;
  maps.reserve(nmap);
  maps.insert(maps.end(), mapA.begin(), mapA.end());
  maps.insert(maps.end(), mapB.begin(), mapB.end());
  maps.insert(maps.end(), mapC.begin(), mapC.end());
  std::vector<int> bases;
  bases.insert(bases.end(), baseA.begin(), baseA.end());
  bases.insert(bases.end(), baseB.begin(), baseB.end());
  bases.insert(bases.end(), baseC.begin(), baseC.end());
  cudaMemcpyAsync(B.desc.ptr, hd.data(), dbytes, cudaMemcpyHostToDevice, B.stream);
  cudaMemcpyAsync(B.map.ptr, maps.data(), nmap * sizeof(int), cudaMemcpyHostToDevice, B.stream);
  cudaMemcpyAsync(B.base.ptr, bases.data(), bases.size() * sizeof(int), cudaMemcpyHostToDevice,
                  B.stream);
  if (cudaStreamSynchronize(B.stream) != cudaSuccess) return -3;
  L.gridA = (int)mapA.size();
  L.gridB = (int)mapB.size();
  L.gridC = (int)mapC.size();
  L.smem = smem;
  L.threadsA = threads;
  L.desc = B.desc.ptr;
  L.mapA = B.map.ptr;
  L.mapB = B.map.ptr + mapA.size();
  L.mapC = B.map.ptr + mapA.size() + mapB.size();
  L.baseA = B.base.ptr;
  L.baseB = B.base.ptr + np;
  L.baseC = B.base.ptr + 2 * np;
  return 0;
}

// One even order's TMA-staged FP32 operator launch.
template <int NX>
cudaError_t batch_tma_nx(const BDesc<float>* D, const BatchLaunch& L, int g, cudaStream_t s) {
  constexpr int EPB = batch_tma_epb<NX>();
  // room for the largest slice set, per device
  static std::atomic<uint32_t> configured{0};
  if (first_on_device(configured)) {
    cudaError_t e = cudaFuncSetAttribute(batch_axhelm_tma_kernel<NX, EPB>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)tma_smem_bytes<NX, float, EPB>(true, 1, 2));
    if (e != cudaSuccess) return e;
    cudaFuncSetAttribute(batch_axhelm_tma_kernel<NX, EPB>,
                         cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    mark_device(configured);
  }
  batch_axhelm_tma_kernel<NX, EPB><<<L.gcount[g], dim3(NX * NX, EPB), L.gsmem[g], s>>>(
      D, L.mapA, L.baseA, L.gstart[g]);
  return cudaSuccess;
}

// One order's operator launch.
template <typename T, int NX>
cudaError_t batch_ops_nx(const BDesc<T>* D, const BatchLaunch& L, int g, cudaStream_t s) {
  if constexpr (std::is_same<T, float>::value && tma_lx1(NX)) {
    if (L.gtma[g]) return batch_tma_nx<NX>(D, L, g, s);
  }
  static std::atomic<uint32_t> configured{0};  // per device
  if (first_on_device(configured)) {
    cudaError_t e = cudaFuncSetAttribute(batch_axhelm_nx_kernel<T, NX>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)batch_smem<T>(NX, batch_epb(NX, kBatchThreads)));
    if (e != cudaSuccess) return e;
    mark_device(configured);
  }
  batch_axhelm_nx_kernel<T, NX><<<L.gcount[g], L.threadsA, L.gsmem[g], s>>>(D, L.mapA, L.baseA,
                                                                           L.gstart[g]);
  return cudaSuccess;
}

// Operator launch g of a batched iteration (one order's problems).
template <typename T>
cudaError_t batch_op_group(const BatchLaunch& L, int g, cudaStream_t s) {
  const BDesc<T>* D = reinterpret_cast<const BDesc<T>*>(L.desc);
  count_launch();
  switch (L.gnx[g]) {
    case 2: return batch_ops_nx<T, 2>(D, L, g, s);
    case 3: return batch_ops_nx<T, 3>(D, L, g, s);
    case 4: return batch_ops_nx<T, 4>(D, L, g, s);
    case 5: return batch_ops_nx<T, 5>(D, L, g, s);
    case 6: return batch_ops_nx<T, 6>(D, L, g, s);
    case 7: return batch_ops_nx<T, 7>(D, L, g, s);
    case 8: return batch_ops_nx<T, 8>(D, L, g, s);
    case 9: return batch_ops_nx<T, 9>(D, L, g, s);
    case 10: return batch_ops_nx<T, 10>(D, L, g, s);
    case 11: return batch_ops_nx<T, 11>(D, L, g, s);
    default: return batch_ops_nx<T, 12>(D, L, g, s);
  }
}

// The operator of one batched iteration: one launch per order present.
template <typename T>
cudaError_t batch_ops(const BatchLaunch& L, cudaStream_t s) {
  for (int g = 0; g < L.ngrp; ++g) {
    const cudaError_t e = batch_op_group<T>(L, g, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

template <typename T>
cudaError_t batch_enqueue(Batch& B, const BatchLaunch& L, int k) {
  const BDesc<T>* D = reinterpret_cast<const BDesc<T>*>(L.desc);
  for (int q = 0; q < k; ++q) {
    cudaError_t e = batch_ops<T>(L, B.stream);
    if (e != cudaSuccess) return e;
    count_launch(2);
    batch_gs_kernel<T><<<L.gridB, kGsThreads, 0, B.stream>>>(D, L.mapB, L.baseB);
    batch_update_kernel<T, false><<<L.gridC, kBatchThreads, 0, B.stream>>>(D, L.mapC, L.baseC);
  }
  return cudaGetLastError();
}

// FP32: per order, the TMA-staged body or the plain one, whichever times
// faster (the two bodies compute the same numbers).  An order is timed the
// first time it appears in a problem set, in three interleaved rounds of 3
// launches of its operator per body, each body keeping its best round; the
// verdict sticks (Batch::tma_pick).  Sets B.tma_off.
template <typename T>
int batch_tune_tma(Batch& B, const std::vector<int>& ids, const std::vector<Coef<T>>& coef,
                   const std::vector<T*>& xs, const std::vector<const T*>& mults,
                   const std::vector<const T*>& binvs) {
  float t[2][NEKGPU_MAX_LX1 + 1];
  int tma_at[NEKGPU_MAX_LX1 + 1] = {};
  for (int v = 0; v < 2; ++v)
    for (int nx = 0; nx <= NEKGPU_MAX_LX1; ++nx) t[v][nx] = 1e30f;
  bool undecided = false;
  {  // orders present where the TMA body applies and no verdict exists yet
    B.tma_off = 0u;
    BatchLaunch L;
    const int rc = batch_tables<T>(B, ids, coef, xs, mults, binvs, L);
    if (rc) return rc;
    for (int g = 0; g < L.ngrp; ++g) {
      tma_at[L.gnx[g]] = L.gtma[g] && B.tma_pick[L.gnx[g]] < 0;
      undecided = undecided || tma_at[L.gnx[g]];
    }
  }
  if (undecided) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return -3;
    const unsigned masks[2] = {0u, ~0u};  // TMA wherever it applies / nowhere
    for (int round = 0; round < 3; ++round)
      for (int v = 0; v < 2; ++v) {
        B.tma_off = masks[v];
        BatchLaunch L;
        int rc = batch_tables<T>(B, ids, coef, xs, mults, binvs, L);
        cudaError_t e = cudaSuccess;
        for (int g = 0; g < L.ngrp && !rc && e == cudaSuccess; ++g) {
          if (!tma_at[L.gnx[g]]) continue;
          e = batch_op_group<T>(L, g, B.stream);  // warm-up
          cudaEventRecord(e0, B.stream);
          for (int q = 0; q < 3 && e == cudaSuccess; ++q) e = batch_op_group<T>(L, g, B.stream);
          cudaEventRecord(e1, B.stream);
          if (e == cudaSuccess) e = cudaGetLastError();
          float ms = 0.f;
          if (e == cudaSuccess) e = cudaEventSynchronize(e1);
          if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
          t[v][L.gnx[g]] = std::min(t[v][L.gnx[g]], ms);
        }
        if (rc || e != cudaSuccess) {
          cudaEventDestroy(e0);
          cudaEventDestroy(e1);
          B.tma_off = 0u;
          if (!rc) B.err = std::string("batch autotune: ") + cudaGetErrorString(e);
          return rc ? rc : -3;
        }
      }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    for (int nx = 0; nx <= NEKGPU_MAX_LX1; ++nx)
      if (tma_at[nx]) B.tma_pick[nx] = t[1][nx] < t[0][nx] ? 0 : 1;
  }
  unsigned off = 0u;
  for (int nx = 0; nx <= NEKGPU_MAX_LX1; ++nx)
    if (B.tma_pick[nx] == 0) off |= 1u << nx;
  B.tma_off = off;
  return 0;
}

// Picks the operator block size for a problem set: times a batched operator
// launch for every candidate (128 or 256 threads; 128 only when every
// element slab fits) and keeps the fastest, once per problem set and
// precision (a subset of a tuned set keeps its pick).  Runs on freshly prepared problems only (beta = 0, p = 0), where
// the launches it times change nothing the first iteration reads.  Every
// size gives the same results (per-element rho partials).
template <typename T>
int batch_tune(Batch& B, const std::vector<int>& ids, const std::vector<Coef<T>>& coef,
               const std::vector<T*>& xs, const std::vector<const T*>& mults,
               const std::vector<const T*>& binvs) {
  const int prec = sizeof(T) == 4 ? 1 : 0;
  if (B.pinned[prec]) {
    B.threads[prec] = B.pinned[prec];
    return 0;
  }
  if (B.persistent) {  // the persistent launch runs every phase with 256 threads
    B.threads[prec] = kBatchThreads;
    return 0;
  }
  // (problem, coefficient modes), sorted: a set already tuned, or a subset of
  // one (the problems a mixed solve still runs as others converge), keeps
  // the pick
  std::vector<int64_t> key;
  int maxnxy = 0;
  for (size_t q = 0; q < ids.size(); ++q) {
    const Mesh& m = B.probs[ids[q]]->mesh;
    key.push_back((int64_t)ids[q] * 16 + coef[q].h1mode * 4 + coef[q].h2mode);
    maxnxy = std::max(maxnxy, m.nx1 * m.nx1);
  }
  std::sort(key.begin(), key.end());
  if (B.threads[prec] &&
      std::includes(B.tkey[prec].begin(), B.tkey[prec].end(), key.begin(), key.end()))
    return 0;  // (a subset's orders all have their TMA verdicts: tma_off stands)
  std::vector<int> cand;
  for (int t : {128, 256})
    if (t >= maxnxy) cand.push_back(t);
  int best = kBatchThreads;
  float best_ms = 0.f;
  if (cand.size() > 1) {
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) return -3;
    best_ms = 1e30f;
    for (int t : cand) {
      BatchLaunch L;
      int rc = batch_tables<T>(B, ids, coef, xs, mults, binvs, L, t);
      if (rc) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return rc;
      }
      cudaError_t e = batch_ops<T>(L, B.stream);  // warm-up
      cudaEventRecord(e0, B.stream);
      for (int q = 0; q < 3 && e == cudaSuccess; ++q) e = batch_ops<T>(L, B.stream);
      cudaEventRecord(e1, B.stream);
      if (e == cudaSuccess) e = cudaGetLastError();
      float ms = 0.f;
      if (e == cudaSuccess) e = cudaEventSynchronize(e1);
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (e != cudaSuccess) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        B.err = std::string("batch autotune: ") + cudaGetErrorString(e);
        return -3;
      }
      if (ms < best_ms) {
        best_ms = ms;
        best = t;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    best_ms /= 3.f;
  } else if (!cand.empty()) {
    best = cand[0];
  }
  B.threads[prec] = best;
  B.tune_ms[prec] = best_ms;
  if (prec == 1) {
    const int rc = batch_tune_tma<T>(B, ids, coef, xs, mults, binvs);
    if (rc) return rc;
  }
  B.tkey[prec] = key;
  return 0;
}

// The persistent form of batch_iterate's loop (after the iteration-1
// check): cooperative launches of batch_persistent_kernel until every problem
// has stopped.  Returns 0, a negative status, or 1 when the device cannot
// take the cooperative launch (then the three-launch form runs).
template <typename T>
int batch_iterate_persistent(Batch& B, const std::vector<int>& ids, const BatchLaunch& L) {
  const int np = (int)ids.size();
  static std::atomic<uint32_t> configured{0};  // per device
  if (first_on_device(configured)) {
    if (cudaFuncSetAttribute(batch_persistent_kernel<T>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)batch_smem_max<T>()) != cudaSuccess)
      return 1;
    mark_device(configured);
  }
  int dev = 0, coop = 0, nsm = 0, per_sm = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  if (!coop ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_persistent_kernel<T>,
                                                    kBatchThreads, L.smem) != cudaSuccess ||
      per_sm < 1) {
    cudaGetLastError();
    return 1;
  }
  const int grid = std::min(per_sm * nsm, std::max({L.gridA, L.gridB, L.gridC, 1}));
  if (B.bar.ensure(2) || B.perr.ensure(1)) return -4;
  const BDesc<T>* D = reinterpret_cast<const BDesc<T>*>(L.desc);
  int gA = L.gridA, gB = L.gridB, gC = L.gridC, kmax = 1 << 30, npp = np;
  unsigned int* bar = B.bar.ptr;
  int* perr = B.perr.ptr;
  const int *mA = L.mapA, *bA = L.baseA, *mB = L.mapB, *bB = L.baseB, *mC = L.mapC,
            *bC = L.baseC;
  void* args[] = {(void*)&D, &npp, (void*)&mA, (void*)&bA, &gA, (void*)&mB, (void*)&bB, &gB,
                  (void*)&mC, (void*)&bC, &gC, &kmax, (void*)&bar, (void*)&perr};
  if (B.cg_all.ensure(np)) return -4;
  for (;;) {
    count_launch();
    batch_gather_cg_kernel<T><<<(np + 7) / 8, 256, 0, B.stream>>>(D, np, B.cg_all.ptr);
    cudaMemcpyAsync(B.cg_host_all, B.cg_all.ptr, sizeof(CgScalars) * np, cudaMemcpyDeviceToHost,
                    B.stream);
    if (cudaStreamSynchronize(B.stream) != cudaSuccess) {
      B.err = std::string("batch: ") + cudaGetErrorString(cudaGetLastError());
      return -3;
    }
    bool all = true;
    for (int q = 0; q < np; ++q) all = all && B.cg_host_all[q].done;
    if (all) break;  // (one launch runs until every problem has stopped)
    cudaMemsetAsync(bar, 0, 2 * sizeof(unsigned int), B.stream);
    cudaMemsetAsync(perr, 0, sizeof(int), B.stream);
    count_launch();
    cudaError_t e = cudaLaunchCooperativeKernel((const void*)batch_persistent_kernel<T>, grid,
                                                kBatchThreads, args, L.smem, B.stream);
    if (e != cudaSuccess) {
      B.err = std::string("batch persistent launch: ") + cudaGetErrorString(e);
      return -3;
    }
    int herr = 0;
    cudaMemcpyAsync(&herr, perr, sizeof(int), cudaMemcpyDeviceToHost, B.stream);
    if (cudaStreamSynchronize(B.stream) != cudaSuccess) {
      B.err = std::string("batch: ") + cudaGetErrorString(cudaGetLastError());
      return -3;
    }
    if (herr) {
      B.err = "batch persistent launch: a grid barrier wait expired";
      return -3;
    }
  }
  for (int q = 0; q < np; ++q) *B.probs[ids[q]]->cg_host = B.cg_host_all[q];
  return 0;
}

// first: run the iteration-1 check of freshly prepared problems first (not
// after a residual replacement, which sets the scalars itself).
// Runs chunks of batched iterations until every problem has stopped, or with
// `any` until at least one problem that was running on entry has stopped.
template <typename T>
int batch_iterate(Batch& B, const std::vector<int>& ids, const BatchLaunch& L, bool first = true,
                  bool any = false) {
  const int np = (int)ids.size();
  const BDesc<T>* D = reinterpret_cast<const BDesc<T>*>(L.desc);
  if (first) {
    count_launch();
    batch_update_kernel<T, true><<<L.gridC, kBatchThreads, 0, B.stream>>>(D, L.mapC, L.baseC);
  }
  if (B.cg_host_cap < (size_t)np) {
    cudaFreeHost(B.cg_host_all);
    if (cudaMallocHost(&B.cg_host_all, sizeof(CgScalars) * np) != cudaSuccess) return -4;
    B.cg_host_cap = np;
  }
  if (B.persistent && L.threadsA == kBatchThreads) {
    const int rc = batch_iterate_persistent<T>(B, ids, L);
    if (rc != 1) return rc;  // 1: cooperative launch unavailable, the launches below run
  }
  bool graph = B.use_graph;
  std::vector<int64_t> key = {(int64_t)sizeof(T), L.gridA, L.gridB, L.gridC, (int64_t)L.smem,
                              L.threadsA,
                              (int64_t)(uintptr_t)L.desc, (int64_t)(uintptr_t)L.mapA, B.chunk};
  for (int g = 0; g < L.ngrp; ++g)  // the operator launches' shapes are baked into the graph
    key.insert(key.end(), {L.gnx[g], L.gstart[g], L.gcount[g], (int64_t)L.gsmem[g], L.gtma[g]});
  if (graph && (!B.gexec || key != B.gkey)) {
    if (B.gexec) cudaGraphExecDestroy(B.gexec);
    B.gexec = nullptr;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(B.stream, cudaStreamCaptureModeRelaxed);
    capturing() = true;
    if (e == cudaSuccess) e = batch_enqueue<T>(B, L, B.chunk);
    capturing() = false;
    cudaError_t e2 = cudaStreamEndCapture(B.stream, &g);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&B.gexec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      cudaGetLastError();
      B.gexec = nullptr;
      graph = false;
    } else {
      B.gkey = key;
    }
  }
  std::vector<char> running(np, 0);
  if (B.cg_all.ensure(np)) return -4;
  for (int round = 0;; ++round) {
    count_launch();
    batch_gather_cg_kernel<T><<<(np + 7) / 8, 256, 0, B.stream>>>(D, np, B.cg_all.ptr);
    cudaMemcpyAsync(B.cg_host_all, B.cg_all.ptr, sizeof(CgScalars) * np, cudaMemcpyDeviceToHost,
                    B.stream);
    if (cudaStreamSynchronize(B.stream) != cudaSuccess) {
      B.err = std::string("batch: ") + cudaGetErrorString(cudaGetLastError());
      return -3;
    }
    bool all = true, stopped = false;
    for (int q = 0; q < np; ++q) {
      const bool done = B.cg_host_all[q].done != 0;
      all = all && done;
      if (round == 0) running[q] = !done;
      else stopped = stopped || (running[q] && done);
    }
    if (all || (any && stopped)) break;
    cudaError_t e;
    if (graph) {
      count_launch((2LL + L.ngrp) * B.chunk);
      e = cudaGraphLaunch(B.gexec, B.stream);
    } else {
      e = batch_enqueue<T>(B, L, B.chunk);
    }
    if (e != cudaSuccess) {
      B.err = std::string("batch launch: ") + cudaGetErrorString(e);
      return -3;
    }
  }
  for (int q = 0; q < np; ++q) *B.probs[ids[q]]->cg_host = B.cg_host_all[q];
  return 0;
}

// Marks a problem finished (trivial right-hand side) on the device.
void mark_done(Handle& h) {
  CgScalars& c = *h.cg_host;
  memset(&c, 0, sizeof(c));
  c.done = 1;
  cudaMemcpyAsync(h.cg, &c, sizeof(CgScalars), cudaMemcpyHostToDevice, h.stream);
}

}  // namespace

// FP64 batched cggo.  Outputs per problem: niter, rbn0, rbn2, status.
int batch_solve_fp64(Batch& B, int np, double* const* x, const double* const* f,
                     const double* const* h1, const double* const* h2,
                     const double* const* mask, const double* const* mult,
                     const double* const* binv, double tin, int maxiter, int* niter,
                     double* rbn0, double* rbn2, int* status) {
  std::vector<int> ids;
  std::vector<Coef<double>> coef;
  std::vector<double*> xs;
  std::vector<const double*> ms, bs;
  for (int p = 0; p < np; ++p) {
    Handle& h = *B.probs[p];
    h.err.clear();
    Coef<double> c;
    if (detect_coef<double>(h, h1[p], h2[p], h.mesh.n, c)) {
      status[p] = NEKGPU_ECUDA;
      continue;
    }
    bool trivial = false;
    PcgResult r = pcg_prepare<double>(h, h.w64, x[p], f[p], c, mask[p], mult[p], tin, maxiter, 0,
                                      nullptr, &trivial);
    status[p] = r.status ? (r.status == -4 ? NEKGPU_ENOMEM : r.status == -1 ? NEKGPU_EINVAL
                                                                             : NEKGPU_ECUDA)
                         : 0;
    niter[p] = 0;
    rbn0[p] = rbn2[p] = 0.0;
    if (r.status) continue;
    if (trivial) {
      mark_done(h);
      continue;
    }
    if (h.mcor) {
      status[p] = NEKGPU_EINVAL;
      set_error(h, "batch: singular operator (no Dirichlet point and h2 = 0): solve it with "
                   "nekgpu_cggo_dev, which applies cggo's null-space correction");
      mark_done(h);
      continue;
    }
    if (pcg_solve_extras<double>(h, h.mesh.f64, h.w64, mult[p], binv[p], c, false)) {
      status[p] = NEKGPU_ENOMEM;
      continue;
    }
    ids.push_back(p);
    coef.push_back(c);
    xs.push_back(x[p]);
    ms.push_back(mult[p]);
    bs.push_back(binv[p]);
  }
  if (ids.empty()) return 0;
  int rc = batch_tune<double>(B, ids, coef, xs, ms, bs);
  if (rc) return rc;
  BatchLaunch L;
  rc = batch_tables<double>(B, ids, coef, xs, ms, bs, L);
  if (rc) return rc;
  rc = batch_iterate<double>(B, ids, L);
  if (rc) return rc;
  for (int p : ids) {
    const CgScalars& c = *B.probs[p]->cg_host;
    niter[p] = c.niter;
    rbn0[p] = c.rbn0;
    rbn2[p] = c.rbn2;
    status[p] = c.nonfinite ? NEKGPU_ENAN
                            : (!(c.rbn2 <= c.tol) && c.iter > c.maxiter) ? NEKGPU_ENOTCONV : 0;
  }
  return 0;
}

// Mixed batched solve: per-problem FP64 defect correction, the FP32 inner
// PCG of all active problems batched.  mode 1: one FP32 PCG per problem with
// residual replacement (mixed_replace) each time its residual has dropped by
// inner_tol; mode 0: a fresh FP32 PCG per outer step.  niter = total inner
// iterations, nouter = outer steps (FP64 residual evaluations).
int batch_solve_mixed(Batch& B, int np, double* const* x, const double* const* f,
                      const double* const* h1, const double* const* h2,
                      const double* const* mask, const double* const* mult,
                      const double* const* binv, double tin, int maxiter, double inner_tol,
                      int mode, int* niter, int* nouter, double* rbn0, double* rbn2,
                      int* status) {
  constexpr int kMaxOuter = 30;
  std::vector<Coef<double>> c64(np);
  std::vector<Coef<float>> c32(np);
  std::vector<double> rbn(np, 0.0), tol(np, 0.0), scale(np, 1.0);
  std::vector<char> active(np, 0);
  for (int p = 0; p < np; ++p) {
    Handle& h = *B.probs[p];
    Mesh& m = h.mesh;
    const int64_t n = m.n;
    h.err.clear();
    niter[p] = nouter[p] = 0;
    rbn0[p] = rbn2[p] = 0.0;
    status[p] = 0;
    PcgWork<float>& wk = h.w32;
    PcgWork<double>& w64 = h.w64;
    if (ensure_f32(h) || wk.mask.ensure(n) || wk.mult.ensure(n) || wk.binv.ensure(n) ||
        wk.x.ensure(n) || wk.f.ensure(n) || wk.d.ensure(n) || wk.h1.ensure(n) ||
        wk.h2.ensure(n) || w64.r.ensure(n) || w64.w.ensure(n) || w64.d.ensure(n)) {
      status[p] = NEKGPU_ENOMEM;
      continue;
    }
    if (detect_coef<double>(h, h1[p], h2[p], n, c64[p])) {
      status[p] = NEKGPU_ECUDA;
      continue;
    }
    if (c64[p].h2mode == 0) {  // no Dirichlet point and h2 = 0: a null space
      int st0 = 0;
      const double skmin = device_sum(h, 6, mask[p], nullptr, nullptr, n, &st0);
      if (!st0 && skmin > 0.0) {
        status[p] = NEKGPU_EINVAL;
        set_error(h, "batch: singular operator (no Dirichlet point and h2 = 0)");
        continue;
      }
    }
    Coef<float>& c = c32[p];
    c.h1mode = c64[p].h1mode;
    c.h2mode = c64[p].h2mode;
    c.h1s = (float)c64[p].h1s;
    c.h2s = (float)c64[p].h2s;
    if (c.h1mode) {
      cast_to_f32(h, wk.h1.ptr, h1[p], 1.0, n);
      c.h1 = wk.h1.ptr;
    }
    if (c.h2mode == 2) {
      cast_to_f32(h, wk.h2.ptr, h2[p], 1.0, n);
      c.h2 = wk.h2.ptr;
    }
    cast_to_f32(h, wk.mask.ptr, mask[p], 1.0, n);
    cast_to_f32(h, wk.mult.ptr, mult[p], 1.0, n);
    cast_to_f32(h, wk.binv.ptr, binv[p], 1.0, n);
    if (setprec_f64(h, w64.d.ptr, c64[p])) {
      status[p] = NEKGPU_ECUDA;
      continue;
    }
    cast_to_f32(h, wk.d.ptr, w64.d.ptr, 1.0, n);
    cudaMemsetAsync(x[p], 0, n * sizeof(double), h.stream);
    cudaMemcpyAsync(w64.r.ptr, f[p], n * sizeof(double), cudaMemcpyDeviceToDevice, h.stream);
    const double r0 = norm64(h, w64.r.ptr, mult[p], binv[p]);
    if (!(r0 >= 0.0) || !std::isfinite(r0)) {
      status[p] = NEKGPU_ENAN;
      continue;
    }
    rbn0[p] = rbn2[p] = rbn[p] = r0;
    tol[p] = tin < 0 ? std::fabs(tin) * r0 : std::fabs(tin);
    active[p] = r0 > 0.0;
  }
  if (mode == 1) {
    // all problems: one FP32 PCG each, prepared once
    std::vector<int> ids;
    std::vector<Coef<float>> coefs;
    std::vector<float*> xs;
    std::vector<const float*> ms, bs;
    for (int p = 0; p < np; ++p) {
      if (!active[p] || status[p]) continue;
      if (rbn[p] <= tol[p]) {
        active[p] = 0;
        continue;
      }
      Handle& h = *B.probs[p];
      const int64_t n = h.mesh.n;
      int st = 0;
      const double amax = device_absmax<double>(h, h.w64.r.ptr, n, &st);
      if (st || amax == 0.0) {
        active[p] = 0;
        continue;
      }
      scale[p] = std::ldexp(1.0, std::ilogb(amax));
      cast_to_f32(h, h.w32.f.ptr, h.w64.r.ptr, 1.0 / scale[p], n);
      bool trivial = false;
      PcgResult r = pcg_prepare<float>(h, h.w32, h.w32.x.ptr, h.w32.f.ptr, c32[p],
                                       h.w32.mask.ptr, h.w32.mult.ptr, -inner_tol, maxiter, 0,
                                       h.w32.d.ptr, &trivial);
      if (r.status) {
        status[p] = r.status == -1 ? NEKGPU_EINVAL : NEKGPU_ECUDA;
        continue;
      }
      if (trivial) {
        active[p] = 0;
        continue;
      }
      if (pcg_solve_extras<float>(h, h.mesh.f32, h.w32, h.w32.mult.ptr, h.w32.binv.ptr, c32[p],
                                  false)) {
        status[p] = NEKGPU_ENOMEM;
        continue;
      }
      ids.push_back(p);
      coefs.push_back(c32[p]);
      xs.push_back(h.w32.x.ptr);
      ms.push_back(h.w32.mult.ptr);
      bs.push_back(h.w32.binv.ptr);
    }
    if (!ids.empty()) {
      const int rc = batch_tune<float>(B, ids, coefs, xs, ms, bs);
      if (rc) return rc;
    }
    // Each problem gets its FP64 residual and replacement as soon as its own
    // FP32 PCG stops (checked after every chunk), and runs on while the
    // others do; a problem that has converged stays in the tables, its
    // blocks returning at once, until the stopped problems hold a quarter of
    // the tables' points -- then the tables (and the captured chunk) are
    // rebuilt without them.
    bool first = true;
    std::vector<char> live(ids.size(), 1);
    int64_t tab_pts = 0, dead_pts = 0;
    for (int p : ids) tab_pts += B.probs[p]->mesh.n;
    BatchLaunch L;
    bool rebuild = true;
    for (int round = 1; !ids.empty() && round <= 100000; ++round) {
      if (rebuild) {
        const int rc = batch_tables<float>(B, ids, coefs, xs, ms, bs, L);
        if (rc) return rc;
        rebuild = false;
      }
      int rc = batch_iterate<float>(B, ids, L, first, true);
      if (rc) return rc;
      first = false;
      int nlive = 0;
      for (size_t q = 0; q < ids.size(); ++q) {
        if (!live[q]) continue;
        const int p = ids[q];
        Handle& h = *B.probs[p];
        if (!h.cg_host->done) {
          ++nlive;
          continue;
        }
        const int64_t n = h.mesh.n;
        const bool capped = h.cg_host->iter > h.cg_host->maxiter;
        niter[p] = h.cg_host->niter;
        ++nouter[p];
        axpy_f32(h, x[p], h.w32.x.ptr, scale[p], n);
        const double rnew = outer_residual(h, h.w64.r.ptr, f[p], x[p], c64[p], mask[p], mult[p],
                                           binv[p], h.w64.w.ptr);
        bool stop = false;
        if (!(rnew >= 0.0) || !std::isfinite(rnew)) {
          status[p] = NEKGPU_ENAN;
          stop = true;
        } else {
          const bool progress = rnew < rbn[p];
          rbn[p] = rbn2[p] = rnew;
          if (rnew <= tol[p] || capped || !progress) {
            stop = true;
          } else {
            const int rr = mixed_replace(h, scale[p], inner_tol, nullptr);
            if (rr < 0) status[p] = NEKGPU_ECUDA;
            stop = rr != 0;
          }
        }
        if (stop) {
          live[q] = 0;
          dead_pts += n;
        } else {
          ++nlive;
        }
      }
      if (nlive == 0) break;
      if (4 * dead_pts > tab_pts) {
        std::vector<int> keep;
        std::vector<Coef<float>> kc;
        std::vector<float*> kx;
        std::vector<const float*> km, kb;
        for (size_t q = 0; q < ids.size(); ++q) {
          if (!live[q]) continue;
          keep.push_back(ids[q]);
          kc.push_back(coefs[q]);
          kx.push_back(xs[q]);
          km.push_back(ms[q]);
          kb.push_back(bs[q]);
        }
        ids.swap(keep);
        coefs.swap(kc);
        xs.swap(kx);
        ms.swap(km);
        bs.swap(kb);
        live.assign(ids.size(), 1);
        tab_pts -= dead_pts;
        dead_pts = 0;
        rebuild = true;
      }
    }
  }
  for (int outer = 1; mode != 1 && outer <= kMaxOuter; ++outer) {
    std::vector<int> ids;
    std::vector<Coef<float>> coefs;
    std::vector<float*> xs;
    std::vector<const float*> ms, bs;
    for (int p = 0; p < np; ++p) {
      if (!active[p] || status[p]) continue;
      if (rbn[p] <= tol[p]) {
        active[p] = 0;
        continue;
      }
      Handle& h = *B.probs[p];
      const int64_t n = h.mesh.n;
      int st = 0;
      const double amax = device_absmax<double>(h, h.w64.r.ptr, n, &st);
      if (st || amax == 0.0) {
        active[p] = 0;
        continue;
      }
      scale[p] = std::ldexp(1.0, std::ilogb(amax));
      cast_to_f32(h, h.w32.f.ptr, h.w64.r.ptr, 1.0 / scale[p], n);
      bool trivial = false;
      PcgResult r = pcg_prepare<float>(h, h.w32, h.w32.x.ptr, h.w32.f.ptr, c32[p],
                                       h.w32.mask.ptr, h.w32.mult.ptr, -inner_tol, maxiter, 0,
                                       h.w32.d.ptr, &trivial);
      if (r.status) {
        status[p] = r.status == -1 ? NEKGPU_EINVAL : NEKGPU_ECUDA;
        continue;
      }
      if (trivial) {
        active[p] = 0;
        continue;
      }
      if (pcg_solve_extras<float>(h, h.mesh.f32, h.w32, h.w32.mult.ptr, h.w32.binv.ptr, c32[p],
                                  false)) {
        status[p] = NEKGPU_ENOMEM;
        continue;
      }
      ids.push_back(p);
      coefs.push_back(c32[p]);
      xs.push_back(h.w32.x.ptr);
      ms.push_back(h.w32.mult.ptr);
      bs.push_back(h.w32.binv.ptr);
    }
    if (ids.empty()) break;
    if (outer == 1) {
      const int rc = batch_tune<float>(B, ids, coefs, xs, ms, bs);
      if (rc) return rc;
    }
    BatchLaunch L;
    int rc = batch_tables<float>(B, ids, coefs, xs, ms, bs, L);
    if (rc) return rc;
    rc = batch_iterate<float>(B, ids, L);
    if (rc) return rc;
    for (int p : ids) {
      Handle& h = *B.probs[p];
      const int64_t n = h.mesh.n;
      niter[p] += h.cg_host->niter;
      nouter[p] = outer;
      axpy_f32(h, x[p], h.w32.x.ptr, scale[p], n);
      const double rnew = outer_residual(h, h.w64.r.ptr, f[p], x[p], c64[p], mask[p], mult[p],
                                         binv[p], h.w64.w.ptr);
      if (!(rnew >= 0.0) || !std::isfinite(rnew)) {
        status[p] = NEKGPU_ENAN;
        continue;
      }
      if (rnew >= rbn[p]) active[p] = 0;  // no progress
      rbn[p] = rbn2[p] = rnew;
    }
  }
  for (int p = 0; p < np; ++p)
    if (!status[p] && rbn0[p] > 0.0 && !(rbn[p] <= tol[p])) status[p] = NEKGPU_ENOTCONV;
  return 0;
}

}  // namespace nekgpu

// ---------------------------------------------------------------------------
// C ABI
using nekgpu::Batch;

namespace {
std::mutex g_bmu;
std::map<int64_t, std::unique_ptr<Batch>> g_batches;
int64_t g_bnext = 1;
thread_local std::string g_berr;

Batch* bget(const int64_t* b) {
  if (!b) return nullptr;
  std::lock_guard<std::mutex> lk(g_bmu);
  auto it = g_batches.find(*b);
  return it == g_batches.end() ? nullptr : it->second.get();
}
int bfail(Batch* B, int code, const std::string& msg) {
  if (B) B->err = msg;
  else g_berr = msg;
  return code;
}
}  // namespace

extern "C" {

int nekgpu_batch_create(const int* device, int64_t* batch) {
  if (!device || !batch) return bfail(nullptr, NEKGPU_EINVAL, "null argument");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return bfail(nullptr, NEKGPU_ECUDA, "no CUDA device");
  if (*device < 0 || *device >= ndev) return bfail(nullptr, NEKGPU_EINVAL, "device out of range");
  auto B = std::make_unique<Batch>();
  B->device = *device;
  cudaSetDevice(B->device);
  if (cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bfail(nullptr, NEKGPU_ECUDA, "stream creation failed");
  std::lock_guard<std::mutex> lk(g_bmu);
  *batch = g_bnext++;
  g_batches[*batch] = std::move(B);
  return NEKGPU_OK;
}

int nekgpu_batch_add(const int64_t* batch, const int* lx1, const int* nel, const double* dxm1,
                     const double* g1, const double* g2, const double* g3, const double* g4,
                     const double* g5, const double* g6, const double* bm1,
                     const int64_t* glo_num, int* index) {
  Batch* B = bget(batch);
  if (!B) return bfail(nullptr, NEKGPU_EHANDLE, "unknown batch");
  if (!lx1 || !nel || !dxm1 || !g1 || !g2 || !g3 || !g4 || !g5 || !g6 || !bm1 || !glo_num)
    return bfail(B, NEKGPU_EINVAL, "null argument");
  cudaSetDevice(B->device);
  auto H = std::make_unique<nekgpu::Handle>();
  H->autotune = false;  // the batched operator launches its own shape
  std::string err;
  if (nekgpu::handle_open(*H, B->device, B->stream, err)) return bfail(B, NEKGPU_ECUDA, err);
  const double* g[6] = {g1, g2, g3, g4, g5, g6};
  const int rc = nekgpu::handle_setup(*H, *lx1, *nel, dxm1, g, bm1, glo_num, err);
  if (rc) {
    nekgpu::handle_close(*H);
    return bfail(B, rc, err);
  }
  B->probs.push_back(std::move(H));
  if (index) *index = (int)B->probs.size() - 1;
  return NEKGPU_OK;
}

int nekgpu_batch_solve_dev(const int64_t* batch, const int* nprob, double* const* x,
                           const double* const* f, const double* const* h1,
                           const double* const* h2, const double* const* mask,
                           const double* const* mult, const double* const* binv,
                           const double* tin, const int* maxit, const int* mixed,
                           const double* inner_tol, int* niter, int* nouter, double* rbn0,
                           double* rbn2, int* status) {
  Batch* B = bget(batch);
  if (!B) return bfail(nullptr, NEKGPU_EHANDLE, "unknown batch");
  if (!nprob || !x || !f || !h1 || !h2 || !mask || !mult || !binv || !tin || !maxit || !niter ||
      !rbn0 || !rbn2 || !status)
    return bfail(B, NEKGPU_EINVAL, "null argument");
  const int np = *nprob;
  if (np != (int)B->probs.size())
    return bfail(B, NEKGPU_EINVAL, "nprob differs from the number of problems added");
  for (int p = 0; p < np; ++p)
    if (!x[p] || !f[p] || !h1[p] || !h2[p] || !mask[p] || !mult[p] || !binv[p])
      return bfail(B, NEKGPU_EINVAL, "null array for problem " + std::to_string(p));
  cudaSetDevice(B->device);
  B->err.clear();
  // The problems' handles share the batch's stream: waiting once makes the
  // batch's kernels start after the caller's queued work (handle_enter).
  if (np > 0 && nekgpu::handle_enter(*B->probs[0]) != cudaSuccess)
    return bfail(B, NEKGPU_ECUDA, "call entry failed");
  int rc;
  if (mixed && *mixed) {
    if (*mixed != 1 && *mixed != 2) return bfail(B, NEKGPU_EINVAL, "mixed must be 0, 1 or 2");
    const int mode = *mixed == 1 ? 1 : 0;
    const double itol = inner_tol ? *inner_tol : (mode == 1 ? 1e-2 : 1e-5);
    if (!(itol > 0.0 && itol < 1.0)) return bfail(B, NEKGPU_EINVAL, "inner_tol must be in (0, 1)");
    std::vector<int> no(np, 0);
    rc = nekgpu::batch_solve_mixed(*B, np, x, f, h1, h2, mask, mult, binv, *tin, *maxit, itol,
                                   mode, niter, no.data(), rbn0, rbn2, status);
    if (nouter)
      for (int p = 0; p < np; ++p) nouter[p] = no[p];
  } else {
    rc = nekgpu::batch_solve_fp64(*B, np, x, f, h1, h2, mask, mult, binv, *tin, *maxit, niter,
                                  rbn0, rbn2, status);
    if (nouter)
      for (int p = 0; p < np; ++p) nouter[p] = 0;
  }
  const cudaError_t le = cudaStreamSynchronize(B->stream);  // finished before the call returns
  if (rc) return bfail(B, rc == -4 ? NEKGPU_ENOMEM : NEKGPU_ECUDA,
                       B->err.empty() ? "batch solve failed" : B->err);
  if (le != cudaSuccess) return bfail(B, NEKGPU_ECUDA, std::string("batch solve: ") + cudaGetErrorString(le));
  for (int p = 0; p < np; ++p)
    if (status[p] && status[p] != NEKGPU_ENOTCONV && B->err.empty())
      B->err = "problem " + std::to_string(p) + ": " + B->probs[p]->err;
  return NEKGPU_OK;
}

int nekgpu_batch_shape(const int64_t* batch, const int* precision, int* threads, double* ms) {
  Batch* B = bget(batch);
  if (!B) return bfail(nullptr, NEKGPU_EHANDLE, "unknown batch");
  if (!precision || (*precision != 0 && *precision != 1))
    return bfail(B, NEKGPU_EINVAL, "precision must be 0 or 1");
  if (threads) *threads = B->threads[*precision];
  if (ms) *ms = B->tune_ms[*precision];
  return NEKGPU_OK;
}

int nekgpu_batch_operator_forms(const int64_t* batch, int* forms) {
  Batch* B = bget(batch);
  if (!B) return bfail(nullptr, NEKGPU_EHANDLE, "unknown batch");
  if (!forms) return bfail(B, NEKGPU_EINVAL, "null argument");
  for (int nx = 0; nx <= NEKGPU_MAX_LX1; ++nx) forms[nx] = B->tma_pick[nx];
  return NEKGPU_OK;
}

int nekgpu_batch_set_shape(const int64_t* batch, const int* precision, const int* threads) {
  Batch* B = bget(batch);
  if (!B) return bfail(nullptr, NEKGPU_EHANDLE, "unknown batch");
  if (!precision || !threads || (*precision != 0 && *precision != 1))
    return bfail(B, NEKGPU_EINVAL, "bad argument");
  if (*threads != 0 && *threads != 128 && *threads != 256)
    return bfail(B, NEKGPU_EINVAL, "threads must be 0 (autotune), 128 or 256");
  B->pinned[*precision] = *threads;
  B->threads[*precision] = 0;
  B->tkey[*precision].clear();
  return NEKGPU_OK;
}

int nekgpu_batch_set_persistent(const int64_t* batch, const int* on) {
  Batch* B = bget(batch);
  if (!B) return bfail(nullptr, NEKGPU_EHANDLE, "unknown batch");
  if (!on) return bfail(B, NEKGPU_EINVAL, "null argument");
  B->persistent = (*on != 0);
  return NEKGPU_OK;
}

int nekgpu_batch_last_error(const int64_t* batch, char* buf, const int* buflen) {
  if (!buf || !buflen || *buflen <= 0) return NEKGPU_EINVAL;
  Batch* B = bget(batch);
  const std::string& m = B ? B->err : g_berr;
  const size_t k = std::min<size_t>(m.size(), (size_t)*buflen - 1);
  std::memcpy(buf, m.data(), k);
  buf[k] = '\0';
  return NEKGPU_OK;
}

int nekgpu_batch_destroy(int64_t* batch) {
  Batch* B = bget(batch);
  if (!B) return bfail(nullptr, NEKGPU_EHANDLE, "unknown batch");
  cudaSetDevice(B->device);
  cudaStreamSynchronize(B->stream);
  for (auto& h : B->probs) nekgpu::handle_close(*h);
  B->probs.clear();
  if (B->gexec) cudaGraphExecDestroy(B->gexec);
  cudaFreeHost(B->cg_host_all);
  B->desc.release();
  B->map.release();
  B->base.release();
  cudaStreamDestroy(B->stream);
  std::lock_guard<std::mutex> lk(g_bmu);
  g_batches.erase(*batch);
  *batch = 0;
  return NEKGPU_OK;
}

}  // extern "C"
