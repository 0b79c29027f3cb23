// tune.cu -- autotuner for the operator's launch shape.
//
// The fastest way to cut an element-major field into thread blocks depends
// on lx1, the precision, the coefficient modes and the mesh size: how many
// elements one block owns trades shared memory (and so blocks per SM)
// against barrier and tail costs, and for FP32 the TMA-staged kernel
// competes with the plain-load one.  On the first solve of a mesh in a
// precision, tune_operator times every candidate shape of the fused PCG
// operator on that mesh (CUDA events on the handle's stream, zeroed work
// vectors as operands) and keeps the fastest.  The candidates are timed in
// kRounds interleaved sweeps and each keeps its best sweep, so a clock that
// is still ramping up, or another process's burst, during one sweep does not
// decide the pick.  Every shape computes the same
// numbers -- pointwise results do not depend on the block a point lands in,
// and the rho partials are per element -- so the pick changes speed only.
// A process-wide cache keyed by device, lx1, nel, precision and coefficient
// modes lets later meshes of the same kind reuse a pick without timing.
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "axhelm_launch.cuh"
#include "impl.cuh"

namespace nekgpu {

std::vector<int> tma_candidates(int nx);  // axhelm_tma.cu

std::vector<AxShapeSel> ax_candidates(int nx, int prec, bool tma) {
  std::vector<AxShapeSel> v;
  const int emax = axhelm_epb(nx);
  for (int e = 1; e <= emax; e *= 2) {
    AxShapeSel s;
    s.kind = 0;
    s.epb = e;
    v.push_back(s);
  }
  if (v.back().epb != emax) {
    AxShapeSel s;
    s.kind = 0;
    s.epb = emax;
    v.push_back(s);
  }
  if (prec == 1 && tma && tma_lx1(nx))
    for (int e : tma_candidates(nx)) {
      AxShapeSel s;
      s.kind = 1;
      s.epb = e;
      v.push_back(s);
    }
  return v;
}

int tma_default_epb(int nx);  // axhelm_tma.cu

AxShapeSel ax_shape_in_use(const Mesh& m, int prec) {
  AxShapeSel sh = prec ? ax_shape<float>(m) : ax_shape<double>(m);
  if (sh.kind == 1 && sh.epb == 0) sh.epb = tma_default_epb(m.nx1);
  return sh;
}

namespace {

using Key = std::tuple<int, int, int, int, int, int, int>;  // dev, nx, nel, prec, h1m, h2m, form
std::mutex g_mu;
std::map<Key, AxShapeSel> g_cache;
std::map<Key, std::pair<int, int>> g_gs_cache;  // boundary-group kernel (threads, gshift)

constexpr int kWarm = 2, kReps = 5, kRounds = 3;

}  // namespace

template <typename T>
int tune_gs(Handle& h, PcgWork<T>& wk);

template <typename T>
int tune_operator(Handle& h, const OpData<T>& op, PcgWork<T>& wk, const Coef<T>& c) {
  Mesh& m = h.mesh;
  const int prec = sizeof(T) == 4 ? 1 : 0;
  if (!h.autotune || m.ax_sel[prec].kind >= 0) return 0;
  // FP32 launches depend on the TMA option, FP64 ones on the double-float one
  const int form = prec ? (int)m.use_tma : (int)(m.use_df && m.has_df);
  const Key key{h.device, m.nx1, m.nel, prec, c.h1mode, c.h2mode, form};
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_cache.find(key);
    if (it != g_cache.end()) {
      m.ax_sel[prec] = it->second;
      auto gt = g_gs_cache.find(key);
      if (gt != g_gs_cache.end()) {
        m.gs.cls_tuned[prec] = gs_shape(m.gs.cls, gt->second.first, gt->second.second);
        m.gs_gshift[prec] = gt->second.second;
      }
      return 0;
    }
  }
  const int64_t n = m.n;
  cudaStream_t s = h.stream;
  if (wk.r.ensure(n) || wk.w.ensure(n) || wk.p.ensure(n) || h.partialA.ensure(m.nel) ||
      h.cg_tune.ensure(1)) {
    set_error(h, "autotune: device allocation failed");
    return -4;
  }
  cudaMemsetAsync(wk.r.ptr, 0, n * sizeof(T), s);
  cudaMemsetAsync(wk.p.ptr, 0, n * sizeof(T), s);
  CgScalars z;
  memset(&z, 0, sizeof(z));  // beta = 0, done = 0
  cudaMemcpyAsync(h.cg_tune.ptr, &z, sizeof(z), cudaMemcpyHostToDevice, s);
  const bool aligned = ((uintptr_t)wk.r.ptr & 15u) == 0 && ((uintptr_t)wk.p.ptr & 15u) == 0;
  const std::vector<AxShapeSel> cand = ax_candidates(m.nx1, prec, m.use_tma && aligned);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    set_error(h, "autotune: cudaEventCreate failed");
    return -3;
  }
  std::vector<float> tbest(cand.size(), 1e30f);
  std::vector<char> usable(cand.size(), 1);
  for (int round = 0; round < kRounds; ++round)
    for (size_t ci = 0; ci < cand.size(); ++ci) {
      if (!usable[ci]) continue;
      m.ax_sel[prec] = cand[ci];
      auto launch = [&]() {
        int np = 0;
        // d = r (zero): the operands' values do not change the launch's cost
        return launch_axhelm_cg<T, false>(m, op, wk.w.ptr, wk.p.ptr, wk.r.ptr, wk.r.ptr, c,
                                          h.cg_tune.ptr, h.partialA.ptr, &np, s);
      };
      cudaError_t e = cudaSuccess;
      for (int q = 0; q < kWarm && e == cudaSuccess; ++q) e = launch();
      cudaEventRecord(e0, s);
      for (int q = 0; q < kReps && e == cudaSuccess; ++q) e = launch();
      cudaEventRecord(e1, s);
      if (e != cudaSuccess) {  // a shape this device cannot launch: skip it
        cudaGetLastError();
        cudaStreamSynchronize(s);
        usable[ci] = 0;
        continue;
      }
      float ms = 0.f;
      if (cudaEventSynchronize(e1) != cudaSuccess ||
          cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        m.ax_sel[prec] = AxShapeSel();
        set_error(h, std::string("autotune: ") + cudaGetErrorString(cudaGetLastError()));
        return -3;
      }
      tbest[ci] = std::min(tbest[ci], ms / kReps);
    }
  AxShapeSel best;
  best.ms = 1e30f;
  for (size_t ci = 0; ci < cand.size(); ++ci)
    if (usable[ci] && tbest[ci] < best.ms) {
      best = cand[ci];
      best.ms = tbest[ci];
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (best.kind < 0) {
    m.ax_sel[prec] = AxShapeSel();
    set_error(h, "autotune: no launch shape could run");
    return -3;
  }
  m.ax_sel[prec] = best;
  const int gst = tune_gs<T>(h, wk);
  if (gst) return gst;
  std::lock_guard<std::mutex> lk(g_mu);
  g_cache[key] = best;
  if (prec == 1) g_gs_cache[key] = {m.gs.cls_tuned[prec].threads, m.gs_gshift[prec]};
  return 0;
}

// The boundary-group kernel's shape: threads per block and groups per thread
// (times 2^gshift of the defaults), timed like the operator's on zeroed data.
// Every shape computes the same sums in the same order per group; the rho
// partials it adds are per block, so the FP64 rho (boundary part) can change
// in its last bits with the shape -- the FP64 shape is therefore left at the
// default, and only the FP32 inner solve (whose rho comes from the operator)
// is tuned.
template <typename T>
int tune_gs(Handle& h, PcgWork<T>& wk) {
  Mesh& m = h.mesh;
  const int prec = sizeof(T) == 4 ? 1 : 0;
  if (prec == 0) return 0;
  const int64_t n = m.n;
  cudaStream_t s = h.stream;
  if (wk.w.ensure(n) || wk.p.ensure(n) || wk.segmask.ensure(m.gs.nbseg) ||
      wk.segmsum.ensure(m.gs.nbseg) || h.partialA.ensure(m.nel) || h.cg_tune.ensure(1)) {
    set_error(h, "autotune: device allocation failed");
    return -4;
  }
  cudaMemsetAsync(wk.w.ptr, 0, n * sizeof(T), s);
  cudaMemsetAsync(wk.p.ptr, 0, n * sizeof(T), s);
  if (m.gs.nbseg) {
    cudaMemsetAsync(wk.segmask.ptr, 0, m.gs.nbseg * sizeof(T), s);
    cudaMemsetAsync(wk.segmsum.ptr, 0, m.gs.nbseg * sizeof(T), s);
  }
  cudaMemsetAsync(h.partialA.ptr, 0, m.nel * sizeof(double), s);
  CgScalars z;
  memset(&z, 0, sizeof(z));
  cudaMemcpyAsync(h.cg_tune.ptr, &z, sizeof(z), cudaMemcpyHostToDevice, s);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    set_error(h, "autotune: cudaEventCreate failed");
    return -3;
  }
  std::vector<std::pair<int, int>> shapes;
  for (int threads : {128, 256, 512})
    for (int gshift : {-1, 0, 1}) shapes.emplace_back(threads, gshift);
  std::vector<float> tbest(shapes.size(), 1e30f);
  for (int round = 0; round < kRounds; ++round)
    for (size_t si = 0; si < shapes.size(); ++si) {
      const GsClasses c = gs_shape(m.gs.cls, shapes[si].first, shapes[si].second);
      if (h.partialB.ensure(gs_cg_blocks(c))) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        set_error(h, "autotune: device allocation failed");
        return -4;
      }
      auto launch = [&]() {
        gs_cg<T>(m.gs, wk.w.ptr, wk.p.ptr, wk.segmask.ptr, wk.segmsum.ptr, h.cg_tune.ptr,
                 h.partialA.ptr, m.nel, h.partialB.ptr, s, false, &c);
      };
      for (int q = 0; q < kWarm; ++q) launch();
      cudaEventRecord(e0, s);
      for (int q = 0; q < kReps; ++q) launch();
      cudaEventRecord(e1, s);
      float ms = 0.f;
      cudaError_t e = cudaEventSynchronize(e1);
      if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
      if (e != cudaSuccess) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        set_error(h, std::string("autotune: ") + cudaGetErrorString(e));
        return -3;
      }
      tbest[si] = std::min(tbest[si], ms / kReps);
    }
  float best = 1e30f;
  GsClasses bestc = m.gs.cls;
  int bestg = 0;
  for (size_t si = 0; si < shapes.size(); ++si)
    if (tbest[si] < best) {
      best = tbest[si];
      bestc = gs_shape(m.gs.cls, shapes[si].first, shapes[si].second);
      bestg = shapes[si].second;
    }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  m.gs.cls_tuned[prec] = bestc;
  m.gs_gshift[prec] = bestg;
  m.gs_ms[prec] = best;
  return 0;
}

template int tune_operator<double>(Handle&, const OpData<double>&, PcgWork<double>&,
                                   const Coef<double>&);
template int tune_operator<float>(Handle&, const OpData<float>&, PcgWork<float>&,
                                  const Coef<float>&);

}  // namespace nekgpu
