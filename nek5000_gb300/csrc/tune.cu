// tune.cu -- autotuner for the operator's launch shape.
//
// The fastest way to cut an element-major field into thread blocks depends
// on lx1, the precision, the coefficient modes and the mesh size: how many
// elements one block owns trades shared memory (and so blocks per SM)
// against barrier and tail costs, and for FP32 the TMA-staged kernel
// competes with the plain-load one.  On the first solve of a mesh in a
// precision, tune_operator times every candidate shape of the fused PCG
// operator on that mesh (CUDA events on the handle's stream, zeroed work
// vectors as operands) and keeps the fastest.  Every shape computes the same
// numbers -- pointwise results do not depend on the block a point lands in,
// and the rho partials are per element -- so the pick changes speed only.
// A process-wide cache keyed by device, lx1, nel, precision and coefficient
// modes lets later meshes of the same kind reuse a pick without timing.
#include <map>
#include <mutex>
#include <tuple>

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
  if (prec == 1 && tma && nx % 2 == 0)
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

using Key = std::tuple<int, int, int, int, int, int, int>;  // dev, nx, nel, prec, h1m, h2m, tma
std::mutex g_mu;
std::map<Key, AxShapeSel> g_cache;

constexpr int kWarm = 2, kReps = 5;

}  // namespace

template <typename T>
int tune_operator(Handle& h, const OpData<T>& op, PcgWork<T>& wk, const Coef<T>& c) {
  Mesh& m = h.mesh;
  const int prec = sizeof(T) == 4 ? 1 : 0;
  if (!h.autotune || m.ax_sel[prec].kind >= 0) return 0;
  const Key key{h.device, m.nx1, m.nel, prec, c.h1mode, c.h2mode, (int)m.use_tma};
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_cache.find(key);
    if (it != g_cache.end()) {
      m.ax_sel[prec] = it->second;
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
  AxShapeSel best;
  best.ms = 1e30f;
  for (const AxShapeSel& sh : cand) {
    m.ax_sel[prec] = sh;
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
      continue;
    }
    float ms = 0.f;
    if (cudaEventSynchronize(e1) != cudaSuccess || cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess) {
      cudaEventDestroy(e0);
      cudaEventDestroy(e1);
      m.ax_sel[prec] = AxShapeSel();
      set_error(h, std::string("autotune: ") + cudaGetErrorString(cudaGetLastError()));
      return -3;
    }
    ms /= kReps;
    if (ms < best.ms) {
      best = sh;
      best.ms = ms;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (best.kind < 0) {
    m.ax_sel[prec] = AxShapeSel();
    set_error(h, "autotune: no launch shape could run");
    return -3;
  }
  m.ax_sel[prec] = best;
  std::lock_guard<std::mutex> lk(g_mu);
  g_cache[key] = best;
  return 0;
}

template int tune_operator<double>(Handle&, const OpData<double>&, PcgWork<double>&,
                                   const Coef<double>&);
template int tune_operator<float>(Handle&, const OpData<float>&, PcgWork<float>&,
                                  const Coef<float>&);

}  // namespace nekgpu
