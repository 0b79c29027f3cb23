// axhelm_launch.cuh -- runtime dispatch of the operator over lx1 and the
// launch shape (kernel kind, elements per block).  Included by one
// translation unit per precision so the instantiations compile in parallel;
// the TMA-staged FP32 kernels live in axhelm_tma.cu.
#pragma once
#include "axhelm.cuh"
#include "impl.cuh"

namespace nekgpu {

// TMA-staged FP32 operator (axhelm_tma.cu): lx1 even, 16-byte aligned arrays;
// epb one of tma_epb_cand<lx1> (0: the built-in count).  Writes one rho
// partial per element when fused.
cudaError_t launch_tma_f32(const Mesh& m, const AxArgs<float>& a, bool fused, int epb,
                           int* nparts, cudaStream_t s);

template <int NX, typename T, bool EXACT, bool FUSED>
static cudaError_t launch_ax_nx(const Mesh& m, const AxArgs<T>& a, int epb, int* nparts,
                                cudaStream_t s) {
  if (epb < 1 || epb * NX * NX > 256) epb = axhelm_epb(NX);
  const size_t smem = axhelm_smem_bytes<NX, T>(epb);
  // per instantiation and device: room for the largest shape
  static std::atomic<uint32_t> configured{0};
  if (first_on_device(configured)) {
    cudaError_t e = cudaFuncSetAttribute(axhelm_kernel<NX, T, EXACT, FUSED>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)axhelm_smem_bytes<NX, T>(axhelm_epb(NX)));
    if (e != cudaSuccess) return e;
    mark_device(configured);
  }
  const int nb = (m.nel + epb - 1) / epb;
  if (nparts) *nparts = m.nel;
  dim3 block(NX * NX, epb);
  count_launch();
  axhelm_kernel<NX, T, EXACT, FUSED><<<nb, block, smem, s>>>(a);
  return cudaGetLastError();
}

inline bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

template <typename T, bool FUSED>
static bool tma_ok(const AxArgs<T>& a) {
  bool ok = aligned16(a.u) && aligned16(a.G) && aligned16(a.D);
  if (a.h2mode) ok = ok && aligned16(a.bm1);
  if (a.h1mode == 1) ok = ok && aligned16(a.h1);
  if (a.h2mode == 2) ok = ok && aligned16(a.h2);
  if (FUSED) ok = ok && aligned16(a.r) && aligned16(a.d);
  return ok;
}

// The launch shape in use for precision T: the autotuner's pick once it has
// run for this mesh, else the built-in one (TMA for FP32 where it applies).
template <typename T>
inline AxShapeSel ax_shape(const Mesh& m) {
  const AxShapeSel& sel = m.ax_sel[sizeof(T) == 4 ? 1 : 0];
  if (sel.kind >= 0) return sel;
  AxShapeSel d;
  d.kind = (sizeof(T) == 4 && m.use_tma && m.nx1 % 2 == 0) ? 1 : 0;
  d.epb = d.kind ? 0 : axhelm_epb(m.nx1);  // 0: the TMA kernel's built-in count
  return d;
}

template <typename T, bool EXACT, bool FUSED>
static cudaError_t launch_ax(const Mesh& m, const AxArgs<T>& a, int* nparts, cudaStream_t s) {
  const AxShapeSel sh = ax_shape<T>(m);
  if constexpr (!EXACT && sizeof(T) == 4) {
    // FP64 is bound by the FP64 pipe, where the plain-load kernel (D in
    // shared memory, higher occupancy) is faster; the TMA form serves FP32.
    if (sh.kind == 1 && m.use_tma && tma_lx1(m.nx1) && tma_ok<T, FUSED>(a))
      return launch_tma_f32(m, a, FUSED, sh.epb, nparts, s);
  }
  const int epb = sh.kind == 0 ? sh.epb : axhelm_epb(m.nx1);
  if constexpr (!EXACT && sizeof(T) == 8) {
    // NEKGPU_OPT_DF: contractions in double-float arithmetic on the FP32 pipe
    if (m.use_df && m.has_df) return launch_axhelm_df(m, a, FUSED, epb, nparts, s);
  }
  switch (m.nx1) {
    case 2: return launch_ax_nx<2, T, EXACT, FUSED>(m, a, epb, nparts, s);
    case 3: return launch_ax_nx<3, T, EXACT, FUSED>(m, a, epb, nparts, s);
    case 4: return launch_ax_nx<4, T, EXACT, FUSED>(m, a, epb, nparts, s);
    case 5: return launch_ax_nx<5, T, EXACT, FUSED>(m, a, epb, nparts, s);
    case 6: return launch_ax_nx<6, T, EXACT, FUSED>(m, a, epb, nparts, s);
    case 7: return launch_ax_nx<7, T, EXACT, FUSED>(m, a, epb, nparts, s);
    case 8: return launch_ax_nx<8, T, EXACT, FUSED>(m, a, epb, nparts, s);
    case 9: return launch_ax_nx<9, T, EXACT, FUSED>(m, a, epb, nparts, s);
    case 10: return launch_ax_nx<10, T, EXACT, FUSED>(m, a, epb, nparts, s);
    case 11: return launch_ax_nx<11, T, EXACT, FUSED>(m, a, epb, nparts, s);
    case 12: return launch_ax_nx<12, T, EXACT, FUSED>(m, a, epb, nparts, s);
    default: return cudaErrorInvalidValue;
  }
}

template <typename T>
static AxArgs<T> make_args(const Mesh& m, const OpData<T>& op, T* au, const T* u,
                           const Coef<T>& c) {
  AxArgs<T> a{};
  a.au = au;
  a.u = u;
  a.G = op.G;
  a.bm1 = op.bm1;
  a.h1 = c.h1;
  a.h2 = c.h2;
  a.h1s = c.h1s;
  a.h2s = c.h2s;
  a.h1mode = c.h1mode;
  a.h2mode = c.h2mode;
  a.hbm = c.h2mode ? c.hbm : nullptr;
  a.D = op.D;
  a.nel = m.nel;
  a.err = m.dev_err;
  a.skip = m.gs.skip;
  a.perm = c.perm;
  return a;
}

template <typename T, bool EXACT>
cudaError_t launch_axhelm(const Mesh& m, const OpData<T>& op, T* au, const T* u, const Coef<T>& c,
                          cudaStream_t s) {
  AxArgs<T> a = make_args(m, op, au, u, c);
  return launch_ax<T, EXACT, false>(m, a, nullptr, s);
}

template <typename T, bool EXACT>
cudaError_t launch_axhelm_cg(const Mesh& m, const OpData<T>& op, T* w, T* p, const T* r,
                             const T* d, const Coef<T>& c, const CgScalars* cg, double* partial,
                             int* nparts, cudaStream_t s) {
  AxArgs<T> a = make_args(m, op, w, p, c);
  a.p = p;
  a.r = r;
  a.d = d;
  a.cg = cg;
  a.partial = partial;
  a.allrho = sizeof(T) == 4 ? 1 : 0;  // FP32: rho over every point (see AxArgs)
  return launch_ax<T, EXACT, true>(m, a, nparts, s);
}

}  // namespace nekgpu
