// axhelm_launch.cuh -- runtime dispatch of axhelm_kernel over lx1.
// Included by one translation unit per precision so the instantiations
// compile in parallel.
#pragma once
#include "axhelm_tma.cuh"
#include "impl.cuh"

namespace nekgpu {

template <int NX, typename T, bool EXACT, bool FUSED>
static cudaError_t launch_ax_nx(const Mesh& m, const AxArgs<T>& a, int* nblocks, cudaStream_t s) {
  const int epb = axhelm_epb(NX);
  const size_t smem = axhelm_smem_bytes<NX, T>(epb);
  static bool configured = false;  // per instantiation
  if (!configured) {
    cudaError_t e = cudaFuncSetAttribute(axhelm_kernel<NX, T, EXACT, FUSED>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    configured = true;
  }
  const int nb = (m.nel + epb - 1) / epb;
  if (nblocks) *nblocks = nb;
  dim3 block(NX * NX, epb);
  count_launch();
  axhelm_kernel<NX, T, EXACT, FUSED><<<nb, block, smem, s>>>(a);
  return cudaGetLastError();
}

// TMA-staged form: even lx1 (so one element's slice is a multiple of 16
// bytes) and 16-byte aligned arrays.
template <int NX, typename T, bool FUSED>
static cudaError_t launch_tma_nx(const Mesh& m, const AxArgs<T>& a, int* nblocks, cudaStream_t s) {
  constexpr int EPB = tma_epb<NX>();
  const size_t smem = tma_smem_bytes<NX, T>(FUSED, a.h1mode, a.h2mode);
  static bool configured = false;
  if (!configured) {
    const int maxb = (int)tma_smem_bytes<NX, T>(true, 1, 2);
    cudaError_t e = cudaFuncSetAttribute(axhelm_tma_kernel<NX, T, FUSED>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, maxb);
    if (e != cudaSuccess) return e;
    cudaFuncSetAttribute(axhelm_tma_kernel<NX, T, FUSED>,
                         cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    configured = true;
  }
  const int nb = (m.nel + EPB - 1) / EPB;
  if (nblocks) *nblocks = nb;
  count_launch();
  axhelm_tma_kernel<NX, T, FUSED><<<nb, dim3(NX * NX, EPB), smem, s>>>(a);
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

template <typename T, bool EXACT, bool FUSED>
static cudaError_t launch_ax(const Mesh& m, const AxArgs<T>& a, int* nblocks, cudaStream_t s) {
  // FP64 is bound by the FP64 pipe, where the plain-load kernel (D in shared
  // memory, higher occupancy) is faster; the TMA form serves FP32.
  if (!EXACT && sizeof(T) == 4 && m.use_tma && tma_ok<T, FUSED>(a)) {
    switch (m.nx1) {
      case 2: return launch_tma_nx<2, T, FUSED>(m, a, nblocks, s);
      case 4: return launch_tma_nx<4, T, FUSED>(m, a, nblocks, s);
      case 6: return launch_tma_nx<6, T, FUSED>(m, a, nblocks, s);
      case 8: return launch_tma_nx<8, T, FUSED>(m, a, nblocks, s);
      case 10: return launch_tma_nx<10, T, FUSED>(m, a, nblocks, s);
      case 12: return launch_tma_nx<12, T, FUSED>(m, a, nblocks, s);
      default: break;
    }
  }
  switch (m.nx1) {
    case 2: return launch_ax_nx<2, T, EXACT, FUSED>(m, a, nblocks, s);
    case 3: return launch_ax_nx<3, T, EXACT, FUSED>(m, a, nblocks, s);
    case 4: return launch_ax_nx<4, T, EXACT, FUSED>(m, a, nblocks, s);
    case 5: return launch_ax_nx<5, T, EXACT, FUSED>(m, a, nblocks, s);
    case 6: return launch_ax_nx<6, T, EXACT, FUSED>(m, a, nblocks, s);
    case 7: return launch_ax_nx<7, T, EXACT, FUSED>(m, a, nblocks, s);
    case 8: return launch_ax_nx<8, T, EXACT, FUSED>(m, a, nblocks, s);
    case 9: return launch_ax_nx<9, T, EXACT, FUSED>(m, a, nblocks, s);
    case 10: return launch_ax_nx<10, T, EXACT, FUSED>(m, a, nblocks, s);
    case 11: return launch_ax_nx<11, T, EXACT, FUSED>(m, a, nblocks, s);
    case 12: return launch_ax_nx<12, T, EXACT, FUSED>(m, a, nblocks, s);
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
  a.D = op.D;
  a.nel = m.nel;
  a.err = m.dev_err;
  a.skip = m.gs.skip;
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
                             int* nblocks, cudaStream_t s) {
  AxArgs<T> a = make_args(m, op, w, p, c);
  a.p = p;
  a.r = r;
  a.d = d;
  a.cg = cg;
  a.partial = partial;
  return launch_ax<T, EXACT, true>(m, a, nblocks, s);
}

}  // namespace nekgpu
