// axhelm_tma.cu -- FP32 instantiations of the TMA-staged operator
// (axhelm_tma.cuh), every lx1 it serves and every candidate block shape.
#include "axhelm_tma.cuh"
#include "impl.cuh"

namespace nekgpu {
namespace {

// The kernel of a shape (lx1 = 10 with one element per block has its own
// register bound).
template <int NX, bool FUSED, int EPB>
constexpr auto tma_kernel() {
  if constexpr (NX == 10 && EPB == 1) return axhelm_tma_kernel_10x1<float, FUSED>;
  else return axhelm_tma_kernel<NX, float, FUSED, EPB>;
}

template <int NX, bool FUSED, int EPB>
cudaError_t launch_one(const Mesh& m, const AxArgs<float>& a, int* nparts, cudaStream_t s) {
  const size_t smem = tma_smem_bytes<NX, float, EPB>(FUSED, a.h1mode, a.h2mode);
  auto kern = tma_kernel<NX, FUSED, EPB>();
  // per instantiation and device: room for the largest slice set
  static std::atomic<uint32_t> configured{0};
  if (first_on_device(configured)) {
    const int maxb = (int)tma_smem_bytes<NX, float, EPB>(true, 1, 2);
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, maxb);
    if (e != cudaSuccess) return e;
    cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    mark_device(configured);
  }
  const int nb = (m.nel + EPB - 1) / EPB;
  if (nparts) *nparts = m.nel;
  count_launch();
  kern<<<nb, dim3(NX * NX, EPB), smem, s>>>(a);
  return cudaGetLastError();
}

template <int NX, bool FUSED>
cudaError_t launch_nx(const Mesh& m, const AxArgs<float>& a, int epb, int* nparts,
                      cudaStream_t s) {
  if (epb == 0 || epb == tma_epb_cand<NX>(1))
    return launch_one<NX, FUSED, tma_epb_cand<NX>(1)>(m, a, nparts, s);
  if (epb == tma_epb_cand<NX>(0)) return launch_one<NX, FUSED, tma_epb_cand<NX>(0)>(m, a, nparts, s);
  if (epb == tma_epb_cand<NX>(2)) return launch_one<NX, FUSED, tma_epb_cand<NX>(2)>(m, a, nparts, s);
  return cudaErrorInvalidValue;
}

template <bool FUSED>
cudaError_t launch_fused(const Mesh& m, const AxArgs<float>& a, int epb, int* nparts,
                         cudaStream_t s) {
  switch (m.nx1) {
    case 2: return launch_nx<2, FUSED>(m, a, epb, nparts, s);
    case 3: return launch_nx<3, FUSED>(m, a, epb, nparts, s);
    case 4: return launch_nx<4, FUSED>(m, a, epb, nparts, s);
    case 5: return launch_nx<5, FUSED>(m, a, epb, nparts, s);
    case 7: return launch_nx<7, FUSED>(m, a, epb, nparts, s);
    case 9: return launch_nx<9, FUSED>(m, a, epb, nparts, s);
    case 6: return launch_nx<6, FUSED>(m, a, epb, nparts, s);
    case 8: return launch_nx<8, FUSED>(m, a, epb, nparts, s);
    case 10: return launch_nx<10, FUSED>(m, a, epb, nparts, s);
    case 12: return launch_nx<12, FUSED>(m, a, epb, nparts, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

cudaError_t launch_tma_f32(const Mesh& m, const AxArgs<float>& a, bool fused, int epb,
                           int* nparts, cudaStream_t s) {
  return fused ? launch_fused<true>(m, a, epb, nparts, s)
               : launch_fused<false>(m, a, epb, nparts, s);
}

// Built-in elements per block of the TMA kernel for lx1 = nx.
int tma_default_epb(int nx) {
  switch (nx) {
    case 2: return tma_epb<2>();
    case 3: return tma_epb<3>();
    case 4: return tma_epb<4>();
    case 5: return tma_epb<5>();
    case 7: return tma_epb<7>();
    case 9: return tma_epb<9>();
    case 6: return tma_epb<6>();
    case 8: return tma_epb<8>();
    case 10: return tma_epb<10>();
    case 12: return tma_epb<12>();
    default: return 0;
  }
}

// TMA candidates of lx1 = nx (the distinct values of tma_epb_cand).
std::vector<int> tma_candidates(int nx) {
  std::vector<int> v;
  auto add = [&](int e) {
    for (int x : v)
      if (x == e) return;
    v.push_back(e);
  };
  switch (nx) {
#define NEKGPU_TMA_CAND(N)                                   \
  case N:                                                    \
    for (int q = 0; q < 3; ++q) add(tma_epb_cand<N>(q));     \
    break;
    NEKGPU_TMA_CAND(2)
    NEKGPU_TMA_CAND(3)
    NEKGPU_TMA_CAND(4)
    NEKGPU_TMA_CAND(5)
    NEKGPU_TMA_CAND(7)
    NEKGPU_TMA_CAND(9)
    NEKGPU_TMA_CAND(6)
    NEKGPU_TMA_CAND(8)
    NEKGPU_TMA_CAND(10)
    NEKGPU_TMA_CAND(12)
#undef NEKGPU_TMA_CAND
    default: break;
  }
  return v;
}

}  // namespace nekgpu
