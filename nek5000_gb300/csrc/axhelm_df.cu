// axhelm_df.cu -- instantiations of the double-float FP64 operator
// (axhelm_df.cuh) and the split geometric factors it reads.
#include "axhelm_df.cuh"
#include "impl.cuh"

namespace nekgpu {
namespace {

__global__ void split_pairs_kernel(float2* __restrict__ o, const double* __restrict__ a,
                                   int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const DfPair p = df_split(a[i]);
    o[i] = make_float2(p.h, p.l);
  }
}

template <int NX, bool FUSED>
cudaError_t launch_nx(const Mesh& m, const DfArgs& A, int epb, cudaStream_t s) {
  if (epb < 1 || epb * NX * NX > 256) epb = axhelm_epb(NX);
  static std::atomic<uint32_t> configured{0};  // per device
  if (first_on_device(configured)) {
    cudaError_t e = cudaFuncSetAttribute(axhelm_df_kernel<NX, FUSED>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)axhelm_df_smem_bytes<NX>(axhelm_epb(NX)));
    if (e != cudaSuccess) return e;
    mark_device(configured);
  }
  const int nb = (m.nel + epb - 1) / epb;
  count_launch();
  axhelm_df_kernel<NX, FUSED><<<nb, dim3(NX * NX, epb), axhelm_df_smem_bytes<NX>(epb), s>>>(A);
  return cudaGetLastError();
}

template <bool FUSED>
cudaError_t launch_fused(const Mesh& m, const DfArgs& A, int epb, cudaStream_t s) {
  switch (m.nx1) {
    case 2: return launch_nx<2, FUSED>(m, A, epb, s);
    case 3: return launch_nx<3, FUSED>(m, A, epb, s);
    case 4: return launch_nx<4, FUSED>(m, A, epb, s);
    case 5: return launch_nx<5, FUSED>(m, A, epb, s);
    case 6: return launch_nx<6, FUSED>(m, A, epb, s);
    case 7: return launch_nx<7, FUSED>(m, A, epb, s);
    case 8: return launch_nx<8, FUSED>(m, A, epb, s);
    case 9: return launch_nx<9, FUSED>(m, A, epb, s);
    case 10: return launch_nx<10, FUSED>(m, A, epb, s);
    case 11: return launch_nx<11, FUSED>(m, A, epb, s);
    case 12: return launch_nx<12, FUSED>(m, A, epb, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

cudaError_t launch_axhelm_df(const Mesh& m, const AxArgs<double>& a, bool fused, int epb,
                             int* nparts, cudaStream_t s) {
  DfArgs A;
  A.a = a;
  A.Gdf = m.Gdf.ptr;
  A.Ddf = m.Ddf.ptr;
  if (nparts) *nparts = m.nel;
  return fused ? launch_fused<true>(m, A, epb, s) : launch_fused<false>(m, A, epb, s);
}

// (hi, lo) pairs of G1..G6 and D for the double-float operator; rebuilt
// after every geometry change while the option is on.
int build_df(Handle& h) {
  Mesh& m = h.mesh;
  m.has_df = false;
  const int64_t n6 = 6 * m.n, nd = (int64_t)m.nx1 * m.nx1;
  if (m.Gdf.ensure((size_t)n6) || m.Ddf.ensure((size_t)nd)) return -4;
  count_launch(2);
  split_pairs_kernel<<<(int)std::min<int64_t>((n6 + 255) / 256, 152 * 16), 256, 0, h.stream>>>(
      m.Gdf.ptr, m.f64.G, n6);
  split_pairs_kernel<<<1, 256, 0, h.stream>>>(m.Ddf.ptr, m.f64.D, nd);
  if (cudaStreamSynchronize(h.stream) != cudaSuccess) return -3;
  m.has_df = true;
  return 0;
}

}  // namespace nekgpu
