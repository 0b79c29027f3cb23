// axhelm_f64.cu -- FP64 instantiations of the operator (exact and fused-multiply-add forms).
#include "axhelm_launch.cuh"

namespace nekgpu {

// Upper bound on the blocks of any operator launch (sizes the rho partials).
int axhelm_blocks(int nx1, int nel) {
  int epb = axhelm_epb(nx1);
  int b = (nel + epb - 1) / epb;
  int t = 1;
  switch (nx1) {
    case 2: t = tma_epb<2>(); break;
    case 4: t = tma_epb<4>(); break;
    case 6: t = tma_epb<6>(); break;
    case 8: t = tma_epb<8>(); break;
    case 10: t = tma_epb<10>(); break;
    case 12: t = tma_epb<12>(); break;
    default: t = epb;
  }
  return std::max(b, (nel + t - 1) / t);
}

template cudaError_t launch_axhelm<double, true>(const Mesh&, const OpData<double>&, double*,
                                                 const double*, const Coef<double>&, cudaStream_t);
template cudaError_t launch_axhelm<double, false>(const Mesh&, const OpData<double>&, double*,
                                                  const double*, const Coef<double>&,
                                                  cudaStream_t);
template cudaError_t launch_axhelm_cg<double, true>(const Mesh&, const OpData<double>&, double*,
                                                    double*, const double*, const double*,
                                                    const Coef<double>&, const CgScalars*,
                                                    double*, int*, cudaStream_t);
template cudaError_t launch_axhelm_cg<double, false>(const Mesh&, const OpData<double>&, double*,
                                                     double*, const double*, const double*,
                                                     const Coef<double>&, const CgScalars*,
                                                     double*, int*, cudaStream_t);

}  // namespace nekgpu
