// axhelm_f64.cu -- FP64 instantiations of the operator (exact and fused-multiply-add forms).
#include "axhelm_launch.cuh"

namespace nekgpu {

// Number of rho partials of a fused operator launch (one per element, for
// every launch shape).
int axhelm_blocks(int nx1, int nel) {
  (void)nx1;
  return nel;
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
