// axhelm_f32.cu -- FP32 instantiations of the operator (inner solve of the mixed-precision PCG).
#include "axhelm_launch.cuh"

namespace nekgpu {

template cudaError_t launch_axhelm<float, false>(const Mesh&, const OpData<float>&, float*,
                                                 const float*, const Coef<float>&, cudaStream_t);
template cudaError_t launch_axhelm_cg<float, false>(const Mesh&, const OpData<float>&, float*,
                                                    float*, const float*, const float*,
                                                    const Coef<float>&, const CgScalars*, double*,
                                                    int*, cudaStream_t);

}  // namespace nekgpu
