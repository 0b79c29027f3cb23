// adjoint.cu -- derivative of the Helmholtz operator with respect to the
// per-point viscosity h1.
//
// The operator of core/hmholtz.f:72-259 is linear in h1:
//   lam^T A(h1) u = sum_e sum_p h1_p (grad^ lam)_p . (G_p grad^ u)_p
// with grad^ = (D_r, D_s, D_t) the reference-element derivatives and G_p the
// symmetric 3x3 matrix (G1 G4 G5; G4 G2 G6; G5 G6 G3) of geodat1.  Hence
//   d(lam^T A u) / d h1_p = (grad^ lam)_p . (G_p grad^ u)_p,
// which this kernel evaluates for every local point (one element per thread
// slab, both fields staged in shared memory, contractions as in axhelm).
// For J(u(h1)) with A(h1) u = f, the adjoint lam solves A lam = dJ/du (A is
// symmetric, so that is the same Jacobi-PCG solve) and
// dJ/dh1 = -d(lam^T A u)/dh1.
#include "impl.cuh"
#include "nekgpu.h"

namespace nekgpu {
namespace {

template <int NX>
__global__ void __launch_bounds__(256)
    adjoint_h1_kernel(double* __restrict__ gh1, const double* __restrict__ lam,
                      const double* __restrict__ u, const double* __restrict__ G,
                      const double* __restrict__ D, int nel) {
  constexpr int P = NX * NX * NX, NXY = NX * NX, R = NX + 1;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  double* sD = reinterpret_cast<double*>(smem_raw);  // D[i][l] at i*R + l
  double* su = sD + NX * R + threadIdx.y * 2 * P;
  double* sl = su + P;
  const int i = threadIdx.x % NX, j = threadIdx.x / NX;
  const int ft = threadIdx.x + NXY * threadIdx.y, nthr = NXY * blockDim.y;
  for (int q = ft; q < NXY; q += nthr) sD[(q / NX) * R + q % NX] = D[q];
  const int e = blockIdx.x * blockDim.y + threadIdx.y;
  const bool act = e < nel;
  const size_t eo = (size_t)(act ? e : 0) * P;
  double ru[NX], rl[NX];
#pragma unroll
  for (int k = 0; k < NX; ++k) {
    const int pt = k * NXY + j * NX + i;
    ru[k] = act ? u[eo + pt] : 0.0;
    rl[k] = act ? lam[eo + pt] : 0.0;
    su[pt] = ru[k];
    sl[pt] = rl[k];
  }
  __syncthreads();
  const double* g = G + (size_t)(act ? e : 0) * 6 * P;
#pragma unroll
  for (int k = 0; k < NX; ++k) {
    double ur = 0, us = 0, ut = 0, lr = 0, ls = 0, lt = 0;
#pragma unroll
    for (int l = 0; l < NX; ++l) {
      const double dil = sD[i * R + l], djl = sD[j * R + l], dkl = sD[k * R + l];
      ur = fma(dil, su[k * NXY + j * NX + l], ur);  // D(i,l) u(l,j,k)
      lr = fma(dil, sl[k * NXY + j * NX + l], lr);
      us = fma(djl, su[k * NXY + l * NX + i], us);  // D(j,l) u(i,l,k)
      ls = fma(djl, sl[k * NXY + l * NX + i], ls);
      ut = fma(dkl, ru[l], ut);                     // D(k,l) u(i,j,l)
      lt = fma(dkl, rl[l], lt);
    }
    const int pt = k * NXY + j * NX + i;
    if (act) {
      const double g1 = g[pt], g2 = g[P + pt], g3 = g[2 * P + pt], g4 = g[3 * P + pt],
                   g5 = g[4 * P + pt], g6 = g[5 * P + pt];
      const double t1 = g1 * ur + g4 * us + g5 * ut;
      const double t2 = g4 * ur + g2 * us + g6 * ut;
      const double t3 = g5 * ur + g6 * us + g3 * ut;
      gh1[eo + pt] = lr * t1 + ls * t2 + lt * t3;
    }
  }
}

template <int NX>
cudaError_t launch_adjoint(const Mesh& m, double* gh1, const double* lam, const double* u,
                           cudaStream_t s) {
  constexpr int P = NX * NX * NX;
  const int epb = axhelm_epb(NX);
  const size_t smem = (size_t)(NX * (NX + 1) + epb * 2 * P) * sizeof(double);
  static std::atomic<uint32_t> configured{0};  // per device
  if (first_on_device(configured)) {
    cudaError_t e = cudaFuncSetAttribute(adjoint_h1_kernel<NX>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    mark_device(configured);
  }
  count_launch();
  adjoint_h1_kernel<NX><<<(m.nel + epb - 1) / epb, dim3(NX * NX, epb), smem, s>>>(
      gh1, lam, u, m.f64.G, m.f64.D, m.nel);
  return cudaGetLastError();
}

}  // namespace

cudaError_t axhelm_adjoint_h1(const Mesh& m, double* gh1, const double* lam, const double* u,
                              cudaStream_t s) {
  switch (m.nx1) {
    case 2: return launch_adjoint<2>(m, gh1, lam, u, s);
    case 3: return launch_adjoint<3>(m, gh1, lam, u, s);
    case 4: return launch_adjoint<4>(m, gh1, lam, u, s);
    case 5: return launch_adjoint<5>(m, gh1, lam, u, s);
    case 6: return launch_adjoint<6>(m, gh1, lam, u, s);
    case 7: return launch_adjoint<7>(m, gh1, lam, u, s);
    case 8: return launch_adjoint<8>(m, gh1, lam, u, s);
    case 9: return launch_adjoint<9>(m, gh1, lam, u, s);
    case 10: return launch_adjoint<10>(m, gh1, lam, u, s);
    case 11: return launch_adjoint<11>(m, gh1, lam, u, s);
    case 12: return launch_adjoint<12>(m, gh1, lam, u, s);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace nekgpu
