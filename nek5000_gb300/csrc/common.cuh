// common.cuh -- internal types and device helpers of the nekgpu library.
//
// Data layout in HBM (one mesh per handle):
//   geometric factors  G[e][m][p], m = 0..5 (G1..G6), p = 0..lx1^3-1
//                      (element-blocked: one element's six factors form one
//                      contiguous 6*lx1^3 block, read once per operator apply)
//   fields             f[e*lx1^3 + p], the reference's element-major layout
//   derivative matrix  D[i][j] row-major (D[i][j] = dl_j/dr at z_i)
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <atomic>
#include <string>

namespace nekgpu {

constexpr int kMaxLx1 = 12;

// Process-wide count of kernel launches made by this library.
inline std::atomic<long long>& launch_counter() {
  static std::atomic<long long> c{0};
  return c;
}
// Launches recorded into a CUDA graph are counted when the graph runs, not
// while it is captured.
inline bool& capturing() {
  static thread_local bool c = false;
  return c;
}
inline void count_launch(long long k = 1) {
  if (!capturing()) launch_counter().fetch_add(k, std::memory_order_relaxed);
}

// Function attributes (the dynamic shared-memory limit, the carveout) belong
// to a kernel on one device: a launch site sets them once per device it
// launches on, recorded in a per-site mask of device bits.
inline bool first_on_device(const std::atomic<uint32_t>& mask) {
  int dev = 0;
  cudaGetDevice(&dev);
  return (mask.load(std::memory_order_relaxed) & (1u << (dev & 31))) == 0;
}
inline void mark_device(std::atomic<uint32_t>& mask) {
  int dev = 0;
  cudaGetDevice(&dev);
  mask.fetch_or(1u << (dev & 31), std::memory_order_relaxed);
}

// ---- reductions: deterministic (fixed tree, no floating-point atomics) ----
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sum over the whole block; the result is valid in every thread.
// `scratch` must hold 32 values of T.
template <typename T>
__device__ __forceinline__ T block_sum(T v, T* scratch) {
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nthr = blockDim.x * blockDim.y * blockDim.z;
  const int lane = tid & 31, wid = tid >> 5, nw = (nthr + 31) >> 5;
  v = warp_sum(v);
  __syncthreads();
  if (lane == 0) scratch[wid] = v;
  __syncthreads();
  T t = (tid < nw) ? scratch[tid] : T(0);
  if (wid == 0) t = warp_sum(t);
  if (tid == 0) scratch[0] = t;
  __syncthreads();
  t = scratch[0];
  __syncthreads();
  return t;
}

// ---- reductions with one FP64 value per warp ---------------------------------
// Compensated (TwoSum) accumulator in field precision.  For float, the
// per-thread sums and the warp tree stay in FP32 with an error term, and only
// the warp result is widened to FP64; on this GPU FP64 issue is 64x slower
// than FP32, so FP64 work per point is avoided in the FP32 kernels.
template <typename T>
struct CompAcc {
  T s = T(0), c = T(0);
  __device__ __forceinline__ void add(T v) {
    const T t = s + v;
    const T bp = t - s;
    c += (s - (t - bp)) + (v - bp);
    s = t;
  }
  __device__ __forceinline__ void add(const CompAcc& o) {
    add(o.s);
    c += o.c;
  }
};

// FP64 fields need no compensation: plain accumulation (FP64 issue is scarce).
template <>
struct CompAcc<double> {
  double s = 0.0, c = 0.0;
  __device__ __forceinline__ void add(double v) { s += v; }
  __device__ __forceinline__ void add(const CompAcc& o) { s += o.s; }
};

// Sum of CompAcc over the block, valid in thread 0.  `scratch`: 32 doubles.
template <typename T>
__device__ __forceinline__ double block_sum_comp(CompAcc<T> a, double* scratch) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    CompAcc<T> b;
    b.s = __shfl_xor_sync(0xffffffffu, a.s, o);
    b.c = __shfl_xor_sync(0xffffffffu, a.c, o);
    a.add(b);
  }
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int nw = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
  __syncthreads();
  if ((tid & 31) == 0) scratch[tid >> 5] = (double)a.s + (double)a.c;  // c == 0 for FP64
  __syncthreads();
  double r = 0.0;
  if (tid == 0)
    for (int q = 0; q < nw; ++q) r += scratch[q];
  __syncthreads();
  return r;
}

// 16-byte vector of T, loaded / stored as one access.
template <typename T>
struct Vec16;
template <>
struct Vec16<float> {
  using type = float4;
};
template <>
struct Vec16<double> {
  using type = double2;
};
template <typename T>
__device__ __forceinline__ void ld16(T* v, const T* base, int64_t iv) {
  using V = typename Vec16<T>::type;
  *reinterpret_cast<V*>(v) = reinterpret_cast<const V*>(base)[iv];
}
template <typename T>
__device__ __forceinline__ void st16(T* base, const T* v, int64_t iv) {
  using V = typename Vec16<T>::type;
  reinterpret_cast<V*>(base)[iv] = *reinterpret_cast<const V*>(v);
}

// L2 eviction priorities for one access (createpolicy + .L2::cache_hint,
// sm_80 and later).  The FP32 PCG keeps its 4-byte-per-point operator output
// w resident in L2 from the operator kernel through the boundary-group and
// update kernels: the operator streams its inputs with evict_first and
// stores w with evict_last, the boundary-group kernel touches w with
// evict_last, and the update kernel's last read of w uses evict_first.
__device__ __forceinline__ uint64_t l2_policy_evict_first() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_policy_evict_normal() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_normal.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint64_t l2_policy_evict_last() {
  uint64_t p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ float ld_hint(const float* a, uint64_t pol) {
  float v;
  asm volatile("ld.global.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ float4 ld_hint4(const float* a, uint64_t pol) {
  float4 v;
  asm volatile("ld.global.L2::cache_hint.v4.f32 {%0, %1, %2, %3}, [%4], %5;"
               : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w)
               : "l"(a), "l"(pol));
  return v;
}
__device__ __forceinline__ void st_hint(float* a, float v, uint64_t pol) {
  asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(a), "f"(v), "l"(pol) : "memory");
}

// Scalars of one PCG solve, resident on the device (no host round trip per
// iteration).  All FP64, whatever the field precision.
struct CgScalars {
  double rtz1, rtz2, rho, alpha, beta;
  double rbn0, rbn2, tol, tin, vol;
  double s1, s2;
  int iter;       // iteration index of the last completed convergence check
  int niter;      // reported iteration count (cggo's niter)
  int done;       // 1 = converged (or stopped), kernels return immediately
  int maxiter;    // min(maxit, maxcg)
  int istep;      // reference istep (for the "at least one iteration" rule)
  int nonfinite;  // set when a non-finite norm is met
  unsigned int counter[4];  // last-block tickets, one per reduction site
  // null-space correction (no Dirichlet point and h2 = 0, hmholtz.f:705-750)
  int mcor;       // 1: active
  double smean;   // -1 / sum bm1
  double zmean;   // rmean of the last check: z = r d + zmean
};

// Exact-order helpers: products and sums are rounded separately (no fused
// multiply-add), reproducing an unfused left-to-right evaluation.
__device__ __forceinline__ double mul_x(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double add_x(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float mul_x(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float add_x(float a, float b) { return __fadd_rn(a, b); }

template <bool EXACT, typename T>
__device__ __forceinline__ T madd(T a, T b, T c) {  // a*b + c
  if constexpr (EXACT) return add_x(mul_x(a, b), c);
  else return fma(a, b, c);
}

}  // namespace nekgpu
