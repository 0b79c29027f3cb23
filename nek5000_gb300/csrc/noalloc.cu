// noalloc.cu -- an operator entry point that allocates no device memory.
//
// nekgpu_axhelm_dev scans h1 and h2 before applying the operator (a uniform
// coefficient is passed as a scalar, an h2 of zero drops the mass term), and
// that scan keeps its per-block minima and maxima in a reduction buffer the
// handle allocates on first use.  Some callers cannot let a library allocate:
// a code that has handed all device memory to its own pool allocator, one
// that runs under a hard memory budget, or a time-step loop that must not
// pay for the device-wide synchronisation cudaMalloc implies.
// nekgpu_axhelm_dev_noalloc serves them: its scan writes the partials to the
// fixed array below, which every GPU that loads this library holds until the
// process exits, and the call itself makes no allocation.
#include <mutex>

#include "impl.cuh"
#include "nekgpu.h"

namespace nekgpu {
namespace {

constexpr int kScanThreads = 256;
constexpr int kPointsPerThread = 8;
constexpr int64_t kPointsPerBlock = (int64_t)kScanThreads * kPointsPerThread;
constexpr int kScanMaxBlocks = NEKGPU_NOALLOC_MAX_POINTS / kPointsPerBlock;

// Four values per scan block: min h1, max h1, min h2, max h2.
static __device__ __align__(256) double g_scan_scratch[4 * kScanMaxBlocks];

// Device address of g_scan_scratch, looked up once per device.
std::mutex g_addr_mu;
double* g_addr[64] = {};

int scratch_address(int device, double** out, std::string& err) {
  if (device < 0 || device >= 64) {
    err = "noalloc: device ordinal out of range";
    return NEKGPU_EINVAL;
  }
  std::lock_guard<std::mutex> lk(g_addr_mu);
  if (!g_addr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_scan_scratch);
    if (e != cudaSuccess) {
      err = std::string("noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e);
      return NEKGPU_ECUDA;
    }
    g_addr[device] = static_cast<double*>(p);
  }
  *out = g_addr[device];
  return 0;
}

// Per-block min and max of h1 and h2; every slot it writes is read by the
// host afterwards, and it writes each slot of the blocks it launches, so no
// slot needs clearing between calls.
__global__ void __launch_bounds__(kScanThreads)
    coef_scan_kernel(const double* __restrict__ h1, const double* __restrict__ h2, int64_t n,
                     double* __restrict__ out) {
  __shared__ double s[4][32];
  double m1 = INFINITY, x1 = -INFINITY, m2 = INFINITY, x2 = -INFINITY;
  const int64_t b0 = blockIdx.x * kPointsPerBlock;
  for (int q = 0; q < kPointsPerThread; ++q) {
    const int64_t i = b0 + (int64_t)q * kScanThreads + threadIdx.x;
    if (i < n) {
      const double a = h1[i], c = h2[i];
      m1 = fmin(m1, a);
      x1 = fmax(x1, a);
      m2 = fmin(m2, c);
      x2 = fmax(x2, c);
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    m1 = fmin(m1, __shfl_xor_sync(0xffffffffu, m1, o));
    x1 = fmax(x1, __shfl_xor_sync(0xffffffffu, x1, o));
    m2 = fmin(m2, __shfl_xor_sync(0xffffffffu, m2, o));
    x2 = fmax(x2, __shfl_xor_sync(0xffffffffu, x2, o));
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    s[0][wid] = m1;
    s[1][wid] = x1;
    s[2][wid] = m2;
    s[3][wid] = x2;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 1; q < kScanThreads / 32; ++q) {
      m1 = fmin(m1, s[0][q]);
      x1 = fmax(x1, s[1][q]);
      m2 = fmin(m2, s[2][q]);
      x2 = fmax(x2, s[3][q]);
    }
    out[4 * blockIdx.x] = m1;
    out[4 * blockIdx.x + 1] = x1;
    out[4 * blockIdx.x + 2] = m2;
    out[4 * blockIdx.x + 3] = x2;
  }
}

}  // namespace
}  // namespace nekgpu

using namespace nekgpu;

// Handle lookup shared with capi.cu.
namespace nekgpu {
Handle* handle_lookup(const int64_t* h);
int handle_fail(Handle* H, int code, const std::string& msg);
}  // namespace nekgpu

extern "C" int nekgpu_axhelm_dev_noalloc(const int64_t* handle, double* au, const double* u,
                                         const double* h1, const double* h2, const int* imesh,
                                         const int* isd) {
  (void)imesh;
  (void)isd;
  Handle* H = handle_lookup(handle);
  if (!H) return handle_fail(nullptr, NEKGPU_EHANDLE, "unknown handle");
  if (handle_enter(*H) != cudaSuccess)
    return handle_fail(H, NEKGPU_ECUDA, "call entry failed");
  if (!H->has_mesh) return handle_fail(H, NEKGPU_ENOSETUP, "mesh not set up (nekgpu_setup)");
  if (!au || !u || !h1 || !h2) return handle_fail(H, NEKGPU_EINVAL, "null array argument");
  const int64_t n = H->mesh.n;
  if (n > NEKGPU_NOALLOC_MAX_POINTS)
    return handle_fail(H, NEKGPU_EINVAL,
                       "axhelm_dev_noalloc: " + std::to_string(n) +
                           " points exceed the fixed scratch (at most " +
                           std::to_string(NEKGPU_NOALLOC_MAX_POINTS) + " points)");
  std::string err;
  double* scratch = nullptr;
  int rc = scratch_address(H->device, &scratch, err);
  if (rc) return handle_fail(H, rc, err);
  const int nb = (int)((n + kPointsPerBlock - 1) / kPointsPerBlock);
  if (H->timing) cudaEventRecord(H->evt0, H->stream);
  count_launch();
  coef_scan_kernel<<<nb, kScanThreads, 0, H->stream>>>(h1, h2, n, scratch);
  // host copy of the partials: per thread, not on the stack (64 KiB)
  static thread_local double part[4 * kScanMaxBlocks];
  cudaError_t e = cudaMemcpyAsync(part, scratch, 4 * (size_t)nb * sizeof(double),
                                  cudaMemcpyDeviceToHost, H->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
  if (e != cudaSuccess)
    return handle_fail(H, NEKGPU_ECUDA, std::string("axhelm_dev_noalloc: ") + cudaGetErrorString(e));
  double mn1 = INFINITY, mx1 = -INFINITY, mn2 = INFINITY, mx2 = -INFINITY;
  for (int b = 0; b < nb; ++b) {
    mn1 = std::min(mn1, part[4 * b]);
    mx1 = std::max(mx1, part[4 * b + 1]);
    mn2 = std::min(mn2, part[4 * b + 2]);
    mx2 = std::max(mx2, part[4 * b + 3]);
  }
  // the same coefficient modes as the allocating entry point
  Coef<double> c;
  c.h1 = h1;
  c.h2 = h2;
  if (mn1 == mx1) {
    c.h1mode = 0;
    c.h1s = mn1;
  } else {
    c.h1mode = 1;
  }
  if (std::max(std::fabs(mn2), std::fabs(mx2)) == 0.0) {
    c.h2mode = 0;
    c.h2s = 0.0;
  } else if (mn2 == mx2) {
    c.h2mode = 1;
    c.h2s = mn2;
  } else {
    c.h2mode = 2;
  }
  e = H->exact ? launch_axhelm<double, true>(H->mesh, H->mesh.f64, au, u, c, H->stream)
               : launch_axhelm<double, false>(H->mesh, H->mesh.f64, au, u, c, H->stream);
  if (e == cudaSuccess && H->timing) e = cudaEventRecord(H->evt1, H->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
  if (e != cudaSuccess)
    return handle_fail(H, NEKGPU_ECUDA, std::string("axhelm_dev_noalloc: ") + cudaGetErrorString(e));
  if (H->timing) {  // as nekgpu_axhelm_dev: scan and operator together
    float ms = 0.f;
    cudaEventElapsedTime(&ms, H->evt0, H->evt1);
    H->ms_total = ms;
    H->ms_axhelm = ms;
    H->n_axhelm = 1;
  }
  return NEKGPU_OK;
}
