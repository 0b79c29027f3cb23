// vecops.cu -- the reference's pointwise and local-sum primitives on device
// arrays, and the interface exchange maps of an element shard: what a
// solve split over several ranks (the reference's own MPI domain
// decomposition) runs between its global sums (gop, core/comm_mpi.f:216)
// and its interface exchanges (the inter-rank part of gs_op).
//
//   col2   a = a * b                 core/math.f:563
//   col3   a = b * c                 core/math.f:597
//   add2s1 a = c1 a + b              core/math.f:677
//   add2s2 a = a + c2 b              core/math.f:689
//   vlsc3  sum a b c (local)         core/navier4.f:323
//   vlsc32 sum b c a^2 (local)       core/hmholtz.f:848
//   invcol1 a = 1 / a                core/math.f:61
//   vlmax  local max |a|, max a, min a (the local part of glamax / glmax /
//          glmin, core/math.f:873-985)
//
// Local sums are block partials added on the host in block order, so they
// are the same from run to run.  Products are rounded one by one
// (__dmul_rn / __dadd_rn), as the reference's loops.
#include <algorithm>
#include <string>
#include <vector>

#include "impl.cuh"

namespace nekgpu {
namespace {

constexpr int kVT = 256;

int vblocks(int64_t n) {
  return (int)std::min<int64_t>(std::max<int64_t>((n + 4 * kVT - 1) / (4 * kVT), 1), 152 * 6);
}

__global__ void col2_kernel(double* __restrict__ a, const double* __restrict__ b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)kVT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kVT)
    a[i] = __dmul_rn(a[i], b[i]);
}

__global__ void col3_kernel(double* __restrict__ a, const double* __restrict__ b,
                            const double* __restrict__ c, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)kVT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kVT)
    a[i] = __dmul_rn(b[i], c[i]);
}

__global__ void add2s1_kernel(double* __restrict__ a, const double* __restrict__ b, double c1,
                              int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)kVT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kVT)
    a[i] = __dadd_rn(__dmul_rn(c1, a[i]), b[i]);
}

__global__ void add2s2_kernel(double* __restrict__ a, const double* __restrict__ b, double c2,
                              int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)kVT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kVT)
    a[i] = __dadd_rn(a[i], __dmul_rn(c2, b[i]));
}

// partial[blk] = sum a b c (mode 0, vlsc3) or sum b c a a (mode 1, vlsc32)
__global__ void __launch_bounds__(kVT) lsum_kernel(const double* __restrict__ a,
                                                   const double* __restrict__ b,
                                                   const double* __restrict__ c, int mode,
                                                   int64_t n, double* __restrict__ partial) {
  __shared__ double red[kVT / 32];
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)kVT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kVT)
    s += mode == 0 ? __dmul_rn(__dmul_rn(a[i], b[i]), c[i])
                   : __dmul_rn(__dmul_rn(__dmul_rn(b[i], c[i]), a[i]), a[i]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < kVT / 32; ++q) t += red[q];
    partial[blockIdx.x] = t;
  }
}

__global__ void invcol1_kernel(double* __restrict__ a, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)kVT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kVT)
    a[i] = __drcp_rn(a[i]);
}

// partial[blk] = max |a| (mode 0), max a (1) or min a (2) over the block's points
__global__ void __launch_bounds__(kVT) lmax_kernel(const double* __restrict__ a, int mode,
                                                   int64_t n, double* __restrict__ partial) {
  __shared__ double red[kVT / 32];
  double s = mode == 2 ? 1.0e300 : (mode == 1 ? -1.0e300 : 0.0);
  for (int64_t i = blockIdx.x * (int64_t)kVT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kVT) {
    const double v = mode == 0 ? fabs(a[i]) : a[i];
    s = mode == 2 ? fmin(s, v) : fmax(s, v);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const double t = __shfl_xor_sync(0xffffffffu, s, o);
    s = mode == 2 ? fmin(s, t) : fmax(s, t);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) red[wid] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = red[0];
    for (int q = 1; q < kVT / 32; ++q) t = mode == 2 ? fmin(t, red[q]) : fmax(t, red[q]);
    partial[blockIdx.x] = t;
  }
}

// buf[k] = u[pos[start[k]]] (every copy of an interface point holds the same
// value after the local dssum)
__global__ void iface_gather_kernel(double* __restrict__ buf, const double* __restrict__ u,
                                    const int64_t* __restrict__ start,
                                    const int64_t* __restrict__ pos, int64_t nk) {
  for (int64_t k = blockIdx.x * (int64_t)kVT + threadIdx.x; k < nk;
       k += (int64_t)gridDim.x * kVT)
    buf[k] = u[pos[start[k]]];
}

// u[pos[q]] = buf[k] for every copy q of interface point k
__global__ void iface_scatter_kernel(double* __restrict__ u, const double* __restrict__ buf,
                                     const int64_t* __restrict__ start,
                                     const int64_t* __restrict__ pos, int64_t nk) {
  for (int64_t k = blockIdx.x * (int64_t)kVT + threadIdx.x; k < nk;
       k += (int64_t)gridDim.x * kVT) {
    const double v = buf[k];
    for (int64_t q = start[k]; q < start[k + 1]; ++q) u[pos[q]] = v;
  }
}

}  // namespace

// interface maps of the handle's shard (vecops.cu)
struct ShardIface {
  int64_t nk = 0;
  DevBuf<int64_t> start, pos;
};

void ShardIfaceDeleter::operator()(ShardIface* p) const { delete p; }

}  // namespace nekgpu

// ---------------------------------------------------------------------------
// C ABI
namespace nekgpu {
Handle* handle_lookup(const int64_t* h);
int handle_fail(Handle* H, int code, const std::string& msg);
}  // namespace nekgpu

using namespace nekgpu;

namespace {

Handle* vec_handle(const int64_t* handle, int* rc) {
  Handle* H = handle_lookup(handle);
  if (!H) {
    *rc = handle_fail(nullptr, NEKGPU_EHANDLE, "unknown handle");
    return nullptr;
  }
  if (handle_enter(*H) != cudaSuccess) {
    *rc = handle_fail(H, NEKGPU_ECUDA, "call entry failed");
    return nullptr;
  }
  if (!H->has_mesh) {
    *rc = handle_fail(H, NEKGPU_ENOSETUP, "mesh not set up (nekgpu_setup)");
    return nullptr;
  }
  *rc = 0;
  return H;
}

// End of a vector call: the kernels must have finished before the call
// returns (the caller may read the outputs from another stream).
int vec_done(Handle* H, const char* what) {
  const cudaError_t e = handle_leave(*H);
  if (e != cudaSuccess) return handle_fail(H, NEKGPU_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return NEKGPU_OK;
}

int local_sum(Handle* H, const double* a, const double* b, const double* c, int mode,
              double* out, const char* what) {
  if (!a || !b || !c || !out) return handle_fail(H, NEKGPU_EINVAL, "null argument");
  const int64_t n = H->mesh.n;
  const int nb = vblocks(n);
  if (H->red.ensure((size_t)nb)) return handle_fail(H, NEKGPU_ENOMEM, "device allocation failed");
  count_launch();
  lsum_kernel<<<nb, kVT, 0, H->stream>>>(a, b, c, mode, n, H->red.ptr);
  std::vector<double> h((size_t)nb);
  cudaMemcpyAsync(h.data(), H->red.ptr, nb * sizeof(double), cudaMemcpyDeviceToHost, H->stream);
  const cudaError_t e = cudaStreamSynchronize(H->stream);
  if (e != cudaSuccess) return handle_fail(H, NEKGPU_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
  double t = 0.0;
  for (int q = 0; q < nb; ++q) t += h[q];
  *out = t;
  return NEKGPU_OK;
}

}  // namespace

#define VEC_PROLOGUE()                   \
  int rc_;                               \
  Handle* H = vec_handle(handle, &rc_);  \
  if (!H) return rc_;                    \
  const int64_t n = H->mesh.n;           \
  cudaStream_t s = H->stream;

extern "C" int nekgpu_col2_dev(const int64_t* handle, double* a, const double* b) {
  VEC_PROLOGUE();
  if (!a || !b) return handle_fail(H, NEKGPU_EINVAL, "null argument");
  count_launch();
  col2_kernel<<<vblocks(n), kVT, 0, s>>>(a, b, n);
  return vec_done(H, "col2");
}

extern "C" int nekgpu_col3_dev(const int64_t* handle, double* a, const double* b, const double* c) {
  VEC_PROLOGUE();
  if (!a || !b || !c) return handle_fail(H, NEKGPU_EINVAL, "null argument");
  count_launch();
  col3_kernel<<<vblocks(n), kVT, 0, s>>>(a, b, c, n);
  return vec_done(H, "col3");
}

extern "C" int nekgpu_add2s1_dev(const int64_t* handle, double* a, const double* b,
                                 const double* c1) {
  VEC_PROLOGUE();
  if (!a || !b || !c1) return handle_fail(H, NEKGPU_EINVAL, "null argument");
  count_launch();
  add2s1_kernel<<<vblocks(n), kVT, 0, s>>>(a, b, *c1, n);
  return vec_done(H, "add2s1");
}

extern "C" int nekgpu_add2s2_dev(const int64_t* handle, double* a, const double* b,
                                 const double* c2) {
  VEC_PROLOGUE();
  if (!a || !b || !c2) return handle_fail(H, NEKGPU_EINVAL, "null argument");
  count_launch();
  add2s2_kernel<<<vblocks(n), kVT, 0, s>>>(a, b, *c2, n);
  return vec_done(H, "add2s2");
}

extern "C" int nekgpu_vlsc3_dev(const int64_t* handle, const double* a, const double* b,
                                const double* c, double* out) {
  VEC_PROLOGUE();
  (void)s;
  (void)n;
  return local_sum(H, a, b, c, 0, out, "vlsc3");
}

extern "C" int nekgpu_vlsc32_dev(const int64_t* handle, const double* a, const double* b,
                                 const double* c, double* out) {
  VEC_PROLOGUE();
  (void)s;
  (void)n;
  return local_sum(H, a, b, c, 1, out, "vlsc32");
}

extern "C" int nekgpu_invcol1_dev(const int64_t* handle, double* a) {
  VEC_PROLOGUE();
  if (!a) return handle_fail(H, NEKGPU_EINVAL, "null argument");
  count_launch();
  invcol1_kernel<<<vblocks(n), kVT, 0, s>>>(a, n);
  return vec_done(H, "invcol1");
}

extern "C" int nekgpu_vlmax_dev(const int64_t* handle, const double* a, const int* mode,
                                double* out) {
  VEC_PROLOGUE();
  if (!a || !mode || !out || *mode < 0 || *mode > 2)
    return handle_fail(H, NEKGPU_EINVAL, "bad argument");
  const int nb = vblocks(n);
  if (H->red.ensure((size_t)nb)) return handle_fail(H, NEKGPU_ENOMEM, "device allocation failed");
  count_launch();
  lmax_kernel<<<nb, kVT, 0, s>>>(a, *mode, n, H->red.ptr);
  std::vector<double> h((size_t)nb);
  cudaMemcpyAsync(h.data(), H->red.ptr, nb * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return vec_done(H, "vlmax");
  double t = h[0];
  for (int q = 1; q < nb; ++q) t = *mode == 2 ? std::min(t, h[q]) : std::max(t, h[q]);
  *out = t;
  return NEKGPU_OK;
}

extern "C" int nekgpu_setprec_local_dev(const int64_t* handle, double* diag, const double* h1,
                                        const double* h2) {
  VEC_PROLOGUE();
  (void)s;
  if (!diag || !h1 || !h2) return handle_fail(H, NEKGPU_EINVAL, "null argument");
  Coef<double> c;
  if (detect_coef<double>(*H, h1, h2, n, c))
    return handle_fail(H, NEKGPU_ECUDA, "coefficient scan failed");
  if (setprec_local_f64(*H, diag, c)) return handle_fail(H, NEKGPU_ECUDA, H->err);
  return vec_done(H, "setprec_local");
}

extern "C" int nekgpu_iface_setup(const int64_t* handle, const int64_t* nk, const int64_t* start,
                                  const int64_t* pos) {
  VEC_PROLOGUE();
  if (!nk || *nk < 0 || (*nk > 0 && (!start || !pos)))
    return handle_fail(H, NEKGPU_EINVAL, "null argument");
  const int64_t m = *nk > 0 ? start[*nk] : 0;
  for (int64_t k = 0; k < *nk; ++k)
    if (start[k + 1] <= start[k]) return handle_fail(H, NEKGPU_EINVAL, "empty interface group");
  for (int64_t q = 0; q < m; ++q)
    if (pos[q] < 0 || pos[q] >= n) return handle_fail(H, NEKGPU_EINVAL, "position out of range");
  std::unique_ptr<ShardIface, ShardIfaceDeleter> f(new ShardIface());
  f->nk = *nk;
  if (f->start.ensure((size_t)*nk + 1) || f->pos.ensure((size_t)std::max<int64_t>(m, 1)))
    return handle_fail(H, NEKGPU_ENOMEM, "device allocation failed");
  cudaMemcpyAsync(f->start.ptr, start ? start : &m, (*nk + 1) * sizeof(int64_t),
                  cudaMemcpyHostToDevice, s);
  if (m) cudaMemcpyAsync(f->pos.ptr, pos, m * sizeof(int64_t), cudaMemcpyHostToDevice, s);
  if (cudaStreamSynchronize(s) != cudaSuccess)
    return handle_fail(H, NEKGPU_ECUDA, "interface upload failed");
  H->iface = std::move(f);
  return NEKGPU_OK;
}

extern "C" int nekgpu_iface_gather_dev(const int64_t* handle, double* buf, const double* u) {
  VEC_PROLOGUE();
  (void)n;
  if (!H->iface) return handle_fail(H, NEKGPU_ENOSETUP, "interface not set up (nekgpu_iface_setup)");
  if (!buf || !u) return handle_fail(H, NEKGPU_EINVAL, "null argument");
  if (H->iface->nk == 0) return NEKGPU_OK;
  count_launch();
  iface_gather_kernel<<<vblocks(H->iface->nk), kVT, 0, s>>>(buf, u, H->iface->start.ptr,
                                                              H->iface->pos.ptr, H->iface->nk);
  return vec_done(H, "iface_gather");
}

extern "C" int nekgpu_iface_scatter_dev(const int64_t* handle, double* u, const double* buf) {
  VEC_PROLOGUE();
  (void)n;
  if (!H->iface) return handle_fail(H, NEKGPU_ENOSETUP, "interface not set up (nekgpu_iface_setup)");
  if (!buf || !u) return handle_fail(H, NEKGPU_EINVAL, "null argument");
  if (H->iface->nk == 0) return NEKGPU_OK;
  count_launch();
  iface_scatter_kernel<<<vblocks(H->iface->nk), kVT, 0, s>>>(u, buf, H->iface->start.ptr,
                                                               H->iface->pos.ptr, H->iface->nk);
  return vec_done(H, "iface_scatter");
}
