// amg.cu -- the algebraic multigrid coarse solve on the device: the
// hierarchy of amg_plan.cpp applied as the reference's amg_exec
// (core/crs_amg.c:129-186) and crs_solve (:186-203), one launch per sparse
// product or vector pass, levels in turn.  Used by the pressure
// preconditioner when its coarse solve is AMG (NEKGPU_OPT_COARSE = 1, the
// reference's param(40) = 1) and by the crs_amg-style entry points
// nekgpu_crs_amg_setup / nekgpu_crs_amg_solve_dev.
#include <algorithm>
#include <vector>

#include "h1mg.h"
#include "impl.cuh"

namespace nekgpu {

struct AmgDevLevel {
  int64_t nf = 0, nc = 0, off = 0, offc = 0;
  int m = 1;
  double rho = 0.0;
  DevBuf<double> dff;
  DevBuf<int64_t> w_ptr, wt_ptr, afc_ptr, aff_ptr;
  DevBuf<int> w_idx, wt_idx, afc_idx, aff_idx;
  DevBuf<double> w_val, wt_val, afc_val, aff_val;
};

struct AmgDev {
  int64_t n = 0, nfmax = 0;
  std::vector<AmgDevLevel> lev;
  DevBuf<int> perm;  // perm[k] = unknown at plan position k
  DevBuf<double> b, x, c, cold, r;
};

void AmgDevDeleter::operator()(AmgDev* p) const { delete p; }

namespace {

constexpr int kT = 256;

inline int grid(int64_t n) {
  return (int)std::min<int64_t>(std::max<int64_t>((n + kT - 1) / kT, 1), 152 * 8);
}
inline int warp_grid(int64_t rows) { return (int)std::max<int64_t>((rows * 32 + kT - 1) / kT, 1); }

// out[r] = alpha y[r] + beta sum_q val[q] in[idx[q]] (one warp per row, lanes
// strided, fixed shuffle tree: the same order every run).  y may alias out.
__global__ void amg_spmv_kernel(double* out, double alpha, const double* y, double beta,
                                const int64_t* __restrict__ ptr, const int* __restrict__ idx,
                                const double* __restrict__ val, const double* __restrict__ in,
                                int64_t rows) {
  const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= rows) return;
  double acc = 0.0;
  for (int64_t q = ptr[row] + lane; q < ptr[row + 1]; q += 32) acc += val[q] * in[idx[q]];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) out[row] = (alpha != 0.0 ? alpha * y[row] : 0.0) + beta * acc;
}

__global__ void amg_gather_kernel(double* __restrict__ b, const double* __restrict__ v,
                                  const int* __restrict__ perm, int64_t n) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x)
    b[k] = v[perm[k]];
}

__global__ void amg_scatter_kernel(double* __restrict__ v, const double* __restrict__ x,
                                   const int* __restrict__ perm, int64_t n) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x)
    v[perm[k]] = x[k];
}

// c = d b
__global__ void amg_jacobi_kernel(double* __restrict__ c, const double* __restrict__ d,
                                  const double* __restrict__ b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    c[i] = d[i] * b[i];
}

// c = beta (cold + d r) - gamma c   (gamma = 0: c = beta (cold + d r))
__global__ void amg_cheb_kernel(double* __restrict__ c, const double* __restrict__ cold,
                                const double* __restrict__ d, const double* __restrict__ r,
                                double beta, double gamma, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double t = beta * (cold[i] + d[i] * r[i]);
    c[i] = gamma != 0.0 ? t - gamma * c[i] : t;
  }
}

__global__ void amg_add_kernel(double* __restrict__ x, const double* __restrict__ c, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] += c[i];
}

__global__ void amg_bottom_kernel(double* __restrict__ x, const double* __restrict__ d,
                                  const double* __restrict__ b) {
  x[0] = d[0] * b[0];
}

// crs_solve's null space: the pinned last unknown 0, then the mean removed.
// One block.
__global__ void crs_mean_kernel(double* __restrict__ x, int64_t n, int pin) {
  __shared__ double red[32];
  if (pin && threadIdx.x == 0) x[n - 1] = 0.0;
  __syncthreads();
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) s += x[i];
  s = block_sum(s, red);
  const double mean = s / (double)n;
  for (int64_t i = threadIdx.x; i < n; i += blockDim.x) x[i] -= mean;
}

template <typename T>
int up(DevBuf<T>& d, const std::vector<T>& v, cudaStream_t s) {
  if (d.ensure(std::max<size_t>(v.size(), 1))) return -4;
  if (!v.empty() &&
      cudaMemcpyAsync(d.ptr, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s) !=
          cudaSuccess)
    return -3;
  return 0;
}

}  // namespace

int amg_upload(const AmgPlan& p, std::unique_ptr<AmgDev, AmgDevDeleter>& out, cudaStream_t s) {
  std::unique_ptr<AmgDev, AmgDevDeleter> a(new AmgDev());
  a->n = p.n;
  std::vector<int> perm(p.perm.begin(), p.perm.end());
  if (up(a->perm, perm, s)) return -4;
  a->lev.resize(p.lev.size());
  for (size_t l = 0; l < p.lev.size(); ++l) {
    const AmgLevel& L = p.lev[l];
    AmgDevLevel& D = a->lev[l];
    D.nf = L.nf;
    D.nc = L.nc;
    D.off = p.off[l];
    D.offc = p.off[l + 1];
    D.m = L.cheb_m;
    D.rho = L.cheb_rho;
    a->nfmax = std::max(a->nfmax, L.nf);
    int rc = up(D.dff, L.dff, s);
    if (!rc && L.nc > 0) {
      rc = up(D.w_ptr, L.w_ptr, s) | up(D.w_idx, L.w_idx, s) | up(D.w_val, L.w_val, s) |
           up(D.wt_ptr, L.wt_ptr, s) | up(D.wt_idx, L.wt_idx, s) | up(D.wt_val, L.wt_val, s) |
           up(D.afc_ptr, L.afc_ptr, s) | up(D.afc_idx, L.afc_idx, s) |
           up(D.afc_val, L.afc_val, s) | up(D.aff_ptr, L.aff_ptr, s) |
           up(D.aff_idx, L.aff_idx, s) | up(D.aff_val, L.aff_val, s);
    }
    if (rc) return -4;
  }
  const size_t nn = (size_t)std::max<int64_t>(p.n, 1), nf = (size_t)std::max<int64_t>(a->nfmax, 1);
  if (a->b.ensure(nn) || a->x.ensure(nn) || a->c.ensure(nf) || a->cold.ensure(nf) ||
      a->r.ensure(nf))
    return -4;
  out = std::move(a);
  return 0;
}

// y = (one V-cycle of the hierarchy) v, both in the unknowns' order (n each).
void amg_apply_dev(AmgDev& a, double* y, const double* v, cudaStream_t s) {
  const int64_t n = a.n;
  if (n == 0) return;
  count_launch();
  amg_gather_kernel<<<grid(n), kT, 0, s>>>(a.b.ptr, v, a.perm.ptr, n);
  const int nl = (int)a.lev.size();
  for (int l = 0; l + 1 < nl; ++l) {  // b_{l+1} += W^T b_l
    AmgDevLevel& L = a.lev[l];
    count_launch();
    amg_spmv_kernel<<<warp_grid(L.nc), kT, 0, s>>>(a.b.ptr + L.offc, 1.0, a.b.ptr + L.offc, 1.0,
                                                   L.wt_ptr.ptr, L.wt_idx.ptr, L.wt_val.ptr,
                                                   a.b.ptr + L.off, L.nc);
  }
  {
    AmgDevLevel& B = a.lev[nl - 1];
    count_launch();
    amg_bottom_kernel<<<1, 1, 0, s>>>(a.x.ptr + B.off, B.dff.ptr, a.b.ptr + B.off);
  }
  for (int l = nl - 2; l >= 0; --l) {
    AmgDevLevel& L = a.lev[l];
    double* bl = a.b.ptr + L.off;
    double* xl = a.x.ptr + L.off;
    const double* xc = a.x.ptr + L.offc;
    const int64_t nf = L.nf;
    double* c = a.c.ptr;
    double* cold = a.cold.ptr;
    double* r = a.r.ptr;
    count_launch(3);
    amg_spmv_kernel<<<warp_grid(nf), kT, 0, s>>>(xl, 0.0, xl, 1.0, L.w_ptr.ptr, L.w_idx.ptr,
                                                 L.w_val.ptr, xc, nf);  // x_l = W x_c
    amg_spmv_kernel<<<warp_grid(nf), kT, 0, s>>>(bl, 1.0, bl, -1.0, L.afc_ptr.ptr, L.afc_idx.ptr,
                                                 L.afc_val.ptr, xc, nf);  // b_l -= AfP x_c
    amg_jacobi_kernel<<<grid(nf), kT, 0, s>>>(c, L.dff.ptr, bl, nf);     // c_1 = D b_l
    double alpha = 0.0, beta = 0.0, gamma = 0.0;
    if (L.m > 1) {
      alpha = L.rho / 2.0;
      alpha *= alpha;
      gamma = 2.0 * alpha / (1.0 - 2.0 * alpha);
      beta = 1.0 + gamma;
      count_launch(2);
      amg_spmv_kernel<<<warp_grid(nf), kT, 0, s>>>(r, 1.0, bl, -1.0, L.aff_ptr.ptr,
                                                   L.aff_idx.ptr, L.aff_val.ptr, c, nf);
      std::swap(c, cold);
      amg_cheb_kernel<<<grid(nf), kT, 0, s>>>(c, cold, L.dff.ptr, r, beta, 0.0, nf);
    }
    for (int ci = 3; ci <= L.m; ++ci) {
      gamma = alpha * beta;
      gamma = gamma / (1.0 - gamma);
      beta = 1.0 + gamma;
      count_launch(2);
      amg_spmv_kernel<<<warp_grid(nf), kT, 0, s>>>(r, 1.0, bl, -1.0, L.aff_ptr.ptr,
                                                   L.aff_idx.ptr, L.aff_val.ptr, c, nf);
      std::swap(c, cold);
      amg_cheb_kernel<<<grid(nf), kT, 0, s>>>(c, cold, L.dff.ptr, r, beta, gamma, nf);
    }
    count_launch();
    amg_add_kernel<<<grid(nf), kT, 0, s>>>(xl, c, nf);
  }
  count_launch();
  amg_scatter_kernel<<<grid(n), kT, 0, s>>>(y, a.x.ptr, a.perm.ptr, n);
}

}  // namespace nekgpu

// ---------------------------------------------------------------------------
// C ABI: the reference's crs_amg interface (core/crs_amg.c:531 setup, :186
// solve) on a handle.
namespace nekgpu {
Handle* handle_lookup(const int64_t* h);
int handle_fail(Handle* H, int code, const std::string& msg);
}  // namespace nekgpu

using namespace nekgpu;

extern "C" int nekgpu_crs_amg_setup(const int64_t* handle, const int64_t* n, const int64_t* nz,
                                    const int* ai, const int* aj, const double* av,
                                    const int* null_space) {
  Handle* H = handle_lookup(handle);
  if (!H) return handle_fail(nullptr, NEKGPU_EHANDLE, "unknown handle");
  if (handle_enter(*H) != cudaSuccess) return handle_fail(H, NEKGPU_ECUDA, "call entry failed");
  if (!n || !nz || *n < 1 || *nz < 0 || (*nz > 0 && (!ai || !aj || !av)))
    return handle_fail(H, NEKGPU_EINVAL, "bad argument");
  const bool ns = null_space && *null_space != 0;
  // the singular (null-space) matrix loses its last unknown, pinned to 0, as
  // the X X^T form of the coarse solve does
  const int64_t m = ns ? *n - 1 : *n;
  std::vector<std::vector<std::pair<int, double>>> rows((size_t)std::max<int64_t>(m, 0));
  for (int64_t q = 0; q < *nz; ++q) {
    const int i = ai[q], j = aj[q];
    if (i < 0 || j < 0 || i >= *n || j >= *n)
      return handle_fail(H, NEKGPU_EINVAL, "crs_amg_setup: index out of range");
    if (i < m && j < m) rows[(size_t)i].push_back({j, av[q]});
  }
  std::vector<int64_t> ptr((size_t)m + 1, 0);
  std::vector<int> idx;
  std::vector<double> val;
  for (int64_t r = 0; r < m; ++r) {  // duplicates summed in the given order
    auto& v = rows[(size_t)r];
    std::stable_sort(v.begin(), v.end(),
                     [](const std::pair<int, double>& a, const std::pair<int, double>& b) {
                       return a.first < b.first;
                     });
    for (size_t q = 0; q < v.size();) {
      double a = 0.0;
      const int c = v[q].first;
      for (; q < v.size() && v[q].first == c; ++q) a += v[q].second;
      idx.push_back(c);
      val.push_back(a);
    }
    ptr[(size_t)r + 1] = (int64_t)idx.size();
  }
  AmgPlan p;
  std::string err;
  int rc = m > 0 ? amg_setup(p, m, ptr, idx, val, err) : 0;
  if (rc) return handle_fail(H, rc, err);
  std::unique_ptr<AmgDev, AmgDevDeleter> a;
  if (m > 0 && amg_upload(p, a, H->stream)) return handle_fail(H, NEKGPU_ENOMEM, "crs_amg_setup: upload failed");
  if (cudaStreamSynchronize(H->stream) != cudaSuccess)
    return handle_fail(H, NEKGPU_ECUDA, "crs_amg_setup: upload failed");
  H->crs_amg = std::move(a);
  H->crs_n = *n;
  H->crs_null = ns;
  return NEKGPU_OK;
}

extern "C" int nekgpu_crs_amg_solve_dev(const int64_t* handle, double* x, const double* b) {
  Handle* H = handle_lookup(handle);
  if (!H) return handle_fail(nullptr, NEKGPU_EHANDLE, "unknown handle");
  if (handle_enter(*H) != cudaSuccess) return handle_fail(H, NEKGPU_ECUDA, "call entry failed");
  if (!H->crs_n) return handle_fail(H, NEKGPU_ENOSETUP, "crs_amg not set up (nekgpu_crs_amg_setup)");
  if (!x || !b) return handle_fail(H, NEKGPU_EINVAL, "null argument");
  cudaStream_t s = H->stream;
  if (H->crs_amg) amg_apply_dev(*H->crs_amg, x, b, s);
  if (H->crs_null) {  // crs_solve (core/crs_amg.c:194-198): the mean removed
    count_launch();
    crs_mean_kernel<<<1, 1024, 0, s>>>(x, H->crs_n, 1);
  }
  const cudaError_t e = handle_leave(*H);
  if (e != cudaSuccess) return handle_fail(H, NEKGPU_ECUDA, std::string("crs_amg_solve: ") + cudaGetErrorString(e));
  return NEKGPU_OK;
}
