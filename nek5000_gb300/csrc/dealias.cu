// dealias.cu -- the convective term with dealiasing (convop with
// param(99) = 4, core/navier1.f:3196-3204 -> convect_new, core/convect.f:
// 639-725): the field and the convecting velocity are interpolated from the
// lx1 GLL points to lxd Gauss points per direction (intp_rstd, :346), the
// field differentiated there, contracted with the metric terms interpolated
// to the Gauss points and weighted by the Gauss weights (set_dealias_rx,
// core/convect2.f:120-175), projected back by the transposed interpolation,
// and divided by bm1.  FP64; one block per element for every tensor step.
// nekgpu_dealias_setup builds the matrices and the fine metric terms once.
#include <cmath>
#include <string>
#include <vector>

#include "impl.cuh"

namespace nekgpu {

struct Dealias {
  int md = 0;
  DevBuf<double> J, Jt, Dd, rxd, wd3;     // rxd: [q][nel][md^3]
  DevBuf<double> uf, fx, fy, fz, uo;      // fine scratch, md^3 nel each
};

void DealiasDeleter::operator()(Dealias* p) const { delete p; }

namespace {

// Gauss-Legendre points and weights: roots of P_m by Newton from the
// Chebyshev guesses, weights 2 / ((1 - x^2) P'_m(x)^2)
void gauss(int m, std::vector<double>& z, std::vector<double>& w) {
  z.assign(m, 0.0);
  w.assign(m, 0.0);
  for (int i = 0; i < m; ++i) {
    double x = -std::cos(M_PI * (i + 0.75) / (m + 0.5)), dp = 1.0;
    for (int it = 0; it < 100; ++it) {
      double p0 = 1.0, p1 = x;
      for (int k = 1; k < m; ++k) {
        const double p2 = ((2 * k + 1) * x * p1 - k * p0) / (k + 1);
        p0 = p1;
        p1 = p2;
      }
      dp = m * (x * p1 - p0) / (x * x - 1.0);
      const double dx = p1 / dp;
      x -= dx;
      if (std::fabs(dx) < 1e-16) break;
    }
    z[i] = x;
    w[i] = 2.0 / ((1.0 - x * x) * dp * dp);
  }
}

// GLL points (roots of (1 - x^2) P'_N)
void gll_points(int np, std::vector<double>& z) {
  const int N = np - 1;
  z.assign(np, 0.0);
  for (int i = 0; i < np; ++i) {
    double x = -std::cos(M_PI * i / N);
    for (int it = 0; it < 100 && i > 0 && i < N; ++it) {
      double p0 = 1.0, p1 = x;
      for (int k = 1; k < N; ++k) {
        const double p2 = ((2 * k + 1) * x * p1 - k * p0) / (k + 1);
        p0 = p1;
        p1 = p2;
      }
      const double dx = (x * p1 - p0) / ((N + 1) * p1);
      x -= dx;
      if (std::fabs(dx) < 1e-16) break;
    }
    z[i] = x;
  }
  z[0] = -1.0;
  z[N] = 1.0;
}

// Lagrange interpolation weights of the nodes x at xx, and their derivatives
void lagrange(double xx, const std::vector<double>& x, double* l, double* dl) {
  const int n = (int)x.size();
  for (int j = 0; j < n; ++j) {
    double p = 1.0, d = 0.0;
    for (int m = 0; m < n; ++m) {
      if (m == j) continue;
      const double f = (xx - x[m]) / (x[j] - x[m]);
      d = d * f + p / (x[j] - x[m]);
      p *= f;
    }
    l[j] = p;
    if (dl) dl[j] = d;
  }
}

// out (nb^3 per element) = [A (x) A (x) A] in (na^3 per element); A nb x na
// column-major.  smem: na^3 + nb na^2 + nb^2 na + nb na doubles.
__global__ void __launch_bounds__(256) tensor3_kernel(double* __restrict__ out,
                                                      const double* __restrict__ in,
                                                      const double* __restrict__ A, int na,
                                                      int nb) {
  extern __shared__ __align__(128) unsigned char dl_smem[];
  const int na3 = na * na * na, nb3 = nb * nb * nb;
  double* u = reinterpret_cast<double*>(dl_smem);
  double* w1 = u + na3;
  double* w2 = w1 + nb * na * na;
  double* sA = w2 + nb * nb * na;
  const int64_t e = blockIdx.x;
  for (int q = threadIdx.x; q < na3; q += blockDim.x) u[q] = in[e * na3 + q];
  for (int q = threadIdx.x; q < nb * na; q += blockDim.x) sA[q] = A[q];
  __syncthreads();
  for (int q = threadIdx.x; q < nb * na * na; q += blockDim.x) {
    const int i = q % nb, jk = q / nb;
    double s = 0.0;
    for (int l = 0; l < na; ++l) s += sA[i + nb * l] * u[l + na * jk];
    w1[q] = s;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < nb * nb * na; q += blockDim.x) {
    const int i = q % nb, j = (q / nb) % nb, k = q / (nb * nb);
    double s = 0.0;
    for (int l = 0; l < na; ++l) s += sA[j + nb * l] * w1[i + nb * (l + na * k)];
    w2[q] = s;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < nb3; q += blockDim.x) {
    const int ij = q % (nb * nb), k = q / (nb * nb);
    double s = 0.0;
    for (int l = 0; l < na; ++l) s += sA[k + nb * l] * w2[ij + nb * nb * l];
    out[e * nb3 + q] = s;
  }
}

__global__ void scale_w3_kernel(double* __restrict__ a, const double* __restrict__ w3, int md3,
                                int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    a[i] *= w3[i % md3];
}

// on the Gauss grid: uo = tr_1 u_r + tr_2 u_s + tr_3 u_t with tr_m = sum_c
// rxd(m, c) f_c.  smem: md^3 + md^2 doubles.
__global__ void __launch_bounds__(256) conv_fine_kernel(double* __restrict__ uo,
                                                        const double* __restrict__ uf,
                                                        const double* __restrict__ fx,
                                                        const double* __restrict__ fy,
                                                        const double* __restrict__ fz,
                                                        const double* __restrict__ rxd,
                                                        const double* __restrict__ Dd, int md,
                                                        int64_t nd) {
  extern __shared__ __align__(128) unsigned char dl_smem[];
  const int md3 = md * md * md;
  double* su = reinterpret_cast<double*>(dl_smem);
  double* sD = su + md3;
  const int64_t e = blockIdx.x, eo = e * md3;
  for (int q = threadIdx.x; q < md3; q += blockDim.x) su[q] = uf[eo + q];
  for (int q = threadIdx.x; q < md * md; q += blockDim.x) sD[q] = Dd[q];
  __syncthreads();
  for (int q = threadIdx.x; q < md3; q += blockDim.x) {
    const int i = q % md, j = (q / md) % md, k = q / (md * md);
    double ur = 0.0, us = 0.0, ut = 0.0;
    for (int l = 0; l < md; ++l) {
      ur += sD[i + md * l] * su[l + md * (j + md * k)];
      us += sD[j + md * l] * su[i + md * (l + md * k)];
      ut += sD[k + md * l] * su[i + md * (j + md * l)];
    }
    const int64_t g = eo + q;
    const double x = fx[g], y = fy[g], z = fz[g];
    const double t1 = rxd[g] * x + rxd[nd + g] * y + rxd[2 * nd + g] * z;
    const double t2 = rxd[3 * nd + g] * x + rxd[4 * nd + g] * y + rxd[5 * nd + g] * z;
    const double t3 = rxd[6 * nd + g] * x + rxd[7 * nd + g] * y + rxd[8 * nd + g] * z;
    uo[g] = t1 * ur + t2 * us + t3 * ut;
  }
}

// conservative form on the Gauss grid: cu = sum_d (D_r p_d rxd(d) + D_s p_d
// rxd(d+3) + D_t p_d rxd(d+6)), p_d = f_d uf (convect_cons).  smem:
// 3 md^3 + md^2 doubles.
__global__ void __launch_bounds__(256) conv_cons_fine_kernel(double* __restrict__ cu,
                                                             const double* __restrict__ uf,
                                                             const double* __restrict__ fx,
                                                             const double* __restrict__ fy,
                                                             const double* __restrict__ fz,
                                                             const double* __restrict__ rxd,
                                                             const double* __restrict__ Dd,
                                                             int md, int64_t nd) {
  extern __shared__ __align__(128) unsigned char dl_smem[];
  const int md3 = md * md * md;
  double* sp = reinterpret_cast<double*>(dl_smem);  // [d][md^3]
  double* sD = sp + 3 * md3;
  const int64_t e = blockIdx.x, eo = e * md3;
  for (int q = threadIdx.x; q < md3; q += blockDim.x) {
    const double u = uf[eo + q];
    sp[q] = fx[eo + q] * u;
    sp[md3 + q] = fy[eo + q] * u;
    sp[2 * md3 + q] = fz[eo + q] * u;
  }
  for (int q = threadIdx.x; q < md * md; q += blockDim.x) sD[q] = Dd[q];
  __syncthreads();
  for (int q = threadIdx.x; q < md3; q += blockDim.x) {
    const int i = q % md, j = (q / md) % md, k = q / (md * md);
    const int64_t g = eo + q;
    double acc = 0.0;
    for (int d = 0; d < 3; ++d) {
      const double* p = sp + d * md3;
      double a = 0.0, b = 0.0, t = 0.0;
      for (int l = 0; l < md; ++l) {
        a += sD[i + md * l] * p[l + md * (j + md * k)];
        b += sD[j + md * l] * p[i + md * (l + md * k)];
        t += sD[k + md * l] * p[i + md * (j + md * l)];
      }
      acc = acc + a * rxd[d * nd + g] + b * rxd[(d + 3) * nd + g] + t * rxd[(d + 6) * nd + g];
    }
    cu[g] = acc;
  }
}

__global__ void div_by_kernel(double* __restrict__ a, const double* __restrict__ b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    a[i] = a[i] / b[i];
}

size_t t3_smem(int na, int nb) {
  return sizeof(double) * ((size_t)na * na * na + (size_t)nb * na * na + (size_t)nb * nb * na +
                           (size_t)nb * na);
}

int vgrid(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 152 * 8); }

}  // namespace

int dealias_setup(Handle& h, int lxd, std::string& err) {
  Mesh& M = h.mesh;
  const int mx = M.nx1, md = lxd;
  if (md < mx || md > 18) {  // shared memory of the tensor steps: at most 142 KB
    err = "dealias: lxd must be between lx1 and 18";
    return NEKGPU_EINVAL;
  }
  std::unique_ptr<Dealias, DealiasDeleter> d(new Dealias());
  d->md = md;
  std::vector<double> zg, zd, wd;
  gll_points(mx, zg);
  gauss(md, zd, wd);
  std::vector<double> J((size_t)md * mx), Jt((size_t)md * mx), Dd((size_t)md * md), l(32), dl(32);
  for (int i = 0; i < md; ++i) {
    lagrange(zd[i], zg, l.data(), nullptr);
    for (int j = 0; j < mx; ++j) J[i + (size_t)md * j] = l[j];
    lagrange(zd[i], zd, l.data(), dl.data());
    for (int j = 0; j < md; ++j) Dd[i + (size_t)md * j] = dl[j];
  }
  for (int i = 0; i < md; ++i)
    for (int j = 0; j < mx; ++j) Jt[j + (size_t)mx * i] = J[i + (size_t)md * j];
  std::vector<double> w3((size_t)md * md * md);
  for (int k = 0; k < md; ++k)
    for (int j = 0; j < md; ++j)
      for (int i = 0; i < md; ++i) w3[i + (size_t)md * (j + (size_t)md * k)] = wd[i] * wd[j] * wd[k];
  const int64_t nd = (int64_t)md * md * md * M.nel;
  if (d->J.ensure(J.size()) || d->Jt.ensure(Jt.size()) || d->Dd.ensure(Dd.size()) ||
      d->wd3.ensure(w3.size()) || d->rxd.ensure((size_t)9 * nd) || d->uf.ensure(nd) ||
      d->fx.ensure(nd) || d->fy.ensure(nd) || d->fz.ensure(nd) || d->uo.ensure(nd)) {
    err = "dealias: device allocation failed";
    return NEKGPU_ENOMEM;
  }
  cudaStream_t s = h.stream;
  cudaMemcpyAsync(d->J.ptr, J.data(), J.size() * 8, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d->Jt.ptr, Jt.data(), Jt.size() * 8, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d->Dd.ptr, Dd.data(), Dd.size() * 8, cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(d->wd3.ptr, w3.data(), w3.size() * 8, cudaMemcpyHostToDevice, s);
  const size_t sm = t3_smem(mx, md);
  cudaFuncSetAttribute(tensor3_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)t3_smem(18, 18));
  cudaFuncSetAttribute(conv_fine_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)(sizeof(double) * (18 * 18 * 18 + 18 * 18)));
  cudaFuncSetAttribute(conv_cons_fine_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)(sizeof(double) * (3 * 18 * 18 * 18 + 18 * 18)));
  for (int q = 0; q < 9; ++q) {  // set_dealias_rx
    count_launch(2);
    tensor3_kernel<<<M.nel, 256, sm, s>>>(d->rxd.ptr + q * nd, M.rst.ptr + (int64_t)q * M.n,
                                          d->J.ptr, mx, md);
    scale_w3_kernel<<<vgrid(nd), 256, 0, s>>>(d->rxd.ptr + q * nd, d->wd3.ptr, md * md * md, nd);
  }
  const cudaError_t e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) {
    err = std::string("dealias setup: ") + cudaGetErrorString(e);
    return NEKGPU_ECUDA;
  }
  h.dealias = std::move(d);
  return NEKGPU_OK;
}

int dealias_lxd(const Handle& h) { return h.dealias ? h.dealias->md : 0; }

int convect_cons_dealias(Handle& h, double* conv, const double* u, const double* vx,
                         const double* vy, const double* vz) {
  Mesh& M = h.mesh;
  Dealias& d = *h.dealias;
  const int mx = M.nx1, md = d.md;
  const int64_t nd = (int64_t)md * md * md * M.nel;
  cudaStream_t s = h.stream;
  const size_t sf = t3_smem(mx, md), sb = t3_smem(md, mx);
  count_launch(7);
  tensor3_kernel<<<M.nel, 256, sf, s>>>(d.uf.ptr, u, d.J.ptr, mx, md);
  tensor3_kernel<<<M.nel, 256, sf, s>>>(d.fx.ptr, vx, d.J.ptr, mx, md);
  tensor3_kernel<<<M.nel, 256, sf, s>>>(d.fy.ptr, vy, d.J.ptr, mx, md);
  tensor3_kernel<<<M.nel, 256, sf, s>>>(d.fz.ptr, vz, d.J.ptr, mx, md);
  conv_cons_fine_kernel<<<M.nel, 256, sizeof(double) * (3 * (size_t)md * md * md + md * md), s>>>(
      d.uo.ptr, d.uf.ptr, d.fx.ptr, d.fy.ptr, d.fz.ptr, d.rxd.ptr, d.Dd.ptr, md, nd);
  tensor3_kernel<<<M.nel, 256, sb, s>>>(conv, d.uo.ptr, d.Jt.ptr, md, mx);
  div_by_kernel<<<vgrid(M.n), 256, 0, s>>>(conv, M.f64.bm1, M.n);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

int convop_dealias(Handle& h, double* conv, const double* u, const double* vx, const double* vy,
                   const double* vz) {
  Mesh& M = h.mesh;
  Dealias& d = *h.dealias;
  const int mx = M.nx1, md = d.md;
  const int64_t nd = (int64_t)md * md * md * M.nel;
  cudaStream_t s = h.stream;
  const size_t sf = t3_smem(mx, md), sb = t3_smem(md, mx);
  count_launch(7);
  tensor3_kernel<<<M.nel, 256, sf, s>>>(d.uf.ptr, u, d.J.ptr, mx, md);
  tensor3_kernel<<<M.nel, 256, sf, s>>>(d.fx.ptr, vx, d.J.ptr, mx, md);
  tensor3_kernel<<<M.nel, 256, sf, s>>>(d.fy.ptr, vy, d.J.ptr, mx, md);
  tensor3_kernel<<<M.nel, 256, sf, s>>>(d.fz.ptr, vz, d.J.ptr, mx, md);
  conv_fine_kernel<<<M.nel, 256, sizeof(double) * ((size_t)md * md * md + md * md), s>>>(
      d.uo.ptr, d.uf.ptr, d.fx.ptr, d.fy.ptr, d.fz.ptr, d.rxd.ptr, d.Dd.ptr, md, nd);
  tensor3_kernel<<<M.nel, 256, sb, s>>>(conv, d.uo.ptr, d.Jt.ptr, md, mx);
  div_by_kernel<<<vgrid(M.n), 256, 0, s>>>(conv, M.f64.bm1, M.n);
  return cudaGetLastError() == cudaSuccess ? 0 : -3;
}

}  // namespace nekgpu

// ---------------------------------------------------------------------------
// C ABI
namespace nekgpu {
Handle* handle_lookup(const int64_t* h);
int handle_fail(Handle* H, int code, const std::string& msg);
}  // namespace nekgpu

using namespace nekgpu;

extern "C" int nekgpu_dealias_setup(const int64_t* handle, const int* lxd) {
  Handle* H = handle_lookup(handle);
  if (!H) return handle_fail(nullptr, NEKGPU_EHANDLE, "unknown handle");
  if (handle_enter(*H) != cudaSuccess)
    return handle_fail(H, NEKGPU_ECUDA, "call entry failed");
  if (!H->has_mesh || !H->mesh.has_rst)
    return handle_fail(H, NEKGPU_ENOSETUP,
                       "metric terms not set up (the geometry must come from coordinates)");
  if (!lxd) return handle_fail(H, NEKGPU_EINVAL, "null argument");
  std::string err;
  const int rc = dealias_setup(*H, *lxd, err);
  return rc ? handle_fail(H, rc, err) : NEKGPU_OK;
}

extern "C" int nekgpu_convop_dev(const int64_t* handle, double* conv, const double* u,
                                 const double* vx, const double* vy, const double* vz) {
  Handle* H = handle_lookup(handle);
  if (!H) return handle_fail(nullptr, NEKGPU_EHANDLE, "unknown handle");
  if (handle_enter(*H) != cudaSuccess)
    return handle_fail(H, NEKGPU_ECUDA, "call entry failed");
  if (!H->has_mesh || !H->mesh.has_rst)
    return handle_fail(H, NEKGPU_ENOSETUP,
                       "metric terms not set up (the geometry must come from coordinates)");
  if (!conv || !u || !vx || !vy || !vz) return handle_fail(H, NEKGPU_EINVAL, "null argument");
  const int rc = H->dealias ? convop_dealias(*H, conv, u, vx, vy, vz)
                            : launch_conv1(*H, conv, u, vx, vy, vz);
  const cudaError_t e = handle_leave(*H);  // finished before the call returns
  if (e != cudaSuccess)
    return handle_fail(H, NEKGPU_ECUDA, std::string("convop: ") + cudaGetErrorString(e));
  if (rc) return handle_fail(H, NEKGPU_ECUDA, "convop failed");
  return NEKGPU_OK;
}

extern "C" int nekgpu_convect_cons_dev(const int64_t* handle, double* conv, const double* u,
                                       const double* vx, const double* vy, const double* vz) {
  Handle* H = handle_lookup(handle);
  if (!H) return handle_fail(nullptr, NEKGPU_EHANDLE, "unknown handle");
  if (handle_enter(*H) != cudaSuccess)
    return handle_fail(H, NEKGPU_ECUDA, "call entry failed");
  if (!H->has_mesh || !H->dealias)
    return handle_fail(H, NEKGPU_ENOSETUP, "dealiasing not set up (nekgpu_dealias_setup)");
  if (!conv || !u || !vx || !vy || !vz) return handle_fail(H, NEKGPU_EINVAL, "null argument");
  const int rc = convect_cons_dealias(*H, conv, u, vx, vy, vz);
  const cudaError_t e = handle_leave(*H);  // finished before the call returns
  if (e != cudaSuccess)
    return handle_fail(H, NEKGPU_ECUDA, std::string("convect_cons: ") + cudaGetErrorString(e));
  if (rc) return handle_fail(H, NEKGPU_ECUDA, "convect_cons failed");
  return NEKGPU_OK;
}
