// gradops.cu -- the gradient-type operators of the PN-PN splitting step on
// the device, in the reference's arithmetic order (each derivative a left-
// to-right sum over the inner index as mxm forms it, products and sums
// rounded one by one), so that they equal the Fortran's unfused FP64 values
// bit for bit:
//
//   wgradm1  core/navier1.f:4170-4230  u_x = w3 (u_r r_x + u_s s_x + u_t t_x)
//   cdtp     core/navier1.f:330-470    D^T (bm1 x / J times r_m, s_m, t_m)
//   dudxyz   core/navier1.f:1156-1220  (u_r r_m + u_s s_m + u_t t_m) / J
//   op_curl  core/plan4.f:368-430      curl from six dudxyz, averaged (bm1,
//                                      dssum, binvm1) when ifavg
//
// One block per element, thread (i, j) walks its z-column; the field and D
// sit in shared memory.  They need the metric terms the geometry keeps when
// it is formed from coordinates (nekgpu_setup_xyz / nekgpu_geom_update_dev).
#include <string>

#include "impl.cuh"

namespace nekgpu {
namespace {

// u_r, u_s, u_t at (i, j, k) of the element held in su (D row-major in sD)
template <int NX>
__device__ __forceinline__ void grad_at(const double* su, const double* sD, int i, int j, int k,
                                        double& ur, double& us, double& ut) {
  ur = __dmul_rn(sD[i * NX], su[NX * (j + NX * k)]);
  us = __dmul_rn(su[i + NX * NX * k], sD[j * NX]);
  ut = __dmul_rn(su[i + NX * j], sD[k * NX]);
#pragma unroll
  for (int l = 1; l < NX; ++l) {
    ur = __dadd_rn(ur, __dmul_rn(sD[i * NX + l], su[l + NX * (j + NX * k)]));
    us = __dadd_rn(us, __dmul_rn(su[i + NX * (l + NX * k)], sD[j * NX + l]));
    ut = __dadd_rn(ut, __dmul_rn(su[i + NX * (j + NX * l)], sD[k * NX + l]));
  }
}

__device__ __forceinline__ double dot3(double a1, double b1, double a2, double b2, double a3,
                                       double b3) {
  return __dadd_rn(__dadd_rn(__dmul_rn(a1, b1), __dmul_rn(a2, b2)), __dmul_rn(a3, b3));
}

template <int NX>
__global__ void __launch_bounds__(NX* NX) wgradm1_kernel(double* __restrict__ ux,
                                                         double* __restrict__ uy,
                                                         double* __restrict__ uz,
                                                         const double* __restrict__ u,
                                                         const double* __restrict__ rst,
                                                         const double* __restrict__ w3,
                                                         const double* __restrict__ D, int64_t n) {
  constexpr int P = NX * NX * NX;
  __shared__ double su[P], sD[NX * NX];
  const int64_t eo = (int64_t)blockIdx.x * P;
  const int tid = threadIdx.x;
  for (int q = tid; q < P; q += NX * NX) su[q] = u[eo + q];
  for (int q = tid; q < NX * NX; q += NX * NX) sD[q] = D[q];
  __syncthreads();
  const int i = tid % NX, j = tid / NX;
  for (int k = 0; k < NX; ++k) {
    const int pt = i + NX * (j + NX * k);
    const int64_t g = eo + pt;
    double ur, us, ut;
    grad_at<NX>(su, sD, i, j, k, ur, us, ut);
    const double w = w3[pt];
    ux[g] = __dmul_rn(w, dot3(ur, rst[g], us, rst[3 * n + g], ut, rst[6 * n + g]));
    uy[g] = __dmul_rn(w, dot3(ur, rst[n + g], us, rst[4 * n + g], ut, rst[7 * n + g]));
    uz[g] = __dmul_rn(w, dot3(ur, rst[2 * n + g], us, rst[5 * n + g], ut, rst[8 * n + g]));
  }
}

// du = (u_r r_m + u_s s_m + u_t t_m) * (1 / J), m = isd - 1 (x, y, z)
template <int NX>
__global__ void __launch_bounds__(NX* NX) dudxyz_kernel(double* __restrict__ du,
                                                        const double* __restrict__ u,
                                                        const double* __restrict__ rst,
                                                        const double* __restrict__ jac,
                                                        const double* __restrict__ D, int m,
                                                        int64_t n) {
  constexpr int P = NX * NX * NX;
  __shared__ double su[P], sD[NX * NX];
  const int64_t eo = (int64_t)blockIdx.x * P;
  const int tid = threadIdx.x;
  for (int q = tid; q < P; q += NX * NX) su[q] = u[eo + q];
  for (int q = tid; q < NX * NX; q += NX * NX) sD[q] = D[q];
  __syncthreads();
  const int i = tid % NX, j = tid / NX;
  const double *rm = rst + (int64_t)m * n, *sm = rst + (int64_t)(m + 3) * n,
               *tm = rst + (int64_t)(m + 6) * n;
  for (int k = 0; k < NX; ++k) {
    const int64_t g = eo + i + NX * (j + NX * k);
    double ur, us, ut;
    grad_at<NX>(su, sD, i, j, k, ur, us, ut);
    double v = __dmul_rn(ur, rm[g]);
    v = __dadd_rn(v, __dmul_rn(us, sm[g]));
    v = __dadd_rn(v, __dmul_rn(ut, tm[g]));
    du[g] = __dmul_rn(v, __ddiv_rn(1.0, jac[g]));
  }
}

// dtx = D_r^T (wx r_m) + D_s^T (wx s_m) + D_t^T (wx t_m), wx = bm1 x / J
template <int NX>
__global__ void __launch_bounds__(NX* NX) cdtp_kernel(double* __restrict__ dtx,
                                                      const double* __restrict__ x,
                                                      const double* __restrict__ rst,
                                                      const double* __restrict__ jac,
                                                      const double* __restrict__ bm1,
                                                      const double* __restrict__ D, int m,
                                                      int64_t n) {
  constexpr int P = NX * NX * NX;
  __shared__ double ta[P], tb[P], tc[P], sD[NX * NX];
  const int64_t eo = (int64_t)blockIdx.x * P;
  const int tid = threadIdx.x;
  const double *rm = rst + (int64_t)m * n, *sm = rst + (int64_t)(m + 3) * n,
               *tm = rst + (int64_t)(m + 6) * n;
  for (int q = tid; q < P; q += NX * NX) {
    const int64_t g = eo + q;
    const double wx = __ddiv_rn(__dmul_rn(bm1[g], x[g]), jac[g]);
    ta[q] = __dmul_rn(wx, rm[g]);
    tb[q] = __dmul_rn(wx, sm[g]);
    tc[q] = __dmul_rn(wx, tm[g]);
  }
  for (int q = tid; q < NX * NX; q += NX * NX) sD[q] = D[q];
  __syncthreads();
  const int i = tid % NX, j = tid / NX;
  for (int k = 0; k < NX; ++k) {
    // sum_l D(l,i) ta(l,j,k), sum_l tb(i,l,k) D(l,j), sum_l tc(i,j,l) D(l,k)
    double r = __dmul_rn(sD[i], ta[NX * (j + NX * k)]);
    double s = __dmul_rn(tb[i + NX * NX * k], sD[j]);
    double t = __dmul_rn(tc[i + NX * j], sD[k]);
#pragma unroll
    for (int l = 1; l < NX; ++l) {
      r = __dadd_rn(r, __dmul_rn(sD[l * NX + i], ta[l + NX * (j + NX * k)]));
      s = __dadd_rn(s, __dmul_rn(tb[i + NX * (l + NX * k)], sD[l * NX + j]));
      t = __dadd_rn(t, __dmul_rn(tc[i + NX * (j + NX * l)], sD[l * NX + k]));
    }
    dtx[eo + i + NX * (j + NX * k)] = __dadd_rn(__dadd_rn(r, s), t);
  }
}

// w1 = du3/dy - du2/dz, w2 = du1/dz - du3/dx, w3 = du2/dx - du1/dy
template <int NX>
__global__ void __launch_bounds__(NX* NX) curl_kernel(double* __restrict__ w1,
                                                      double* __restrict__ w2,
                                                      double* __restrict__ w3,
                                                      const double* __restrict__ u1,
                                                      const double* __restrict__ u2,
                                                      const double* __restrict__ u3,
                                                      const double* __restrict__ rst,
                                                      const double* __restrict__ jac,
                                                      const double* __restrict__ D, int64_t n) {
  constexpr int P = NX * NX * NX;
  __shared__ double s1[P], s2[P], s3[P], sD[NX * NX];
  const int64_t eo = (int64_t)blockIdx.x * P;
  const int tid = threadIdx.x;
  for (int q = tid; q < P; q += NX * NX) {
    s1[q] = u1[eo + q];
    s2[q] = u2[eo + q];
    s3[q] = u3[eo + q];
  }
  for (int q = tid; q < NX * NX; q += NX * NX) sD[q] = D[q];
  __syncthreads();
  const int i = tid % NX, j = tid / NX;
  for (int k = 0; k < NX; ++k) {
    const int64_t g = eo + i + NX * (j + NX * k);
    const double jm = __ddiv_rn(1.0, jac[g]);
    // d/dx_m of a field whose r, s, t derivatives are given
    auto dd = [&](double ur, double us, double ut, int m) {
      double v = __dmul_rn(ur, rst[(int64_t)m * n + g]);
      v = __dadd_rn(v, __dmul_rn(us, rst[(int64_t)(m + 3) * n + g]));
      v = __dadd_rn(v, __dmul_rn(ut, rst[(int64_t)(m + 6) * n + g]));
      return __dmul_rn(v, jm);
    };
    double a1r, a1s, a1t, a2r, a2s, a2t, a3r, a3s, a3t;
    grad_at<NX>(s1, sD, i, j, k, a1r, a1s, a1t);
    grad_at<NX>(s2, sD, i, j, k, a2r, a2s, a2t);
    grad_at<NX>(s3, sD, i, j, k, a3r, a3s, a3t);
    w1[g] = __dsub_rn(dd(a3r, a3s, a3t, 1), dd(a2r, a2s, a2t, 2));
    w2[g] = __dsub_rn(dd(a1r, a1s, a1t, 2), dd(a3r, a3s, a3t, 0));
    w3[g] = __dsub_rn(dd(a2r, a2s, a2t, 0), dd(a1r, a1s, a1t, 1));
  }
}

// du = (1/J) (vx (rx u_r + sx u_s + tx u_t) + vy (...) + vz (...))   (conv1)
template <int NX>
__global__ void __launch_bounds__(NX* NX) conv1_kernel(double* __restrict__ du,
                                                       const double* __restrict__ u,
                                                       const double* __restrict__ vx,
                                                       const double* __restrict__ vy,
                                                       const double* __restrict__ vz,
                                                       const double* __restrict__ rst,
                                                       const double* __restrict__ jac,
                                                       const double* __restrict__ D, int64_t n) {
  constexpr int P = NX * NX * NX;
  __shared__ double su[P], sD[NX * NX];
  const int64_t eo = (int64_t)blockIdx.x * P;
  const int tid = threadIdx.x;
  for (int q = tid; q < P; q += NX * NX) su[q] = u[eo + q];
  for (int q = tid; q < NX * NX; q += NX * NX) sD[q] = D[q];
  __syncthreads();
  const int i = tid % NX, j = tid / NX;
  for (int k = 0; k < NX; ++k) {
    const int64_t g = eo + i + NX * (j + NX * k);
    double ur, us, ut;
    grad_at<NX>(su, sD, i, j, k, ur, us, ut);
    const double a = dot3(rst[g], ur, rst[3 * n + g], us, rst[6 * n + g], ut);
    const double b = dot3(rst[n + g], ur, rst[4 * n + g], us, rst[7 * n + g], ut);
    const double c = dot3(rst[2 * n + g], ur, rst[5 * n + g], us, rst[8 * n + g], ut);
    const double sum = dot3(vx[g], a, vy[g], b, vz[g], c);
    du[g] = __dmul_rn(__ddiv_rn(1.0, jac[g]), sum);
  }
}

// dtfi = (D_r^T t_r + D_s^T t_s + D_t^T t_t) / bm1, t_q = w3 (((m_qx vx) fi +
// (m_qy vy) fi) + (m_qz vz) fi)   (conv2, core/navier1.f:1288-1388)
template <int NX>
__global__ void __launch_bounds__(NX* NX) conv2_kernel(double* __restrict__ dtfi,
                                                       const double* __restrict__ fi,
                                                       const double* __restrict__ vx,
                                                       const double* __restrict__ vy,
                                                       const double* __restrict__ vz,
                                                       const double* __restrict__ rst,
                                                       const double* __restrict__ w3,
                                                       const double* __restrict__ bm1,
                                                       const double* __restrict__ D, int64_t n) {
  constexpr int P = NX * NX * NX;
  __shared__ double ta[P], tb[P], tc[P], sD[NX * NX];
  const int64_t eo = (int64_t)blockIdx.x * P;
  const int tid = threadIdx.x;
  double* t3[3] = {ta, tb, tc};
  for (int q = tid; q < P; q += NX * NX) {
    const int64_t g = eo + q;
    const double f = fi[g], a1 = vx[g], a2 = vy[g], a3 = vz[g];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      double a = __dmul_rn(__dmul_rn(rst[(int64_t)(3 * d) * n + g], a1), f);
      a = __dadd_rn(a, __dmul_rn(__dmul_rn(rst[(int64_t)(3 * d + 1) * n + g], a2), f));
      a = __dadd_rn(a, __dmul_rn(__dmul_rn(rst[(int64_t)(3 * d + 2) * n + g], a3), f));
      t3[d][q] = __dmul_rn(a, w3[q]);
    }
  }
  for (int q = tid; q < NX * NX; q += NX * NX) sD[q] = D[q];
  __syncthreads();
  const int i = tid % NX, j = tid / NX;
  for (int k = 0; k < NX; ++k) {
    double r = __dmul_rn(sD[i], ta[NX * (j + NX * k)]);
    double s = __dmul_rn(tb[i + NX * NX * k], sD[j]);
    double t = __dmul_rn(tc[i + NX * j], sD[k]);
#pragma unroll
    for (int l = 1; l < NX; ++l) {
      r = __dadd_rn(r, __dmul_rn(sD[l * NX + i], ta[l + NX * (j + NX * k)]));
      s = __dadd_rn(s, __dmul_rn(tb[i + NX * (l + NX * k)], sD[l * NX + j]));
      t = __dadd_rn(t, __dmul_rn(tc[i + NX * (j + NX * l)], sD[l * NX + k]));
    }
    const int64_t g = eo + i + NX * (j + NX * k);
    dtfi[g] = __ddiv_rn(__dadd_rn(__dadd_rn(r, s), t), bm1[g]);
  }
}

// cmask (core/navier1.f:1390): c1 = 0, c2 = 1 on the points of flagged
// (outflow) faces, else 1 and 0; element-local
__global__ void cmask_kernel(double* __restrict__ c1, double* __restrict__ c2,
                             const int* __restrict__ ofc, int nx1) {
  const int64_t e = blockIdx.x, nxyz = (int64_t)nx1 * nx1 * nx1;
  const int N = nx1 - 1;
  const int* of = ofc + 6 * e;
  for (int q = threadIdx.x; q < nxyz; q += blockDim.x) {
    const int i = q % nx1, j = (q / nx1) % nx1, k = q / (nx1 * nx1);
    const bool on = (of[0] && j == 0) || (of[1] && i == N) || (of[2] && j == N) ||
                    (of[3] && i == 0) || (of[4] && k == 0) || (of[5] && k == N);
    c1[e * nxyz + q] = on ? 0.0 : 1.0;
    c2[e * nxyz + q] = on ? 1.0 : 0.0;
  }
}

// a = b c   (col3)
__global__ void col3_kernel(double* __restrict__ a, const double* __restrict__ b,
                            const double* __restrict__ c, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    a[i] = __dmul_rn(b[i], c[i]);
}

// conv = conv + coef (dm cmask)   (col3 then add2s2 / add2)
__global__ void acc_kernel(double* __restrict__ conv, const double* __restrict__ dm,
                           const double* __restrict__ cm, double coef, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    conv[i] = __dadd_rn(conv[i], __dmul_rn(coef, __dmul_rn(dm[i], cm[i])));
}

// bf = bf - bm1 ta   (subcol3)
__global__ void subcol3_kernel(double* __restrict__ bf, const double* __restrict__ bm1,
                               const double* __restrict__ ta, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    bf[i] = __dsub_rn(bf[i], __dmul_rn(bm1[i], ta[i]));
}

__global__ void mul_by_kernel(double* __restrict__ a, const double* __restrict__ b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    a[i] = __dmul_rn(a[i], b[i]);
}

int nblk(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 152 * 8); }

}  // namespace

// op: 0 wgradm1, 1 dudxyz, 2 cdtp, 3 curl.  Returns 0 or -1 (lx1 out of range).
int launch_gradop(Handle& h, int op, double* o1, double* o2, double* o3, const double* i1,
                  const double* i2, const double* i3, int m, const double* bm1) {
  Mesh& M = h.mesh;
  const int64_t n = M.n;
  cudaStream_t s = h.stream;
  const double *rst = M.rst.ptr, *jac = M.jac.ptr, *w3 = M.w3.ptr, *D = M.f64.D;
  count_launch();
  switch (M.nx1) {
#define NEKGPU_GRAD_CASE(N)                                                                    \
  case N:                                                                                      \
    if (op == 0)                                                                               \
      wgradm1_kernel<N><<<M.nel, N * N, 0, s>>>(o1, o2, o3, i1, rst, w3, D, n);                \
    else if (op == 1)                                                                          \
      dudxyz_kernel<N><<<M.nel, N * N, 0, s>>>(o1, i1, rst, jac, D, m, n);                     \
    else if (op == 2)                                                                          \
      cdtp_kernel<N><<<M.nel, N * N, 0, s>>>(o1, i1, rst, jac, bm1, D, m, n);                  \
    else                                                                                       \
      curl_kernel<N><<<M.nel, N * N, 0, s>>>(o1, o2, o3, i1, i2, i3, rst, jac, D, n);          \
    break;
    NEKGPU_GRAD_CASE(2)
    NEKGPU_GRAD_CASE(3)
    NEKGPU_GRAD_CASE(4)
    NEKGPU_GRAD_CASE(5)
    NEKGPU_GRAD_CASE(6)
    NEKGPU_GRAD_CASE(7)
    NEKGPU_GRAD_CASE(8)
    NEKGPU_GRAD_CASE(9)
    NEKGPU_GRAD_CASE(10)
    NEKGPU_GRAD_CASE(11)
    NEKGPU_GRAD_CASE(12)
#undef NEKGPU_GRAD_CASE
    default:
      return -1;
  }
  return 0;
}

int launch_conv1(Handle& h, double* du, const double* u, const double* vx, const double* vy,
                 const double* vz) {
  Mesh& M = h.mesh;
  const int64_t n = M.n;
  count_launch();
  switch (M.nx1) {
#define NEKGPU_CONV_CASE(N)                                                                      \
  case N:                                                                                        \
    conv1_kernel<N><<<M.nel, N * N, 0, h.stream>>>(du, u, vx, vy, vz, M.rst.ptr, M.jac.ptr,      \
                                                   M.f64.D, n);                                  \
    break;
    NEKGPU_CONV_CASE(2)
    NEKGPU_CONV_CASE(3)
    NEKGPU_CONV_CASE(4)
    NEKGPU_CONV_CASE(5)
    NEKGPU_CONV_CASE(6)
    NEKGPU_CONV_CASE(7)
    NEKGPU_CONV_CASE(8)
    NEKGPU_CONV_CASE(9)
    NEKGPU_CONV_CASE(10)
    NEKGPU_CONV_CASE(11)
    NEKGPU_CONV_CASE(12)
#undef NEKGPU_CONV_CASE
    default:
      return -1;
  }
  return 0;
}

int launch_conv2(Handle& h, double* dtfi, const double* fi, const double* vx, const double* vy,
                 const double* vz) {
  Mesh& M = h.mesh;
  const int64_t n = M.n;
  count_launch();
  switch (M.nx1) {
#define NEKGPU_CONV2_CASE(N)                                                                     \
  case N:                                                                                        \
    conv2_kernel<N><<<M.nel, N * N, 0, h.stream>>>(dtfi, fi, vx, vy, vz, M.rst.ptr, M.w3.ptr,    \
                                                   M.f64.bm1, M.f64.D, n);                       \
    break;
    NEKGPU_CONV2_CASE(2)
    NEKGPU_CONV2_CASE(3)
    NEKGPU_CONV2_CASE(4)
    NEKGPU_CONV2_CASE(5)
    NEKGPU_CONV2_CASE(6)
    NEKGPU_CONV2_CASE(7)
    NEKGPU_CONV2_CASE(8)
    NEKGPU_CONV2_CASE(9)
    NEKGPU_CONV2_CASE(10)
    NEKGPU_CONV2_CASE(11)
    NEKGPU_CONV2_CASE(12)
#undef NEKGPU_CONV2_CASE
    default:
      return -1;
  }
  return 0;
}

void launch_subcol3(Handle& h, double* bf, const double* ta) {
  count_launch();
  subcol3_kernel<<<nblk(h.mesh.n), 256, 0, h.stream>>>(bf, h.mesh.f64.bm1, ta, h.mesh.n);
}

void launch_mul_by(Handle& h, double* a, const double* b) {
  count_launch();
  mul_by_kernel<<<nblk(h.mesh.n), 256, 0, h.stream>>>(a, b, h.mesh.n);
}

}  // namespace nekgpu

// ---------------------------------------------------------------------------
// C ABI
namespace nekgpu {
Handle* handle_lookup(const int64_t* h);
int handle_fail(Handle* H, int code, const std::string& msg);
}  // namespace nekgpu

using namespace nekgpu;

namespace {

Handle* grad_handle(const int64_t* handle, int* rc) {
  Handle* H = handle_lookup(handle);
  if (!H) {
    *rc = handle_fail(nullptr, NEKGPU_EHANDLE, "unknown handle");
    return nullptr;
  }
  if (handle_enter(*H) != cudaSuccess) {
    *rc = handle_fail(H, NEKGPU_ECUDA, "call entry failed");
    return nullptr;
  }
  if (!H->has_mesh || !H->mesh.has_rst) {
    *rc = handle_fail(H, NEKGPU_ENOSETUP,
                      "metric terms not set up (the geometry must come from coordinates: "
                      "nekgpu_setup_xyz or nekgpu_geom_update_dev)");
    return nullptr;
  }
  *rc = 0;
  return H;
}

// End of a gradient-type call: the kernels must have finished before the
// call returns (the caller may read the outputs from another stream).
int grad_done(Handle* H, int rc, const char* what) {
  const cudaError_t e = handle_leave(*H);
  if (rc) return handle_fail(H, NEKGPU_EINVAL, std::string(what) + ": lx1 out of range");
  if (e != cudaSuccess) return handle_fail(H, NEKGPU_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
  return NEKGPU_OK;
}

}  // namespace

extern "C" int nekgpu_wgradm1_dev(const int64_t* handle, double* ux, double* uy, double* uz,
                                  const double* u) {
  int rc;
  Handle* H = grad_handle(handle, &rc);
  if (!H) return rc;
  if (!ux || !uy || !uz || !u) return handle_fail(H, NEKGPU_EINVAL, "null argument");
  return grad_done(H, launch_gradop(*H, 0, ux, uy, uz, u, nullptr, nullptr, 0, nullptr),
                   "wgradm1");
}

extern "C" int nekgpu_dudxyz_dev(const int64_t* handle, double* du, const double* u,
                                 const int* isd) {
  int rc;
  Handle* H = grad_handle(handle, &rc);
  if (!H) return rc;
  if (!du || !u || !isd || *isd < 1 || *isd > 3)
    return handle_fail(H, NEKGPU_EINVAL, "bad argument (isd 1, 2 or 3)");
  return grad_done(H, launch_gradop(*H, 1, du, nullptr, nullptr, u, nullptr, nullptr, *isd - 1,
                                    nullptr),
                   "dudxyz");
}

extern "C" int nekgpu_cdtp_dev(const int64_t* handle, double* dtx, const double* x,
                               const int* isd) {
  int rc;
  Handle* H = grad_handle(handle, &rc);
  if (!H) return rc;
  if (!dtx || !x || !isd || *isd < 1 || *isd > 3)
    return handle_fail(H, NEKGPU_EINVAL, "bad argument (isd 1, 2 or 3)");
  return grad_done(H, launch_gradop(*H, 2, dtx, nullptr, nullptr, x, nullptr, nullptr, *isd - 1,
                                    H->mesh.f64.bm1),
                   "cdtp");
}

extern "C" int nekgpu_op_curl_dev(const int64_t* handle, double* w1, double* w2, double* w3,
                                  const double* u1, const double* u2, const double* u3,
                                  const int* ifavg, const double* binv) {
  int rc;
  Handle* H = grad_handle(handle, &rc);
  if (!H) return rc;
  const bool avg = ifavg && *ifavg != 0;
  if (!w1 || !w2 || !w3 || !u1 || !u2 || !u3 || (avg && !binv))
    return handle_fail(H, NEKGPU_EINVAL, "null argument");
  rc = grad_done(H, launch_gradop(*H, 3, w1, w2, w3, u1, u2, u3, 0, nullptr), "op_curl");
  if (rc || !avg) return rc;
  double* w[3] = {w1, w2, w3};
  for (double* c : w) {  // opcolv bm1, opdssum, opcolv binvm1
    launch_mul_by(*H, c, H->mesh.f64.bm1);
    gs_op<double>(H->mesh.gs, c, 0, H->stream);
    launch_mul_by(*H, c, binv);
  }
  return grad_done(H, 0, "op_curl average");
}

extern "C" int nekgpu_conv1_dev(const int64_t* handle, double* du, const double* u,
                                const double* vx, const double* vy, const double* vz) {
  int rc;
  Handle* H = grad_handle(handle, &rc);
  if (!H) return rc;
  if (!du || !u || !vx || !vy || !vz) return handle_fail(H, NEKGPU_EINVAL, "null argument");
  return grad_done(H, launch_conv1(*H, du, u, vx, vy, vz), "conv1");
}

extern "C" int nekgpu_advab_dev(const int64_t* handle, double* bfx, double* bfy, double* bfz,
                                const double* vx, const double* vy, const double* vz) {
  int rc;
  Handle* H = grad_handle(handle, &rc);
  if (!H) return rc;
  if (!bfx || !bfy || !bfz || !vx || !vy || !vz)
    return handle_fail(H, NEKGPU_EINVAL, "null argument");
  if (H->io0.ensure(H->mesh.n)) return handle_fail(H, NEKGPU_ENOMEM, "device allocation failed");
  double* bf[3] = {bfx, bfy, bfz};
  const double* v[3] = {vx, vy, vz};
  for (int c = 0; c < 3; ++c) {  // convop: dealiased once nekgpu_dealias_setup has run
    const int rc2 = H->dealias ? convop_dealias(*H, H->io0.ptr, v[c], vx, vy, vz)
                               : launch_conv1(*H, H->io0.ptr, v[c], vx, vy, vz);
    if (rc2) return grad_done(H, -1, "advab");
    launch_subcol3(*H, bf[c], H->io0.ptr);
  }
  return grad_done(H, 0, "advab");
}

extern "C" int nekgpu_conv2_dev(const int64_t* handle, double* dtfi, const double* fi,
                                const double* vx, const double* vy, const double* vz) {
  int rc;
  Handle* H = grad_handle(handle, &rc);
  if (!H) return rc;
  if (!dtfi || !fi || !vx || !vy || !vz) return handle_fail(H, NEKGPU_EINVAL, "null argument");
  return grad_done(H, launch_conv2(*H, dtfi, fi, vx, vy, vz), "conv2");
}

extern "C" int nekgpu_convopo_dev(const int64_t* handle, double* conv, const double* fi,
                                  const double* vx, const double* vy, const double* vz,
                                  const int* ofc) {
  int rc;
  Handle* H = grad_handle(handle, &rc);
  if (!H) return rc;
  if (!conv || !fi || !vx || !vy || !vz) return handle_fail(H, NEKGPU_EINVAL, "null argument");
  const int64_t n = H->mesh.n;
  const int nel = H->mesh.nel;
  cudaStream_t s = H->stream;
  if (H->io0.ensure(n) || H->io1.ensure(n) || H->io2.ensure(n) || H->io3.ensure(n) ||
      H->p4_fbc.ensure((size_t)6 * nel))
    return handle_fail(H, NEKGPU_ENOMEM, "device allocation failed");
  double *c1 = H->io0.ptr, *c2 = H->io1.ptr, *mfi = H->io2.ptr, *dm = H->io3.ptr;
  if (ofc) {
    cudaMemcpyAsync(H->p4_fbc.ptr, ofc, (size_t)6 * nel * sizeof(int), cudaMemcpyHostToDevice, s);
  } else {
    cudaMemsetAsync(H->p4_fbc.ptr, 0, (size_t)6 * nel * sizeof(int), s);
  }
  count_launch(2);
  cmask_kernel<<<nel, 128, 0, s>>>(c1, c2, H->p4_fbc.ptr, H->mesh.nx1);
  cudaMemsetAsync(conv, 0, n * sizeof(double), s);
  const int nb = nblk(n);
  auto acc = [&](const double* cm, double coef) {
    count_launch();
    acc_kernel<<<nb, 256, 0, s>>>(conv, dm, cm, coef, n);
  };
  col3_kernel<<<nb, 256, 0, s>>>(mfi, fi, c1, n);
  if (launch_conv1(*H, dm, mfi, vx, vy, vz)) return grad_done(H, -1, "convopo");
  acc(c1, 0.5);
  acc(c2, 1.0);
  launch_conv2(*H, dm, mfi, vx, vy, vz);
  acc(c1, -0.5);
  count_launch();
  col3_kernel<<<nb, 256, 0, s>>>(mfi, fi, c2, n);
  launch_conv1(*H, dm, mfi, vx, vy, vz);
  acc(c2, 0.5);
  launch_conv2(*H, dm, mfi, vx, vy, vz);
  acc(c1, -1.0);
  acc(c2, 0.5);
  return grad_done(H, 0, "convopo");
}
