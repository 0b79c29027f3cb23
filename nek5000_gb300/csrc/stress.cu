// stress.cu -- the stress formulation's coupled velocity operator and solve
// (plan4 with ifstrs), FP64, in the reference's arithmetic order:
//
//   axsf     core/subs1.f:2031-2116  axsf_e_3d per element (axhmsf's default
//            path for a fluid, :1240-1315): grad u from local_grad3 and the
//            metric terms, the symmetric strain times h1 w3 / J, contracted
//            back with the metric terms and local_grad3_t, plus h2 B u
//   hmhzsf   core/subs1.f:1093-1147 without the projection onto previous
//            solutions: the volume masks of rmask (qmask, core/subs2.f:1800),
//            opdssum, chktcgs (subs1.f:1149-1238), cggosf (:2-165, Jacobi-PCG
//            on the three coupled components, capped at 200 iterations as
//            the reference sets it)
//
// The operator is one block per element: thread (i, j) walks its z-column;
// the three fields, D and the nine per-point tensor components sit in shared
// memory between the forward and the transposed contractions.  Products and
// sums are rounded one by one (bit-identical to the oracle's restatement).
// The solve's dot products are block-order sums of per-point values (host
// adds the block partials in order), so they differ from the serial sums in
// the last bits.  Needs the metric terms (geometry from coordinates).
#include <cmath>
#include <string>
#include <vector>

#include "impl.cuh"
#include "nekgpu.h"

namespace nekgpu {

Handle* handle_lookup(const int64_t* h);  // capi.cu
int handle_fail(Handle* H, int code, const std::string& msg);

namespace {

constexpr int kSfThreads = 256;

inline int sf_blocks(int64_t n) {
  return (int)std::min<int64_t>(std::max<int64_t>((n + kSfThreads - 1) / kSfThreads, 1), 152 * 4);
}

__device__ __forceinline__ double dot3x(double a1, double b1, double a2, double b2, double a3,
                                        double b3) {
  return __dadd_rn(__dadd_rn(__dmul_rn(a1, b1), __dmul_rn(a2, b2)), __dmul_rn(a3, b3));
}

template <int NX>
constexpr size_t axsf_smem_bytes() {
  return (size_t)(12 * NX * NX * NX + NX * NX) * sizeof(double);
}

template <int NX>
__global__ void __launch_bounds__(NX* NX)
    axsf_kernel(double* __restrict__ au, double* __restrict__ av, double* __restrict__ aw,
                const double* __restrict__ u, const double* __restrict__ v,
                const double* __restrict__ w, const double* __restrict__ h1,
                const double* __restrict__ h2, const double* __restrict__ rst,
                const double* __restrict__ jac, const double* __restrict__ bm1,
                const double* __restrict__ w3, const double* __restrict__ D, int64_t n) {
  constexpr int P = NX * NX * NX, NXY = NX * NX;
  extern __shared__ __align__(16) double sf_smem[];
  double* sf = sf_smem;              // [3][P]: u, v, w of the element
  double* sr = sf + 3 * P;           // [9][P]: ur(., a, b) at sr[(a + 3 b) P]
  double* sD = sr + 9 * P;           // D[i][l]
  const int64_t eo = (int64_t)blockIdx.x * P;
  const int tid = threadIdx.x;
  for (int q = tid; q < P; q += NXY) {
    sf[q] = u[eo + q];
    sf[P + q] = v[eo + q];
    sf[2 * P + q] = w[eo + q];
  }
  for (int q = tid; q < NXY; q += NXY) sD[q] = D[q];
  __syncthreads();
  const int i = tid % NX, j = tid / NX;
  const double *rx = rst, *ry = rst + n, *rz = rst + 2 * n, *sx = rst + 3 * n, *sy = rst + 4 * n,
               *sz = rst + 5 * n, *tx = rst + 6 * n, *ty = rst + 7 * n, *tz = rst + 8 * n;
  for (int k = 0; k < NX; ++k) {
    const int pt = i + NX * (j + NX * k);
    const int64_t g = eo + pt;
    // local_grad3 of the three fields (the mxm order of core/mxm_std.f)
    double gr[3], gs[3], gt[3];
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      const double* su = sf + f * P;
      double a = __dmul_rn(sD[i * NX], su[NX * (j + NX * k)]);
      double b = __dmul_rn(su[i + NXY * k], sD[j * NX]);
      double c = __dmul_rn(su[i + NX * j], sD[k * NX]);
#pragma unroll
      for (int l = 1; l < NX; ++l) {
        a = __dadd_rn(a, __dmul_rn(sD[i * NX + l], su[l + NX * (j + NX * k)]));
        b = __dadd_rn(b, __dmul_rn(su[i + NX * (l + NX * k)], sD[j * NX + l]));
        c = __dadd_rn(c, __dmul_rn(su[i + NX * (j + NX * l)], sD[k * NX + l]));
      }
      gr[f] = a;
      gs[f] = b;
      gt[f] = c;
    }
    const double mrx = rx[g], mry = ry[g], mrz = rz[g], msx = sx[g], msy = sy[g], msz = sz[g],
                 mtx = tx[g], mty = ty[g], mtz = tz[g];
    const double u1 = dot3x(gr[0], mrx, gs[0], msx, gt[0], mtx);
    const double u2 = dot3x(gr[0], mry, gs[0], msy, gt[0], mty);
    const double u3 = dot3x(gr[0], mrz, gs[0], msz, gt[0], mtz);
    const double v1 = dot3x(gr[1], mrx, gs[1], msx, gt[1], mtx);
    const double v2 = dot3x(gr[1], mry, gs[1], msy, gt[1], mty);
    const double v3 = dot3x(gr[1], mrz, gs[1], msz, gt[1], mtz);
    const double w1 = dot3x(gr[2], mrx, gs[2], msx, gt[2], mtx);
    const double w2 = dot3x(gr[2], mry, gs[2], msy, gt[2], mty);
    const double ww = dot3x(gr[2], mrz, gs[2], msz, gt[2], mtz);
    const double dj = __dmul_rn(__dmul_rn(h1[g], w3[pt]), __ddiv_rn(1.0, jac[g]));
    const double s11 = __dmul_rn(dj, __dadd_rn(u1, u1)), s12 = __dmul_rn(dj, __dadd_rn(u2, v1)),
                 s13 = __dmul_rn(dj, __dadd_rn(u3, w1));
    const double s21 = __dmul_rn(dj, __dadd_rn(v1, u2)), s22 = __dmul_rn(dj, __dadd_rn(v2, v2)),
                 s23 = __dmul_rn(dj, __dadd_rn(v3, w2));
    const double s31 = __dmul_rn(dj, __dadd_rn(w1, u3)), s32 = __dmul_rn(dj, __dadd_rn(w2, v3)),
                 s33 = __dmul_rn(dj, __dadd_rn(ww, ww));
    sr[0 * P + pt] = dot3x(mrx, s11, mry, s12, mrz, s13);
    sr[1 * P + pt] = dot3x(msx, s11, msy, s12, msz, s13);
    sr[2 * P + pt] = dot3x(mtx, s11, mty, s12, mtz, s13);
    sr[3 * P + pt] = dot3x(mrx, s21, mry, s22, mrz, s23);
    sr[4 * P + pt] = dot3x(msx, s21, msy, s22, msz, s23);
    sr[5 * P + pt] = dot3x(mtx, s21, mty, s22, mtz, s23);
    sr[6 * P + pt] = dot3x(mrx, s31, mry, s32, mrz, s33);
    sr[7 * P + pt] = dot3x(msx, s31, msy, s32, msz, s33);
    sr[8 * P + pt] = dot3x(mtx, s31, mty, s32, mtz, s33);
  }
  __syncthreads();
  double* out[3] = {au, av, aw};
  for (int k = 0; k < NX; ++k) {
    const int pt = i + NX * (j + NX * k);
    const int64_t g = eo + pt;
    const double hb = __dmul_rn(h2[g], bm1[g]);
#pragma unroll
    for (int f = 0; f < 3; ++f) {
      // local_grad3_t: sum_l D(l,i) ta(l,j,k) + sum_l tb(i,l,k) D(l,j) + sum_l tc(i,j,l) D(l,k)
      const double* ta = sr + (3 * f) * P;
      const double* tb = sr + (3 * f + 1) * P;
      const double* tc = sr + (3 * f + 2) * P;
      double r = __dmul_rn(sD[i], ta[NX * (j + NX * k)]);
      double s = __dmul_rn(tb[i + NXY * k], sD[j]);
      double t = __dmul_rn(tc[i + NX * j], sD[k]);
#pragma unroll
      for (int l = 1; l < NX; ++l) {
        r = __dadd_rn(r, __dmul_rn(sD[l * NX + i], ta[l + NX * (j + NX * k)]));
        s = __dadd_rn(s, __dmul_rn(tb[i + NX * (l + NX * k)], sD[l * NX + j]));
        t = __dadd_rn(t, __dmul_rn(tc[i + NX * (j + NX * l)], sD[l * NX + k]));
      }
      const double a = __dadd_rn(__dadd_rn(r, s), t);
      out[f][g] = __dadd_rn(a, __dmul_rn(hb, sf[f * P + pt]));
    }
  }
}

template <int NX>
cudaError_t launch_axsf_nx(const Mesh& m, double* au, double* av, double* aw, const double* u,
                           const double* v, const double* w, const double* h1, const double* h2,
                           cudaStream_t s) {
  static std::atomic<uint32_t> configured{0};  // per device
  if (first_on_device(configured)) {
    cudaError_t e = cudaFuncSetAttribute(axsf_kernel<NX>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)axsf_smem_bytes<NX>());
    if (e != cudaSuccess) return e;
    mark_device(configured);
  }
  count_launch();
  axsf_kernel<NX><<<m.nel, NX * NX, axsf_smem_bytes<NX>(), s>>>(
      au, av, aw, u, v, w, h1, h2, m.rst.ptr, m.jac.ptr, m.f64.bm1, m.w3.ptr, m.f64.D, m.n);
  return cudaGetLastError();
}

cudaError_t launch_axsf(const Mesh& m, double* au, double* av, double* aw, const double* u,
                        const double* v, const double* w, const double* h1, const double* h2,
                        cudaStream_t s) {
  switch (m.nx1) {
#define NEKGPU_SF_CASE(N) \
  case N: return launch_axsf_nx<N>(m, au, av, aw, u, v, w, h1, h2, s);
    NEKGPU_SF_CASE(2)
    NEKGPU_SF_CASE(3)
    NEKGPU_SF_CASE(4)
    NEKGPU_SF_CASE(5)
    NEKGPU_SF_CASE(6)
    NEKGPU_SF_CASE(7)
    NEKGPU_SF_CASE(8)
    NEKGPU_SF_CASE(9)
    NEKGPU_SF_CASE(10)
    NEKGPU_SF_CASE(11)
    NEKGPU_SF_CASE(12)
#undef NEKGPU_SF_CASE
    default: return cudaErrorInvalidValue;
  }
}

#define SF_FOR(i, n)                                                              \
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); \
       i += (int64_t)gridDim.x * blockDim.x)

// r_c = r_c * m_c (the volume masks of qmask)
__global__ void sf_mask_kernel(double* r1, double* r2, double* r3, const double* m1,
                               const double* m2, const double* m3, int64_t n) {
  SF_FOR(i, n) {
    r1[i] = __dmul_rn(r1[i], m1[i]);
    r2[i] = __dmul_rn(r2[i], m2[i]);
    r3[i] = __dmul_rn(r3[i], m3[i]);
  }
}

// Block partials of sum_i f(i):
//   kind 0: (a.b) binv mult          (opdot then glsc3, cggosf's norm)
//   kind 1: mult (a.b)               (op_glsc2_wt / glsc2 of opdot)
//   kind 2: mult (m1 + m2 + m3)      (chktcgs's Neumann test, add4 then glsc2)
//   kind 3: mult                     (glsum)
//   kind 4: mult ((a1 + a2) + a3)    (chktcgs's mean)
__global__ void __launch_bounds__(kSfThreads)
    sf_sum_kernel(double* __restrict__ part, int kind, const double* a1, const double* a2,
                  const double* a3, const double* b1, const double* b2, const double* b3,
                  const double* __restrict__ binv, const double* __restrict__ mult, int64_t n) {
  __shared__ double red[kSfThreads];
  double acc = 0.0;
  SF_FOR(i, n) {
    double val;
    if (kind == 0) {
      val = __dmul_rn(__dmul_rn(dot3x(a1[i], b1[i], a2[i], b2[i], a3[i], b3[i]), binv[i]), mult[i]);
    } else if (kind == 1) {
      val = __dmul_rn(mult[i], dot3x(a1[i], b1[i], a2[i], b2[i], a3[i], b3[i]));
    } else if (kind == 3) {
      val = mult[i];
    } else {
      val = __dmul_rn(__dadd_rn(__dadd_rn(a1[i], a2[i]), a3[i]), mult[i]);
    }
    acc = __dadd_rn(acc, val);
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int w = kSfThreads / 2; w > 0; w >>= 1) {
    if ((int)threadIdx.x < w) red[threadIdx.x] = __dadd_rn(red[threadIdx.x], red[threadIdx.x + w]);
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// dpc = (s + s) + s   (the three setprec diagonals of cggosf, equal in 3-D)
__global__ void sf_dpc_kernel(double* dpc, int64_t n) {
  SF_FOR(i, n) {
    const double s = dpc[i];
    dpc[i] = __dadd_rn(__dadd_rn(s, s), s);
  }
}

// pp_c = dpc r_c; with init also p_c = 0 + pp_c
__global__ void sf_prec_kernel(double* pp1, double* pp2, double* pp3, double* p1, double* p2,
                               double* p3, const double* r1, const double* r2, const double* r3,
                               const double* dpc, int init, int64_t n) {
  SF_FOR(i, n) {
    const double d = dpc[i];
    const double a = __dmul_rn(d, r1[i]), b = __dmul_rn(d, r2[i]), c = __dmul_rn(d, r3[i]);
    pp1[i] = a;
    pp2[i] = b;
    pp3[i] = c;
    if (init) {
      p1[i] = __dadd_rn(0.0, a);
      p2[i] = __dadd_rn(0.0, b);
      p3[i] = __dadd_rn(0.0, c);
    }
  }
}

// u_c += alpha p_c ; r_c += (-alpha) ap_c   (opadds isc = 2, twice)
__global__ void sf_step_kernel(double* u1, double* u2, double* u3, double* r1, double* r2,
                               double* r3, const double* p1, const double* p2, const double* p3,
                               const double* q1, const double* q2, const double* q3,
                               double alpha, int64_t n) {
  SF_FOR(i, n) {
    u1[i] = __dadd_rn(u1[i], __dmul_rn(alpha, p1[i]));
    u2[i] = __dadd_rn(u2[i], __dmul_rn(alpha, p2[i]));
    u3[i] = __dadd_rn(u3[i], __dmul_rn(alpha, p3[i]));
    r1[i] = __dadd_rn(r1[i], __dmul_rn(-alpha, q1[i]));
    r2[i] = __dadd_rn(r2[i], __dmul_rn(-alpha, q2[i]));
    r3[i] = __dadd_rn(r3[i], __dmul_rn(-alpha, q3[i]));
  }
}

// p_c = beta p_c + pp_c   (opadds isc = 1)
__global__ void sf_dir_kernel(double* p1, double* p2, double* p3, const double* pp1,
                              const double* pp2, const double* pp3, double beta, int64_t n) {
  SF_FOR(i, n) {
    p1[i] = __dadd_rn(__dmul_rn(beta, p1[i]), pp1[i]);
    p2[i] = __dadd_rn(__dmul_rn(beta, p2[i]), pp2[i]);
    p3[i] = __dadd_rn(__dmul_rn(beta, p3[i]), pp3[i]);
  }
}

// A reduction's value: the block partials summed on the host in block order.
struct SfSum {
  Handle& h;
  DevBuf<double>& part;
  std::vector<double> host;
  int nb;
  double operator()(int kind, const double* a1, const double* a2, const double* a3,
                    const double* b1, const double* b2, const double* b3, const double* binv,
                    const double* mult, int* st) {
    count_launch();
    sf_sum_kernel<<<nb, kSfThreads, 0, h.stream>>>(part.ptr, kind, a1, a2, a3, b1, b2, b3, binv,
                                                   mult, h.mesh.n);
    if (cudaMemcpyAsync(host.data(), part.ptr, nb * sizeof(double), cudaMemcpyDeviceToHost,
                        h.stream) != cudaSuccess ||
        cudaStreamSynchronize(h.stream) != cudaSuccess) {
      *st = -3;
      return 0.0;
    }
    double s = 0.0;
    for (double x : host) s += x;
    return s;
  }
};

int sf_fail(Handle* H, int code, const std::string& what) {
  const cudaError_t e = cudaStreamSynchronize(H->stream);
  if (e != cudaSuccess) return handle_fail(H, NEKGPU_ECUDA, what + ": " + cudaGetErrorString(e));
  return handle_fail(H, code, what);
}

Handle* sf_handle(const int64_t* handle, int* rc) {
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
                      "metric terms not set up (the geometry must come from coordinates)");
    return nullptr;
  }
  *rc = 0;
  return H;
}

}  // namespace

extern "C" int nekgpu_axhmsf_dev(const int64_t* handle, double* au1, double* au2, double* au3,
                                 const double* u1, const double* u2, const double* u3,
                                 const double* h1, const double* h2) {
  int rc;
  Handle* H = sf_handle(handle, &rc);
  if (!H) return rc;
  if (!au1 || !au2 || !au3 || !u1 || !u2 || !u3 || !h1 || !h2)
    return handle_fail(H, NEKGPU_EINVAL, "null argument");
  cudaError_t e = launch_axsf(H->mesh, au1, au2, au3, u1, u2, u3, h1, h2, H->stream);
  if (e == cudaSuccess) e = handle_leave(*H);
  if (e != cudaSuccess) return handle_fail(H, NEKGPU_ECUDA, std::string("axhmsf: ") + cudaGetErrorString(e));
  return NEKGPU_OK;
}

extern "C" int nekgpu_hmhzsf_dev(const int64_t* handle, double* u1, double* u2, double* u3,
                                 double* r1, double* r2, double* r3, const double* h1,
                                 const double* h2, const double* m1, const double* m2,
                                 const double* m3, const double* mult, const double* binv,
                                 const double* tol, int* niter, double* rbn0, double* rbn2) {
  int rc;
  Handle* H = sf_handle(handle, &rc);
  if (!H) return rc;
  if (!u1 || !u2 || !u3 || !r1 || !r2 || !r3 || !h1 || !h2 || !m1 || !m2 || !m3 || !mult ||
      !binv || !tol)
    return handle_fail(H, NEKGPU_EINVAL, "null argument");
  Mesh& M = H->mesh;
  const int64_t n = M.n;
  cudaStream_t s = H->stream;
  const int nb = sf_blocks(n);
  for (DevBuf<double>& b : H->sfw)
    if (b.ensure(n)) return handle_fail(H, NEKGPU_ENOMEM, "device allocation failed");
  if (H->sf_part.ensure(nb)) return handle_fail(H, NEKGPU_ENOMEM, "device allocation failed");
  DevBuf<double>& dpc = H->sfw[9];
  double *p[3] = {H->sfw[0].ptr, H->sfw[1].ptr, H->sfw[2].ptr},
         *pp[3] = {H->sfw[3].ptr, H->sfw[4].ptr, H->sfw[5].ptr},
         *ap[3] = {H->sfw[6].ptr, H->sfw[7].ptr, H->sfw[8].ptr};
  double* r[3] = {r1, r2, r3};
  double* u[3] = {u1, u2, u3};
  SfSum sum{*H, H->sf_part, std::vector<double>((size_t)nb), nb};
  int st = 0;
  // hmhzsf: rmask, opdssum, u = 0
  count_launch();
  sf_mask_kernel<<<nb, kSfThreads, 0, s>>>(r1, r2, r3, m1, m2, m3, n);
  for (int c = 0; c < 3; ++c) {
    gs_op<double>(M.gs, r[c], 0, s);
    cudaMemsetAsync(u[c], 0, n * sizeof(double), s);
  }
  // chktcgs (EIGAA = 0: ACONDNO = 10; FP64: EPS = 1e-13)
  double tl = *tol;
  {
    const double s0 = sum(0, r1, r2, r3, r1, r2, r3, binv, mult, &st);
    const double rmin = 1e-13 * std::sqrt(s0 / M.vol);
    if (tl < rmin) tl = rmin;
    const double b1 = sum(2, m1, m2, m3, nullptr, nullptr, nullptr, nullptr, mult, &st);
    const double b2 = sum(3, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, mult,
                          &st);
    if (std::fabs(b1 - 3.0 * b2) < 0.1) {
      const double o = sum(4, r1, r2, r3, nullptr, nullptr, nullptr, nullptr, mult, &st);
      const double tolmin = std::fabs(o / 3.0) * 10.0;
      if (tl < tolmin) tl = tolmin;
    }
  }
  if (st) return sf_fail(H, NEKGPU_ECUDA, "hmhzsf: reduction failed");
  // cggosf
  double rbnorm = std::sqrt(sum(0, r1, r2, r3, r1, r2, r3, binv, mult, &st) / M.vol);
  if (rbn0) *rbn0 = rbnorm;
  if (rbnorm < tl * tl) {
    if (niter) *niter = 0;
    if (rbn2) *rbn2 = rbnorm;
    const cudaError_t e = handle_leave(*H);
    if (e != cudaSuccess) return handle_fail(H, NEKGPU_ECUDA, std::string("hmhzsf: ") + cudaGetErrorString(e));
    return NEKGPU_OK;
  }
  Coef<double> c;
  if (detect_coef<double>(*H, h1, h2, n, c) || setprec_f64(*H, dpc.ptr, c))
    return sf_fail(H, NEKGPU_ECUDA, "hmhzsf: setprec failed");
  count_launch(2);
  sf_dpc_kernel<<<nb, kSfThreads, 0, s>>>(dpc.ptr, n);
  sf_prec_kernel<<<nb, kSfThreads, 0, s>>>(pp[0], pp[1], pp[2], p[0], p[1], p[2], r1, r2, r3,
                                           dpc.ptr, 1, n);
  double rpp1 = sum(1, p[0], p[1], p[2], r1, r2, r3, nullptr, mult, &st);
  int it_done = -1;
  constexpr int kMaxIt = 200;  // cggosf sets maxit = 200 (core/subs1.f:107)
  for (int iter = 1; iter <= kMaxIt && !st; ++iter) {
    if (launch_axsf(M, ap[0], ap[1], ap[2], p[0], p[1], p[2], h1, h2, s) != cudaSuccess)
      return sf_fail(H, NEKGPU_ECUDA, "hmhzsf: operator launch failed");
    count_launch();
    sf_mask_kernel<<<nb, kSfThreads, 0, s>>>(ap[0], ap[1], ap[2], m1, m2, m3, n);
    for (int k = 0; k < 3; ++k) gs_op<double>(M.gs, ap[k], 0, s);
    const double pap = sum(1, p[0], p[1], p[2], ap[0], ap[1], ap[2], nullptr, mult, &st);
    const double alpha = rpp1 / pap;
    count_launch();
    sf_step_kernel<<<nb, kSfThreads, 0, s>>>(u1, u2, u3, r1, r2, r3, p[0], p[1], p[2], ap[0],
                                             ap[1], ap[2], alpha, n);
    rbnorm = std::sqrt(sum(0, r1, r2, r3, r1, r2, r3, binv, mult, &st) / M.vol);
    if (iter == 1 && rbn0) *rbn0 = rbnorm;
    if (rbnorm < tl) {
      it_done = iter;
      break;
    }
    count_launch();
    sf_prec_kernel<<<nb, kSfThreads, 0, s>>>(pp[0], pp[1], pp[2], nullptr, nullptr, nullptr, r1,
                                             r2, r3, dpc.ptr, 0, n);
    const double rpp2 = rpp1;
    rpp1 = sum(1, r1, r2, r3, pp[0], pp[1], pp[2], nullptr, mult, &st);
    const double beta = rpp1 / rpp2;
    count_launch();
    sf_dir_kernel<<<nb, kSfThreads, 0, s>>>(p[0], p[1], p[2], pp[0], pp[1], pp[2], beta, n);
  }
  if (st) return sf_fail(H, NEKGPU_ECUDA, "hmhzsf: reduction failed");
  const cudaError_t e = handle_leave(*H);
  if (e != cudaSuccess) return handle_fail(H, NEKGPU_ECUDA, std::string("hmhzsf: ") + cudaGetErrorString(e));
  if (niter) *niter = it_done < 0 ? kMaxIt : it_done;
  if (rbn2) *rbn2 = rbnorm;
  if (it_done < 0) return handle_fail(H, NEKGPU_ENOTCONV, "hmhzsf: 200 iterations without convergence");
  return NEKGPU_OK;
}

}  // namespace nekgpu
