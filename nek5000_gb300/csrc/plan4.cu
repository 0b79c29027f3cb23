// plan4.cu -- the explicit right-hand sides of the PN-PN splitting step
// (plan4, core/plan4.f) on the device, composed from the library's
// operator (axhelm), gradient-type operators (gradops.cu) and gather-scatter:
//
//   cresvsp  core/plan4.f:264-306  velocity residual
//   cresvsp_weak  core/plan4.f:308-361  the same with the weak pressure
//            gradient (the stress formulation's branch, plan4.f:84-86)
//            resv = -A(h1, h2) v - opgrad(pr - vdiff qtl / 3) + bf
//   crespsp  core/plan4.f:99-230   pressure right-hand side from the
//            curl-curl of the extrapolated velocity, qtl, the pressure's own
//            operator and the forcing
//
// Pointwise steps are rounded one by one in the reference's order; with the
// handle's exact option the operator is too, and both residuals are then the
// reference's unfused FP64 values bit for bit.  Not served: the stress
// formulation (ifstrs).
#include <string>
#include <vector>

#include "impl.cuh"

namespace nekgpu {
namespace {

int pblocks(int64_t n) { return (int)std::min<int64_t>((n + 255) / 256, 152 * 8); }

#define PFOR(i, n) \
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)

// ta = scale (vdiff qtl) + pr   (col3, add2s1)
__global__ void p4_ta4_kernel(double* __restrict__ ta, const double* __restrict__ vdiff,
                              const double* __restrict__ qtl, const double* __restrict__ pr,
                              double scale, int64_t n) {
  PFOR(i, n) ta[i] = __dadd_rn(__dmul_rn(scale, __dmul_rn(vdiff[i], qtl[i])), pr[i]);
}

// r = ((-r) - t) + bf   (opchsgn, opsub2, opadd2)
__global__ void p4_resv_kernel(double* __restrict__ r, const double* __restrict__ t,
                               const double* __restrict__ bf, int64_t n) {
  PFOR(i, n) r[i] = __dadd_rn(__dsub_rn(-r[i], t[i]), bf[i]);
}

// ta = (vdiff qtl) scale   (col3, cmult)
__global__ void p4_ta4w_kernel(double* __restrict__ ta, const double* __restrict__ vdiff,
                               const double* __restrict__ qtl, double scale, int64_t n) {
  PFOR(i, n) ta[i] = __dmul_rn(__dmul_rn(vdiff[i], qtl[i]), scale);
}

// t = t - wa   (sub2)
__global__ void p4_sub_kernel(double* __restrict__ t, const double* __restrict__ wa, int64_t n) {
  PFOR(i, n) t[i] = __dsub_rn(t[i], wa[i]);
}

// wa = (wa bm1 + ta scale) (vdiff / vtrans)   (opcolv, opadd2cm, invcol3, opcolv)
__global__ void p4_wa_kernel(double* __restrict__ wa, const double* __restrict__ ta,
                             const double* __restrict__ bm1, const double* __restrict__ vdiff,
                             const double* __restrict__ vtrans, double scale, int64_t n) {
  PFOR(i, n) {
    const double w = __dadd_rn(__dmul_rn(wa[i], bm1[i]), __dmul_rn(ta[i], scale));
    wa[i] = __dmul_rn(w, __ddiv_rn(vdiff[i], vtrans[i]));
  }
}

// h1 = 1 / vtrans, h2 = 0   (invers2, rzero)
__global__ void p4_h_kernel(double* __restrict__ h1, double* __restrict__ h2,
                            const double* __restrict__ vtrans, int64_t n) {
  PFOR(i, n) {
    h1[i] = __ddiv_rn(1.0, vtrans[i]);
    h2[i] = 0.0;
  }
}

// ta = bf / vtrans - wa
__global__ void p4_tb_kernel(double* __restrict__ ta, const double* __restrict__ bf,
                             const double* __restrict__ vtrans, const double* __restrict__ wa,
                             int64_t n) {
  PFOR(i, n) ta[i] = __dsub_rn(__ddiv_rn(bf[i], vtrans[i]), wa[i]);
}

// respr = (((-respr) + wa1 + wa2 + wa3) + (qtl bm1) dtbd)   (chsign, sum, admcol3)
__global__ void p4_respr_kernel(double* __restrict__ respr, const double* __restrict__ w1,
                                const double* __restrict__ w2, const double* __restrict__ w3,
                                const double* __restrict__ qtl, const double* __restrict__ bm1,
                                double dtbd, int64_t n) {
  PFOR(i, n) {
    double r = __dadd_rn(__dadd_rn(__dadd_rn(-respr[i], w1[i]), w2[i]), w3[i]);
    respr[i] = __dadd_rn(r, __dmul_rn(__dmul_rn(qtl[i], bm1[i]), dtbd));
  }
}

// partial[blk] = sum over the block's points (the ortho mean)
__global__ void __launch_bounds__(256) p4_sum_kernel(const double* __restrict__ a, int64_t n,
                                                     double* __restrict__ partial) {
  __shared__ double red[8];
  double s = 0.0;
  PFOR(i, n) s += a[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int q = 0; q < 8; ++q) t += red[q];
    partial[blockIdx.x] = t;
  }
}

__global__ void p4_cadd_kernel(double* __restrict__ a, double c, int64_t n) {
  PFOR(i, n) a[i] = __dadd_rn(a[i], c);
}

// makeabf, one component: ta = ab1 abx1 + ab2 abx2; abx2 = abx1; abx1 = bf;
// bf = (ab0 bf + ta) vtrans
__global__ void p4_makeabf_kernel(double* __restrict__ bf, double* __restrict__ abx1,
                                  double* __restrict__ abx2, const double* __restrict__ vtrans,
                                  double ab0, double ab1, double ab2, int64_t n) {
  PFOR(i, n) {
    const double a1 = abx1[i];
    const double ta = __dadd_rn(__dmul_rn(ab1, a1), __dmul_rn(ab2, abx2[i]));
    const double b = bf[i];
    abx2[i] = a1;
    abx1[i] = b;
    bf[i] = __dmul_rn(__dadd_rn(__dmul_rn(ab0, b), ta), vtrans[i]);
  }
}

struct Bd {
  double c[4];
};

// makebdf, one component: bf += (v bm1 bd1 + sum_l vlag_l bm1 bd_{l+1}) (vtrans / dt)
__global__ void p4_makebdf_kernel(double* __restrict__ bf, const double* __restrict__ v,
                                  const double* __restrict__ vlag, int nlag,
                                  const double* __restrict__ bm1,
                                  const double* __restrict__ vtrans, Bd bd, double cnst,
                                  int64_t n) {
  PFOR(i, n) {
    const double h2 = __dmul_rn(vtrans[i], cnst);
    double tb = __dmul_rn(__dmul_rn(v[i], bm1[i]), bd.c[1]);
    for (int l = 0; l < nlag; ++l)
      tb = __dadd_rn(tb, __dmul_rn(__dmul_rn(vlag[(int64_t)l * n + i], bm1[i]), bd.c[l + 2]));
    bf[i] = __dadd_rn(bf[i], __dmul_rn(tb, h2));
  }
}

// sumab: v = ab0 vv + ab1 vvlag_1 (+ ab2 vvlag_2)
__global__ void p4_sumab_kernel(double* __restrict__ v, const double* __restrict__ vv,
                                const double* __restrict__ vvlag, double ab0, double ab1,
                                double ab2, int nab, int64_t n) {
  PFOR(i, n) {
    double a = __dadd_rn(__dmul_rn(ab0, vv[i]), __dmul_rn(ab1, vvlag[i]));
    if (nab == 3) a = __dadd_rn(a, __dmul_rn(ab2, vvlag[n + i]));
    v[i] = a;
  }
}

// crespsp's face terms (core/plan4.f:219-258), one block per element, the
// six faces in preprocessor order one after another (edge points of two
// marked faces take both subtractions in that order).  Face f's outward
// normal is +-(the r, s or t cofactor triple) / its length and its area
// that length times the two GLL weights (area3 / unitvec, core/coef.f:
// 1354-1445).  Types: 1 velocity times dtbd, 2 velocity ('shl'), 3 'SYM'
// (the fields s1..s3).
__global__ void p4_face_kernel(double* __restrict__ respr, const double* __restrict__ v1,
                               const double* __restrict__ v2, const double* __restrict__ v3,
                               const double* __restrict__ s1, const double* __restrict__ s2,
                               const double* __restrict__ s3, const int* __restrict__ fbc,
                               const double* __restrict__ rst, const double* __restrict__ w,
                               double dtbd, int nx1, int64_t n) {
  const int64_t e = blockIdx.x, eo = e * (int64_t)nx1 * nx1 * nx1;
  const int N = nx1 - 1;
  for (int f = 1; f <= 6; ++f) {
    const int t = fbc[6 * e + f - 1];  // the same for the whole block
    if (t >= 1 && t <= 3) {
      const int d = (f == 2 || f == 4) ? 0 : (f == 1 || f == 3) ? 1 : 2;
      const double sg = (f == 1 || f == 4 || f == 5) ? -1.0 : 1.0;
      const double *b1 = t == 3 ? s1 : v1, *b2 = t == 3 ? s2 : v2, *b3 = t == 3 ? s3 : v3;
      for (int q = threadIdx.x; q < nx1 * nx1; q += blockDim.x) {
        const int a = q % nx1, b = q / nx1;
        int i, j, k;
        if (d == 0) {
          i = f == 2 ? N : 0;
          j = a;
          k = b;
        } else if (d == 1) {
          i = a;
          j = f == 3 ? N : 0;
          k = b;
        } else {
          i = a;
          j = b;
          k = f == 6 ? N : 0;
        }
        const int64_t p = eo + i + nx1 * (j + nx1 * k);
        const double c1 = rst[(int64_t)(3 * d) * n + p], c2 = rst[(int64_t)(3 * d + 1) * n + p],
                     c3 = rst[(int64_t)(3 * d + 2) * n + p];
        const double len =
            __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(c1, c1), __dmul_rn(c2, c2)), __dmul_rn(c3, c3)));
        double nx = sg * c1, ny = sg * c2, nz = sg * c3;
        if (len != 0.0) {
          nx = __ddiv_rn(nx, len);
          ny = __ddiv_rn(ny, len);
          nz = __ddiv_rn(nz, len);
        }
        const double area = __dmul_rn(len, __dmul_rn(w[a], w[b]));
        double v = __dmul_rn(b1[p], nx);
        v = __dadd_rn(v, __dmul_rn(b2[p], ny));
        v = __dadd_rn(v, __dmul_rn(b3[p], nz));
        v = __dmul_rn(v, area);
        if (t == 1) v = __dmul_rn(v, dtbd);
        respr[p] = __dsub_rn(respr[p], v);
      }
    }
    __syncthreads();
  }
}

#undef PFOR

int axhelm_any(Handle& h, double* au, const double* u, const Coef<double>& c) {
  const cudaError_t e = h.exact ? launch_axhelm<double, true>(h.mesh, h.mesh.f64, au, u, c, h.stream)
                                : launch_axhelm<double, false>(h.mesh, h.mesh.f64, au, u, c, h.stream);
  return e == cudaSuccess ? 0 : -3;
}

}  // namespace
}  // namespace nekgpu

// ---------------------------------------------------------------------------
// C ABI
namespace nekgpu {
Handle* handle_lookup(const int64_t* h);
int handle_fail(Handle* H, int code, const std::string& msg);
}  // namespace nekgpu

using namespace nekgpu;

namespace {

Handle* p4_handle(const int64_t* handle, int* rc) {
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

// End of a splitting-step call: the kernels must have finished before the
// call returns (the caller may read the outputs from another stream).  A
// nonzero rc is a failure the call detected itself (an allocation or a
// launch); its message names the call, not the CUDA status.
int p4_done(Handle* H, int rc, const char* what) {
  const cudaError_t e = handle_leave(*H);
  if (e != cudaSuccess)
    return handle_fail(H, NEKGPU_ECUDA, std::string(what) + ": " + cudaGetErrorString(e));
  if (rc) return handle_fail(H, rc < 0 ? rc : NEKGPU_ECUDA, std::string(what) + " failed");
  return NEKGPU_OK;
}

}  // namespace

extern "C" int nekgpu_cresvsp_dev(const int64_t* handle, double* r1, double* r2, double* r3,
                                  const double* vx, const double* vy, const double* vz,
                                  const double* h1, const double* h2, const double* vdiff,
                                  const double* qtl, const double* pr, const double* bfx,
                                  const double* bfy, const double* bfz) {
  int rc;
  Handle* H = p4_handle(handle, &rc);
  if (!H) return rc;
  if (!r1 || !r2 || !r3 || !vx || !vy || !vz || !h1 || !h2 || !vdiff || !qtl || !pr || !bfx ||
      !bfy || !bfz)
    return handle_fail(H, NEKGPU_EINVAL, "null argument");
  const int64_t n = H->mesh.n;
  cudaStream_t s = H->stream;
  if (H->io0.ensure(n) || H->io1.ensure(n) || H->io2.ensure(n) || H->io3.ensure(n))
    return handle_fail(H, NEKGPU_ENOMEM, "device allocation failed");
  Coef<double> c;
  if (detect_coef<double>(*H, h1, h2, n, c))
    return handle_fail(H, NEKGPU_ECUDA, "coefficient scan failed");
  double* r[3] = {r1, r2, r3};
  const double* v[3] = {vx, vy, vz};
  const double* bf[3] = {bfx, bfy, bfz};
  for (int k = 0; k < 3; ++k)  // ophx
    if (axhelm_any(*H, r[k], v[k], c)) return p4_done(H, -3, "cresvsp operator");
  double *ta = H->io0.ptr, *t[3] = {H->io1.ptr, H->io2.ptr, H->io3.ptr};
  count_launch();
  p4_ta4_kernel<<<pblocks(n), 256, 0, s>>>(ta, vdiff, qtl, pr, -1. / 3., n);
  if (launch_gradop(*H, 0, t[0], t[1], t[2], ta, nullptr, nullptr, 0, nullptr))
    return handle_fail(H, NEKGPU_EINVAL, "cresvsp: lx1 out of range");
  for (int k = 0; k < 3; ++k) {
    count_launch();
    p4_resv_kernel<<<pblocks(n), 256, 0, s>>>(r[k], t[k], bf[k], n);
  }
  return p4_done(H, 0, "cresvsp");
}

extern "C" int nekgpu_cresvsp_weak_dev(const int64_t* handle, double* r1, double* r2, double* r3,
                                       const double* vx, const double* vy, const double* vz,
                                       const double* h1, const double* h2, const double* vdiff,
                                       const double* qtl, const double* pr, const double* bfx,
                                       const double* bfy, const double* bfz, const int* stress) {
  int rc;
  Handle* H = p4_handle(handle, &rc);
  if (!H) return rc;
  if (!r1 || !r2 || !r3 || !vx || !vy || !vz || !h1 || !h2 || !vdiff || !qtl || !pr || !bfx ||
      !bfy || !bfz || !stress)
    return handle_fail(H, NEKGPU_EINVAL, "null argument");
  const int64_t n = H->mesh.n;
  cudaStream_t s = H->stream;
  if (H->io0.ensure(n) || H->io1.ensure(n) || H->io2.ensure(n) || H->io3.ensure(n) ||
      H->io4.ensure(n))
    return handle_fail(H, NEKGPU_ENOMEM, "device allocation failed");
  Coef<double> c;
  if (detect_coef<double>(*H, h1, h2, n, c))
    return handle_fail(H, NEKGPU_ECUDA, "coefficient scan failed");
  double* r[3] = {r1, r2, r3};
  const double* v[3] = {vx, vy, vz};
  const double* bf[3] = {bfx, bfy, bfz};
  for (int k = 0; k < 3; ++k)  // ophx
    if (axhelm_any(*H, r[k], v[k], c)) return p4_done(H, -3, "cresvsp_weak operator");
  double *ta = H->io0.ptr, *t[3] = {H->io1.ptr, H->io2.ptr, H->io3.ptr}, *wa = H->io4.ptr;
  count_launch();
  p4_ta4w_kernel<<<pblocks(n), 256, 0, s>>>(ta, vdiff, qtl, *stress ? 2. / 3. : -1. / 3., n);
  if (launch_gradop(*H, 0, t[0], t[1], t[2], ta, nullptr, nullptr, 0, nullptr))  // opgrad
    return handle_fail(H, NEKGPU_EINVAL, "cresvsp_weak: lx1 out of range");
  for (int k = 0; k < 3; ++k) {
    launch_gradop(*H, 2, wa, nullptr, nullptr, pr, nullptr, nullptr, k, H->mesh.f64.bm1);  // cdtp
    count_launch();
    p4_sub_kernel<<<pblocks(n), 256, 0, s>>>(t[k], wa, n);
  }
  for (int k = 0; k < 3; ++k) {
    count_launch();
    p4_resv_kernel<<<pblocks(n), 256, 0, s>>>(r[k], t[k], bf[k], n);
  }
  return p4_done(H, 0, "cresvsp_weak");
}

extern "C" int nekgpu_crespsp_dev(const int64_t* handle, double* respr, const double* vxe,
                                  const double* vye, const double* vze, const double* pr,
                                  const double* qtl, const double* vdiff, const double* vtrans,
                                  const double* bfx, const double* bfy, const double* bfz,
                                  const double* binv, const double* dtbd, const int* null_space,
                                  const double* vx, const double* vy, const double* vz,
                                  const int* fbc) {
  int rc;
  Handle* H = p4_handle(handle, &rc);
  if (!H) return rc;
  if (!respr || !vxe || !vye || !vze || !pr || !qtl || !vdiff || !vtrans || !bfx || !bfy ||
      !bfz || !binv || !dtbd)
    return handle_fail(H, NEKGPU_EINVAL, "null argument");
  const int64_t n = H->mesh.n;
  cudaStream_t s = H->stream;
  if (H->io0.ensure(n) || H->io1.ensure(n) || H->io2.ensure(n) || H->io3.ensure(n) ||
      H->io4.ensure(n) || H->io5.ensure(n) || H->io6.ensure(n) || H->io7.ensure(n) ||
      H->red.ensure(152 * 8))
    return handle_fail(H, NEKGPU_ENOMEM, "device allocation failed");
  const double* bm1 = H->mesh.f64.bm1;
  double *ta[3] = {H->io0.ptr, H->io1.ptr, H->io2.ptr}, *wa[3] = {H->io3.ptr, H->io4.ptr, H->io5.ptr};
  double *hh1 = H->io6.ptr, *hh2 = H->io7.ptr;
  const double* bf[3] = {bfx, bfy, bfz};
  // curl curl of the extrapolated velocity, both curls averaged
  if (launch_gradop(*H, 3, ta[0], ta[1], ta[2], vxe, vye, vze, 0, nullptr))
    return handle_fail(H, NEKGPU_EINVAL, "crespsp: lx1 out of range");
  for (double* w : ta) {
    launch_mul_by(*H, w, bm1);
    gs_op<double>(H->mesh.gs, w, 0, s);
    launch_mul_by(*H, w, binv);
  }
  launch_gradop(*H, 3, wa[0], wa[1], wa[2], ta[0], ta[1], ta[2], 0, nullptr);
  for (double* w : wa) {
    launch_mul_by(*H, w, bm1);
    gs_op<double>(H->mesh.gs, w, 0, s);
    launch_mul_by(*H, w, binv);
  }
  launch_gradop(*H, 0, ta[0], ta[1], ta[2], qtl, nullptr, nullptr, 0, nullptr);  // opgrad(qtl)
  for (int k = 0; k < 3; ++k) {
    count_launch();
    p4_wa_kernel<<<pblocks(n), 256, 0, s>>>(wa[k], ta[k], bm1, vdiff, vtrans, -4. / 3., n);
  }
  count_launch();
  p4_h_kernel<<<pblocks(n), 256, 0, s>>>(hh1, hh2, vtrans, n);
  Coef<double> c;
  if (detect_coef<double>(*H, hh1, hh2, n, c))
    return handle_fail(H, NEKGPU_ECUDA, "coefficient scan failed");
  if (axhelm_any(*H, respr, pr, c)) return p4_done(H, -3, "crespsp operator");
  for (int k = 0; k < 3; ++k) {
    count_launch();
    p4_tb_kernel<<<pblocks(n), 256, 0, s>>>(ta[k], bf[k], vtrans, wa[k], n);
    gs_op<double>(H->mesh.gs, ta[k], 0, s);
    launch_mul_by(*H, ta[k], binv);
    launch_gradop(*H, 2, wa[k], nullptr, nullptr, ta[k], nullptr, nullptr, k, bm1);  // cdtp
  }
  count_launch();
  p4_respr_kernel<<<pblocks(n), 256, 0, s>>>(respr, wa[0], wa[1], wa[2], qtl, bm1, *dtbd, n);
  if (fbc) {  // face terms on velocity and symmetry faces
    bool vel = false;
    for (int q = 0; q < 6 * H->mesh.nel; ++q) {
      if (fbc[q] < 0 || fbc[q] > 3) return handle_fail(H, NEKGPU_EINVAL, "face types are 0..3");
      vel = vel || fbc[q] == 1 || fbc[q] == 2;
    }
    if (vel && (!vx || !vy || !vz))
      return handle_fail(H, NEKGPU_EINVAL, "velocity faces need vx, vy, vz");
    if (H->p4_fbc.ensure((size_t)6 * H->mesh.nel))
      return handle_fail(H, NEKGPU_ENOMEM, "device allocation failed");
    cudaMemcpyAsync(H->p4_fbc.ptr, fbc, (size_t)6 * H->mesh.nel * sizeof(int),
                    cudaMemcpyHostToDevice, s);
    count_launch();
    p4_face_kernel<<<H->mesh.nel, 64, 0, s>>>(respr, vx, vy, vz, ta[0], ta[1], ta[2],
                                              H->p4_fbc.ptr, H->mesh.rst.ptr, H->mesh.w1.ptr,
                                              *dtbd, H->mesh.nx1, n);
  }
  if (null_space && *null_space) {  // ortho
    const int nb = pblocks(n);
    count_launch();
    p4_sum_kernel<<<nb, 256, 0, s>>>(respr, n, H->red.ptr);
    std::vector<double> part((size_t)nb);
    cudaMemcpyAsync(part.data(), H->red.ptr, nb * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (cudaStreamSynchronize(s) != cudaSuccess) return p4_done(H, -3, "crespsp ortho");
    double sum = 0.0;
    for (double v : part) sum += v;
    count_launch();
    p4_cadd_kernel<<<pblocks(n), 256, 0, s>>>(respr, -(sum / (double)n), n);
  }
  return p4_done(H, 0, "crespsp");
}

namespace {

Handle* p4_mesh_handle(const int64_t* handle, int* rc) {
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

}  // namespace

extern "C" int nekgpu_makeabf_dev(const int64_t* handle, double* bf, double* abx1, double* abx2,
                                  const double* vtrans, const double* ab) {
  int rc;
  Handle* H = p4_mesh_handle(handle, &rc);
  if (!H) return rc;
  if (!bf || !abx1 || !abx2 || !vtrans || !ab) return handle_fail(H, NEKGPU_EINVAL, "null argument");
  const int64_t n = H->mesh.n;
  count_launch();
  p4_makeabf_kernel<<<pblocks(n), 256, 0, H->stream>>>(bf, abx1, abx2, vtrans, ab[0], ab[1],
                                                      ab[2], n);
  return p4_done(H, 0, "makeabf");
}

extern "C" int nekgpu_makebdf_dev(const int64_t* handle, double* bf, const double* v,
                                  const double* vlag, const double* vtrans, const double* bd,
                                  const int* nbd, const double* dt) {
  int rc;
  Handle* H = p4_mesh_handle(handle, &rc);
  if (!H) return rc;
  if (!bf || !v || !vtrans || !bd || !nbd || !dt || *nbd < 1 || *nbd > 3 || (*nbd > 1 && !vlag))
    return handle_fail(H, NEKGPU_EINVAL, "bad argument (1 <= nbd <= 3, lags for nbd > 1)");
  const int64_t n = H->mesh.n;
  Bd c{{0.0, 0.0, 0.0, 0.0}};
  for (int q = 0; q <= *nbd; ++q) c.c[q] = bd[q];
  count_launch();
  p4_makebdf_kernel<<<pblocks(n), 256, 0, H->stream>>>(bf, v, vlag, *nbd - 1, H->mesh.f64.bm1,
                                                      vtrans, c, 1. / *dt, n);
  return p4_done(H, 0, "makebdf");
}

extern "C" int nekgpu_sumab_dev(const int64_t* handle, double* v, const double* vv,
                                const double* vvlag, const double* ab, const int* nab) {
  int rc;
  Handle* H = p4_mesh_handle(handle, &rc);
  if (!H) return rc;
  if (!v || !vv || !vvlag || !ab || !nab || *nab < 2 || *nab > 3)
    return handle_fail(H, NEKGPU_EINVAL, "bad argument (nab 2 or 3)");
  const int64_t n = H->mesh.n;
  count_launch();
  p4_sumab_kernel<<<pblocks(n), 256, 0, H->stream>>>(v, vv, vvlag, ab[0], ab[1],
                                                    *nab == 3 ? ab[2] : 0.0, *nab, n);
  return p4_done(H, 0, "sumab");
}
