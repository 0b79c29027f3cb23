// geom.cu -- geometric factors and mass on the device from the GLL
// coordinates: the reference's xyzrst (core/coef.f:879-926), glmapm1
// (:555-631) and geodat1 (:633-784), with W3M1 = w(i) w(j) w(k) (genwz
// :263-267).  Every product, sum and the reciprocal of the Jacobian are
// rounded one by one in the reference's order (no fused multiply-adds), so
// the result is the reference's bit for bit.  Used by nekgpu_setup_xyz and,
// for a moving mesh, nekgpu_geom_update_dev.
#include <string>
#include <vector>

#include "impl.cuh"

namespace nekgpu {
namespace {

// One element per block, thread (i, j) walks its z-column.  D row-major
// (D(i, l) at D[i NX + l]); w the GLL weights; G packed [e][6][P].
template <int NX>
__global__ void __launch_bounds__(NX* NX) geom_kernel(const double* __restrict__ x,
                                                      const double* __restrict__ y,
                                                      const double* __restrict__ z,
                                                      const double* __restrict__ D,
                                                      const double* __restrict__ w,
                                                      double* __restrict__ G,
                                                      double* __restrict__ bm1, int* bad,
                                                      double* __restrict__ rst,
                                                      double* __restrict__ jacm1, int64_t n) {
  constexpr int P = NX * NX * NX, NXY = NX * NX;
  __shared__ double sx[P], sy[P], sz[P], sD[NXY], sw[NX];
  const int e = blockIdx.x, tid = threadIdx.x;
  const size_t eo = (size_t)e * P;
  for (int q = tid; q < P; q += NXY) {
    sx[q] = x[eo + q];
    sy[q] = y[eo + q];
    sz[q] = z[eo + q];
  }
  for (int q = tid; q < NXY; q += NXY) sD[q] = D[q];
  if (tid < NX) sw[tid] = w[tid];
  __syncthreads();
  const int i = tid % NX, j = tid / NX;
  double* Ge = G + (size_t)e * 6 * P;
  for (int k = 0; k < NX; ++k) {
    const int pt = i + NX * (j + NX * k);
    // d/dr: sum_l D(i,l) u(l,j,k); d/ds: sum_l u(i,l,k) D(j,l); d/dt: sum_l u(i,j,l) D(k,l)
    double d[3][3];  // [u = x, y, z][r, s, t]
    const double* su[3] = {sx, sy, sz};
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double* u = su[c];
      double r = __dmul_rn(sD[i * NX], u[NX * (j + NX * k)]);
      double s = __dmul_rn(u[i + NX * NX * k], sD[j * NX]);
      double t = __dmul_rn(u[i + NX * j], sD[k * NX]);
#pragma unroll
      for (int l = 1; l < NX; ++l) {
        r = __dadd_rn(r, __dmul_rn(sD[i * NX + l], u[l + NX * (j + NX * k)]));
        s = __dadd_rn(s, __dmul_rn(u[i + NX * (l + NX * k)], sD[j * NX + l]));
        t = __dadd_rn(t, __dmul_rn(u[i + NX * (j + NX * l)], sD[k * NX + l]));
      }
      d[c][0] = r;
      d[c][1] = s;
      d[c][2] = t;
    }
    const double xr = d[0][0], xs = d[0][1], xt = d[0][2];
    const double yr = d[1][0], ys = d[1][1], yt = d[1][2];
    const double zr = d[2][0], zs = d[2][1], zt = d[2][2];
    auto m3 = [](double a, double b, double c) { return __dmul_rn(__dmul_rn(a, b), c); };
    // Jacobian: three products added, three subtracted (glmapm1's ADDCOL4 / SUBCOL4)
    double jac = __dadd_rn(0.0, m3(xr, ys, zt));
    jac = __dadd_rn(jac, m3(xt, yr, zs));
    jac = __dadd_rn(jac, m3(xs, yt, zr));
    jac = __dsub_rn(jac, m3(xr, yt, zs));
    jac = __dsub_rn(jac, m3(xs, yr, zt));
    jac = __dsub_rn(jac, m3(xt, ys, zr));
    // cofactors (ASCOL5): J grad r, J grad s, J grad t
    auto cof = [](double a, double b, double c, double d2) {
      return __dsub_rn(__dmul_rn(a, b), __dmul_rn(c, d2));
    };
    const double rx = cof(ys, zt, yt, zs), ry = cof(xt, zs, xs, zt), rz = cof(xs, yt, xt, ys);
    const double sxv = cof(yt, zr, yr, zt), syv = cof(xr, zt, xt, zr), szv = cof(xt, yr, xr, yt);
    const double tx = cof(yr, zs, ys, zr), ty = cof(xs, zr, xr, zs), tz = cof(xr, ys, xs, yr);
    auto dot3 = [](double a1, double b1, double a2, double b2, double a3, double b3) {
      return __dadd_rn(__dadd_rn(__dmul_rn(a1, b1), __dmul_rn(a2, b2)), __dmul_rn(a3, b3));
    };
    const double wj = __ddiv_rn(1.0, jac);
    const double w3 = __dmul_rn(__dmul_rn(sw[i], sw[j]), sw[k]);
    const double a[6] = {dot3(rx, rx, ry, ry, rz, rz),    dot3(sxv, sxv, syv, syv, szv, szv),
                         dot3(tx, tx, ty, ty, tz, tz),    dot3(rx, sxv, ry, syv, rz, szv),
                         dot3(rx, tx, ry, ty, rz, tz),    dot3(sxv, tx, syv, ty, szv, tz)};
#pragma unroll
    for (int q = 0; q < 6; ++q) Ge[q * P + pt] = __dmul_rn(__dmul_rn(a[q], wj), w3);
    bm1[eo + pt] = __dmul_rn(jac, w3);
    if (rst) {  // the metric terms and the Jacobian themselves
      const double m9[9] = {rx, ry, rz, sxv, syv, szv, tx, ty, tz};
#pragma unroll
      for (int q = 0; q < 9; ++q) rst[(int64_t)q * n + eo + pt] = m9[q];
      jacm1[eo + pt] = jac;
    }
    if (!(jac > 0.0)) atomicOr(bad, 1);
  }
}

template <int NX>
void launch_nx(int nel, const double* x, const double* y, const double* z, const double* D,
               const double* w, double* G, double* bm1, int* bad, double* rst, double* jac,
               int64_t n, cudaStream_t s) {
  count_launch();
  geom_kernel<NX><<<nel, NX * NX, 0, s>>>(x, y, z, D, w, G, bm1, bad, rst, jac, n);
}

}  // namespace

// G and bm1 of the handle's mesh (allocated, D set) from device coordinates;
// vol = glsum(bm1) summed left to right on the host as one rank of the
// reference.  w: host GLL weights.  Returns 0 or an NEKGPU_E* code.
int geom_from_xyz(Handle& H, const double* x, const double* y, const double* z, const double* w,
                  std::string& err) {
  Mesh& m = H.mesh;
  const int64_t n = m.n;
  DevBuf<double> wd;
  const int64_t nxyz = (int64_t)m.nx1 * m.nx1 * m.nx1;
  if (wd.ensure(m.nx1) || m.rst.ensure((size_t)9 * n) || m.jac.ensure(n) || m.w3.ensure(nxyz) ||
      m.w1.ensure(m.nx1)) {
    err = "geometry: allocation failed";
    return NEKGPU_ENOMEM;
  }
  cudaMemcpyAsync(wd.ptr, w, m.nx1 * sizeof(double), cudaMemcpyHostToDevice, H.stream);
  cudaMemcpyAsync(m.w1.ptr, w, m.nx1 * sizeof(double), cudaMemcpyHostToDevice, H.stream);
  {  // w3m1 = w(i) w(j) w(k), in that order (genwz)
    std::vector<double> w3((size_t)nxyz);
    for (int k = 0; k < m.nx1; ++k)
      for (int j = 0; j < m.nx1; ++j)
        for (int i = 0; i < m.nx1; ++i) w3[i + m.nx1 * (j + (int64_t)m.nx1 * k)] = w[i] * w[j] * w[k];
    cudaMemcpyAsync(m.w3.ptr, w3.data(), nxyz * sizeof(double), cudaMemcpyHostToDevice, H.stream);
    cudaStreamSynchronize(H.stream);  // w3 is a host temporary
  }
  cudaMemsetAsync(H.flag, 0, sizeof(int), H.stream);
  switch (m.nx1) {
#define NEKGPU_GEOM_CASE(N) \
  case N:                                                                                    \
    launch_nx<N>(m.nel, x, y, z, m.f64.D, wd.ptr, m.f64.G, m.f64.bm1, H.flag, m.rst.ptr, m.jac.ptr, \
                 n, H.stream);                                                                  \
    break;
    NEKGPU_GEOM_CASE(2)
    NEKGPU_GEOM_CASE(3)
    NEKGPU_GEOM_CASE(4)
    NEKGPU_GEOM_CASE(5)
    NEKGPU_GEOM_CASE(6)
    NEKGPU_GEOM_CASE(7)
    NEKGPU_GEOM_CASE(8)
    NEKGPU_GEOM_CASE(9)
    NEKGPU_GEOM_CASE(10)
    NEKGPU_GEOM_CASE(11)
    NEKGPU_GEOM_CASE(12)
#undef NEKGPU_GEOM_CASE
    default:
      err = "geometry: lx1 out of range";
      return NEKGPU_EINVAL;
  }
  int bad = 0;
  cudaMemcpyAsync(&bad, H.flag, sizeof(int), cudaMemcpyDeviceToHost, H.stream);
  std::vector<double> hb((size_t)n);
  cudaMemcpyAsync(hb.data(), m.f64.bm1, n * sizeof(double), cudaMemcpyDeviceToHost, H.stream);
  cudaError_t e = cudaStreamSynchronize(H.stream);
  if (e != cudaSuccess) {
    err = std::string("geometry: ") + cudaGetErrorString(e);
    return NEKGPU_ECUDA;
  }
  if (bad) {
    err = "geometry: non-positive Jacobian (tangled element map)";
    return NEKGPU_EINVAL;
  }
  double vol = 0.0;
  for (int64_t i = 0; i < n; ++i) vol = vol + hb[(size_t)i];
  m.vol = vol;
  m.has_rst = true;
  if (H.dealias) {  // the fine-grid metric terms follow the moved geometry
    const int md = dealias_lxd(H);
    const int rc = dealias_setup(H, md, err);
    if (rc) return rc;
  }
  // the FP32 copy of the operator data no longer matches
  m.f32.release();
  m.has_f32 = false;
  m.has_df = false;
  return NEKGPU_OK;
}

}  // namespace nekgpu
