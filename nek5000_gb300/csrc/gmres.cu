// gmres.cu -- the pressure solve's Krylov method on the device: hmh_gmres
// (core/gmres.f:304-560), right-preconditioned restarted GMRES on
// ax() = mask * dssum(axhelm(x)) (gmres.f:284-302) with weights wt (vmult).
//
// Per inner iteration: z_j = M v_j (and the mean removed when the operator
// has a null space, ortho, core/navier1.f:223-256), w = A z_j, the j
// weighted dot products (w, v_i) in one pass per eight vectors, w -= sum
// h_ij v_i point by point in i order fused with (w, w), then the Givens
// rotation, the residual estimate and v_{j+1} = w / alpha.  Pointwise
// arithmetic is rounded as the reference's (no fused multiply-adds); the
// dot products are block sums added on the host in block order.
//
// The reference preconditions with h1mg_solve (gmres.f:407-411), the
// multilevel Schwarz method of h1mg.cu; M is that once nekgpu_h1mg_setup
// has run on the handle, else the Jacobi diagonal of setprec (iteration
// counts then are that method's; the solution is the same linear system's
// to the tolerance).
#include <cmath>
#include <string>
#include <vector>

#include "impl.cuh"

namespace nekgpu {
namespace {

constexpr int kT = 256;
constexpr int kDots = 8;  // weighted dot products per pass

inline int nblocks(int64_t n) {  // about four points per thread, at most 152 x 6 blocks
  return (int)std::min<int64_t>(std::max<int64_t>((n + 4 * kT - 1) / (4 * kT), 1), 152 * 6);
}

__device__ __forceinline__ double block_reduce(double v, double* red) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x == 0)
    for (int q = 0; q < kT / 32; ++q) s += red[q];
  return s;
}

// partial[blk] = sum a b wt over the block's points (glsc3 / vlsc3 terms)
__global__ void __launch_bounds__(kT) wdot_kernel(const double* __restrict__ a,
                                                  const double* __restrict__ b,
                                                  const double* __restrict__ wt, int64_t n,
                                                  double* __restrict__ partial) {
  __shared__ double red[kT / 32];
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)kT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kT)
    s += __dmul_rn(__dmul_rn(a[i], b[i]), wt[i]);
  s = block_reduce(s, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// partial[blk * kDots + k] = sum w v_k wt, k < CNT, v_k = V + k n; the CNT
// sums of a block reduced together (one shared-memory exchange)
template <int CNT>
__global__ void __launch_bounds__(kT) mdot_kernel(const double* __restrict__ w,
                                                  const double* __restrict__ V,
                                                  const double* __restrict__ wt, int64_t n,
                                                  double* __restrict__ partial) {
  __shared__ double red[kT / 32][CNT];
  double acc[CNT];
#pragma unroll
  for (int k = 0; k < CNT; ++k) acc[k] = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)kT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kT) {
    const double ww = w[i], t = wt[i];
#pragma unroll
    for (int k = 0; k < CNT; ++k) acc[k] += __dmul_rn(__dmul_rn(ww, V[(int64_t)k * n + i]), t);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < CNT; ++k) {
    double v = acc[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[wid][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < CNT) {
    double t = 0.0;
    for (int q = 0; q < kT / 32; ++q) t += red[q][threadIdx.x];
    partial[(int64_t)blockIdx.x * kDots + threadIdx.x] = t;
  }
}

void launch_mdot(int cnt, int nb, cudaStream_t s, const double* w, const double* V,
                 const double* wt, int64_t n, double* partial) {
  count_launch();
  switch (cnt) {
#define NEKGPU_MDOT(C) \
  case C: mdot_kernel<C><<<nb, kT, 0, s>>>(w, V, wt, n, partial); break;
    NEKGPU_MDOT(1)
    NEKGPU_MDOT(2)
    NEKGPU_MDOT(3)
    NEKGPU_MDOT(4)
    NEKGPU_MDOT(5)
    NEKGPU_MDOT(6)
    NEKGPU_MDOT(7)
    default: mdot_kernel<8><<<nb, kT, 0, s>>>(w, V, wt, n, partial); break;
#undef NEKGPU_MDOT
  }
}

// w = w + (-h_i) v_i for i < j in order (add2s2), then partial = sum w w wt
__global__ void __launch_bounds__(kT) msub_kernel(double* __restrict__ w,
                                                  const double* __restrict__ V, int j,
                                                  const double* __restrict__ h,
                                                  const double* __restrict__ wt, int64_t n,
                                                  double* __restrict__ partial) {
  __shared__ double red[kT / 32];
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)kT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kT) {
    double v = w[i];
    for (int k = 0; k < j; ++k) v = __dadd_rn(v, __dmul_rn(-h[k], V[(int64_t)k * n + i]));
    w[i] = v;
    s += __dmul_rn(__dmul_rn(v, v), wt[i]);
  }
  s = block_reduce(s, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

// x = x + c_i z_i for i < j in order (add2s2)
__global__ void xupd_kernel(double* __restrict__ x, const double* __restrict__ Z, int j,
                            const double* __restrict__ c, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    double v = x[i];
    for (int k = 0; k < j; ++k) v = __dadd_rn(v, __dmul_rn(c[k], Z[(int64_t)k * n + i]));
    x[i] = v;
  }
}

// z = d (1 v) (the preconditioner on mu v); partial = sum z (for ortho)
__global__ void __launch_bounds__(kT) prec_kernel(double* __restrict__ z,
                                                  const double* __restrict__ d,
                                                  const double* __restrict__ v, int64_t n,
                                                  double* __restrict__ partial) {
  __shared__ double red[kT / 32];
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)kT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kT) {
    const double zz = __dmul_rn(d[i], v[i]);
    z[i] = zz;
    s += zz;
  }
  s = block_reduce(s, red);
  if (threadIdx.x == 0 && partial) partial[blockIdx.x] = s;
}

__global__ void sum_kernel(const double* __restrict__ a, int64_t n, double* __restrict__ partial) {
  __shared__ double red[kT / 32];
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)kT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kT)
    s += a[i];
  s = block_reduce(s, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

__global__ void cadd_kernel(double* __restrict__ a, double c, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    a[i] = __dadd_rn(a[i], c);
}

__global__ void scale_kernel(double* __restrict__ dst, const double* __restrict__ src, double c,
                             int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = __dmul_rn(src[i], c);
}

__global__ void mask_kernel(double* __restrict__ w, const double* __restrict__ m, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    w[i] = __dmul_rn(w[i], m[i]);
}

// r = res + (-1) w (copy + add2s2)
__global__ void resid_kernel(double* __restrict__ r, const double* __restrict__ res,
                             const double* __restrict__ w, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    r[i] = __dadd_rn(res[i], -w[i]);
}

// Flexible CG (hmh_flex_cg): z = M r; t = r1 - r (sub2); partial sums
// (z wt) r and (z wt) t; then r1 = r (the lagged residual)
__global__ void __launch_bounds__(kT) fcg_rho_kernel(double* __restrict__ z,
                                                     const double* __restrict__ d,
                                                     const double* __restrict__ r,
                                                     double* __restrict__ r1,
                                                     const double* __restrict__ wt, int64_t n,
                                                     double* __restrict__ partial) {
  __shared__ double red[kT / 32][2];
  double a = 0.0, b = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)kT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kT) {
    const double ri = r[i];
    const double zz = d ? __dmul_rn(d[i], ri) : z[i];  // d null: z = M r already formed
    const double t = __dsub_rn(r1[i], ri);
    const double zw = __dmul_rn(zz, wt[i]);
    a += __dmul_rn(zw, ri);
    b += __dmul_rn(zw, t);
    if (d) z[i] = zz;
    r1[i] = ri;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (lane == 0) {
    red[wid][0] = a;
    red[wid][1] = b;
  }
  __syncthreads();
  if (threadIdx.x < 2) {
    double s = 0.0;
    for (int q = 0; q < kT / 32; ++q) s += red[q][threadIdx.x];
    partial[(int64_t)blockIdx.x * 2 + threadIdx.x] = s;
  }
}

// p = beta p + z (add2s1)
__global__ void fcg_p_kernel(double* __restrict__ p, const double* __restrict__ z, double beta,
                             int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    p[i] = __dadd_rn(__dmul_rn(beta, p[i]), z[i]);
}

// x += alpha p; r -= alpha w; partial = sum (r r) wt
__global__ void __launch_bounds__(kT) fcg_xr_kernel(double* __restrict__ x,
                                                    double* __restrict__ r,
                                                    const double* __restrict__ p,
                                                    const double* __restrict__ w, double alpha,
                                                    const double* __restrict__ wt, int64_t n,
                                                    double* __restrict__ partial) {
  __shared__ double red[kT / 32];
  double s = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)kT + threadIdx.x; i < n; i += (int64_t)gridDim.x * kT) {
    x[i] = __dadd_rn(x[i], __dmul_rn(alpha, p[i]));
    const double rr = __dsub_rn(r[i], __dmul_rn(alpha, w[i]));
    r[i] = rr;
    s += __dmul_rn(__dmul_rn(rr, rr), wt[i]);
  }
  s = block_reduce(s, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

struct Gm {
  Handle& h;
  cudaStream_t s;
  int64_t n;
  int nb;
  std::vector<double> host;

  // the block partials (nb * per) summed in block order
  int sums(int per, int cnt, double* out) {
    host.resize((size_t)nb * per);
    cudaMemcpyAsync(host.data(), h.red.ptr, host.size() * sizeof(double), cudaMemcpyDeviceToHost,
                    s);
    if (cudaStreamSynchronize(s) != cudaSuccess) {
      set_error(h, std::string("gmres: ") + cudaGetErrorString(cudaGetLastError()));
      return -3;
    }
    for (int k = 0; k < cnt; ++k) {
      double t = 0.0;
      for (int b = 0; b < nb; ++b) t += host[(size_t)b * per + k];
      out[k] = t;
    }
    return 0;
  }
};

}  // namespace

// hmh_gmres with the Jacobi preconditioner; res: in the right-hand side, out
// the solution.  Returns 0, -3 (CUDA), -4 (allocation), -5 (iteration cap
// reached above the tolerance).
int gmres_solve(Handle& h, double* res, const double* h1, const double* h2, const double* wt,
                const double* mask, double tol, int maxit, int m, bool null_space, int* niter,
                double* div0_out, double* rnorm_out) {
  Mesh& msh = h.mesh;
  const int64_t n = msh.n;
  cudaStream_t s = h.stream;
  Gm g{h, s, n, nblocks(n), {}};
  const int nb = g.nb;
  if (h.gm_V.ensure((size_t)m * n) || h.gm_Z.ensure((size_t)m * n) || h.gm_r.ensure(n) ||
      h.gm_w.ensure(n) || h.gm_x.ensure(n) || h.gm_d.ensure(n) || h.gm_c.ensure(m + 1) ||
      h.red.ensure((size_t)nb * kDots)) {
    set_error(h, "gmres: device allocation failed");
    return -4;
  }
  Coef<double> c;
  if (detect_coef<double>(h, h1, h2, n, c)) {
    set_error(h, "gmres: coefficient scan failed");
    return -3;
  }
  if (setprec_f64(h, h.gm_d.ptr, c)) {
    set_error(h, "gmres: setprec failed");
    return -3;
  }
  double *V = h.gm_V.ptr, *Z = h.gm_Z.ptr, *r = h.gm_r.ptr, *w = h.gm_w.ptr, *x = h.gm_x.ptr;
  const double* d = h.gm_d.ptr;
  auto apply_A = [&](double* out, const double* in) -> int {
    cudaError_t e = h.exact ? launch_axhelm<double, true>(msh, msh.f64, out, in, c, s)
                            : launch_axhelm<double, false>(msh, msh.f64, out, in, c, s);
    if (e != cudaSuccess) {
      set_error(h, std::string("gmres: operator launch: ") + cudaGetErrorString(e));
      return -3;
    }
    gs_op<double>(msh.gs, out, 0, s);
    count_launch();
    mask_kernel<<<nb, kT, 0, s>>>(out, mask, n);
    return 0;
  };
  auto ortho = [&](double* z, const double* partial_done) -> int {
    if (!null_space) return 0;
    if (!partial_done) {
      count_launch();
      sum_kernel<<<nb, kT, 0, s>>>(z, n, h.red.ptr);
    }
    double sum = 0.0;
    if (g.sums(1, 1, &sum)) return -3;
    count_launch();
    cadd_kernel<<<nb, kT, 0, s>>>(z, -(sum / (double)n), n);
    return 0;
  };
  cudaMemsetAsync(x, 0, n * sizeof(double), s);
  const double norm_fac = 1.0 / std::sqrt(msh.vol);
  double tolpss = std::fabs(tol), div0 = 0.0, rnorm = 0.0;
  std::vector<double> H((size_t)(m + 1) * (m + 1), 0.0), cs((size_t)m + 1), sn((size_t)m + 1),
      gam((size_t)m + 2), hcol((size_t)m + 1);
  auto HM = [&](int i, int j) -> double& { return H[(size_t)i + (size_t)(m + 1) * j]; };
  int iter = 0;
  bool conv = false;
  while (!conv) {
    if (iter == 0) {
      cudaMemcpyAsync(r, res, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
    } else {
      if (apply_A(w, x)) return -3;
      count_launch();
      resid_kernel<<<nb, kT, 0, s>>>(r, res, w, n);
    }
    count_launch();
    wdot_kernel<<<nb, kT, 0, s>>>(r, r, wt, n, h.red.ptr);
    double rr = 0.0;
    if (g.sums(1, 1, &rr)) return -3;
    gam[0] = std::sqrt(rr);
    if (iter == 0) {
      div0 = gam[0] * norm_fac;
      if (tol < 0) tolpss = std::fabs(tol) * div0;
    }
    rnorm = 0.0;
    if (gam[0] == 0.0) break;  // lucky convergence
    count_launch();
    scale_kernel<<<nb, kT, 0, s>>>(V, r, 1.0 / gam[0], n);
    int j = 0;
    for (j = 0; j < m; ++j) {
      ++iter;
      double* zj = Z + (size_t)n * j;
      const double* vj = V + (size_t)n * j;
      if (h.mg) {  // h1mg_solve(z_j, w = mu v_j); w is masked in place, then overwritten
        cudaMemcpyAsync(w, vj, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
        if (h1mg_apply(h, zj, w)) return -3;
        if (ortho(zj, nullptr)) return -3;
      } else {
        count_launch();
        prec_kernel<<<nb, kT, 0, s>>>(zj, d, vj, n, null_space ? h.red.ptr : nullptr);
        if (ortho(zj, null_space ? h.red.ptr : nullptr)) return -3;
      }
      if (apply_A(w, zj)) return -3;
      // h_ij = (w, v_i), i <= j, eight vectors per pass
      for (int i0 = 0; i0 <= j; i0 += kDots) {
        const int cnt = std::min(kDots, j + 1 - i0);
        launch_mdot(cnt, nb, s, w, V + (size_t)n * i0, wt, n, h.red.ptr);
        if (g.sums(kDots, cnt, &hcol[(size_t)i0])) return -3;
      }
      for (int i = 0; i <= j; ++i) HM(i, j) = hcol[(size_t)i];
      cudaMemcpyAsync(h.gm_c.ptr, hcol.data(), (j + 1) * sizeof(double), cudaMemcpyHostToDevice,
                      s);
      count_launch();
      msub_kernel<<<nb, kT, 0, s>>>(w, V, j + 1, h.gm_c.ptr, wt, n, h.red.ptr);
      double ww = 0.0;
      if (g.sums(1, 1, &ww)) return -3;
      for (int i = 0; i < j; ++i) {  // Givens rotations on the new column
        const double t = HM(i, j);
        HM(i, j) = cs[(size_t)i] * t + sn[(size_t)i] * HM(i + 1, j);
        HM(i + 1, j) = -sn[(size_t)i] * t + cs[(size_t)i] * HM(i + 1, j);
      }
      const double alpha = std::sqrt(ww);
      rnorm = 0.0;
      if (alpha == 0.0) {
        conv = true;
        break;
      }
      const double l = std::sqrt(HM(j, j) * HM(j, j) + alpha * alpha);
      const double tmp = 1.0 / l;
      cs[(size_t)j] = HM(j, j) * tmp;
      sn[(size_t)j] = alpha * tmp;
      HM(j, j) = l;
      gam[(size_t)j + 1] = -sn[(size_t)j] * gam[(size_t)j];
      gam[(size_t)j] = cs[(size_t)j] * gam[(size_t)j];
      rnorm = std::fabs(gam[(size_t)j + 1]) * norm_fac;
      if (iter + 1 > maxit || rnorm < tolpss) {
        conv = true;
        break;
      }
      if (j == m - 1) break;  // restart
      count_launch();
      scale_kernel<<<nb, kT, 0, s>>>(V + (size_t)n * (j + 1), w, 1.0 / alpha, n);
    }
    // back substitution, then x += sum c_i z_i
    const int jj = j < m ? j : m - 1;
    for (int k = jj; k >= 0; --k) {
      double t = gam[(size_t)k];
      for (int i = jj; i > k; --i) t = t - HM(k, i) * cs[(size_t)i];
      cs[(size_t)k] = t / HM(k, k);
    }
    cudaMemcpyAsync(h.gm_c.ptr, cs.data(), (jj + 1) * sizeof(double), cudaMemcpyHostToDevice, s);
    count_launch();
    xupd_kernel<<<nb, kT, 0, s>>>(x, Z, jj + 1, h.gm_c.ptr, n);
  }
  cudaMemcpyAsync(res, x, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  if (ortho(res, nullptr)) return -3;
  if (cudaStreamSynchronize(s) != cudaSuccess) {
    set_error(h, std::string("gmres: ") + cudaGetErrorString(cudaGetLastError()));
    return -3;
  }
  *niter = iter;
  *div0_out = div0;
  *rnorm_out = rnorm;
  if (!(rnorm < tolpss) && rnorm != 0.0 && gam[0] != 0.0) {
    set_error(h, "gmres: iteration cap reached above the tolerance");
    return -5;
  }
  return 0;
}

// hmh_flex_cg (core/hmholtz.f:2164-2289) with the Jacobi preconditioner:
// flexible (Polak-Ribiere) PCG on the same operator and weights as
// gmres_solve.  res: in the right-hand side, out the solution.  Returns 0,
// -3, -4 or -5 as gmres_solve.
int flex_cg_solve(Handle& h, double* res, const double* h1, const double* h2, const double* wt,
                  const double* mask, double tol, int maxit, bool null_space, int* niter,
                  double* div0_out, double* rnorm_out) {
  Mesh& msh = h.mesh;
  const int64_t n = msh.n;
  cudaStream_t s = h.stream;
  Gm g{h, s, n, nblocks(n), {}};
  const int nb = g.nb;
  // r, r1 (lagged residual), p, z, w: work vectors of the GMRES pool
  if (h.gm_Z.ensure((size_t)3 * n) || h.gm_r.ensure(n) || h.gm_w.ensure(n) || h.gm_d.ensure(n) ||
      h.red.ensure((size_t)nb * kDots)) {
    set_error(h, "flex cg: device allocation failed");
    return -4;
  }
  Coef<double> c;
  if (detect_coef<double>(h, h1, h2, n, c)) {
    set_error(h, "flex cg: coefficient scan failed");
    return -3;
  }
  if (setprec_f64(h, h.gm_d.ptr, c)) {
    set_error(h, "flex cg: setprec failed");
    return -3;
  }
  double *r = h.gm_r.ptr, *w = h.gm_w.ptr, *r1 = h.gm_Z.ptr, *p = r1 + n, *z = r1 + 2 * n;
  const double* d = h.gm_d.ptr;
  cudaMemcpyAsync(r, res, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  cudaMemsetAsync(res, 0, n * sizeof(double), s);
  cudaMemsetAsync(r1, 0, 2 * n * sizeof(double), s);  // r1 and p
  count_launch();
  wdot_kernel<<<nb, kT, 0, s>>>(r, wt, r, n, h.red.ptr);  // glsc3(r, wt, r)
  double t = 0.0;
  if (g.sums(1, 1, &t)) return -3;
  const double div0 = std::sqrt(t / msh.vol);
  const double tolpss = tol < 0 ? std::fabs(tol) * div0 : std::fabs(tol);
  double rho1 = 1.0, rnorm = div0;
  int iter = 0;
  // a zero right-hand side is solved by x = 0 (the reference's loop would
  // divide 0 by 0)
  for (int k = 1; k <= maxit && div0 != 0.0; ++k) {
    if (h.mg && h1mg_apply(h, z, r)) return -3;  // h1mg_solve(z, r): r masked in place
    count_launch();
    fcg_rho_kernel<<<nb, kT, 0, s>>>(z, h.mg ? nullptr : d, r, r1, wt, n, h.red.ptr);
    double rr[2];
    if (g.sums(2, 2, rr)) return -3;
    const double rho0 = rho1;
    rho1 = rr[0];
    const double beta = -rr[1] / rho0;
    count_launch();
    fcg_p_kernel<<<nb, kT, 0, s>>>(p, z, beta, n);
    cudaError_t e = h.exact ? launch_axhelm<double, true>(msh, msh.f64, w, p, c, s)
                            : launch_axhelm<double, false>(msh, msh.f64, w, p, c, s);
    if (e != cudaSuccess) {
      set_error(h, std::string("flex cg: operator launch: ") + cudaGetErrorString(e));
      return -3;
    }
    gs_op<double>(msh.gs, w, 0, s);
    count_launch(2);
    mask_kernel<<<nb, kT, 0, s>>>(w, mask, n);
    wdot_kernel<<<nb, kT, 0, s>>>(w, wt, p, n, h.red.ptr);  // glsc3(w, wt, p)
    double den = 0.0;
    if (g.sums(1, 1, &den)) return -3;
    const double alpha = rho1 / den;
    count_launch();
    fcg_xr_kernel<<<nb, kT, 0, s>>>(res, r, p, w, alpha, wt, n, h.red.ptr);
    double rn = 0.0;
    if (g.sums(1, 1, &rn)) return -3;
    rnorm = std::sqrt(rn / msh.vol);
    ++iter;
    if (rnorm < tolpss) break;
  }
  if (null_space) {  // ortho on the solution
    count_launch();
    sum_kernel<<<nb, kT, 0, s>>>(res, n, h.red.ptr);
    double sm = 0.0;
    if (g.sums(1, 1, &sm)) return -3;
    count_launch();
    cadd_kernel<<<nb, kT, 0, s>>>(res, -(sm / (double)n), n);
  }
  if (cudaStreamSynchronize(s) != cudaSuccess) {
    set_error(h, std::string("flex cg: ") + cudaGetErrorString(cudaGetLastError()));
    return -3;
  }
  *niter = iter;
  *div0_out = div0;
  *rnorm_out = rnorm;
  if (!(rnorm < tolpss) && div0 != 0.0) {
    set_error(h, "flex cg: iteration cap reached above the tolerance");
    return -5;
  }
  return 0;
}

}  // namespace nekgpu

// ---------------------------------------------------------------------------
// C ABI
namespace nekgpu {
Handle* handle_lookup(const int64_t* h);
int handle_fail(Handle* H, int code, const std::string& msg);
}  // namespace nekgpu

using namespace nekgpu;

extern "C" int nekgpu_hmh_gmres_dev(const int64_t* handle, double* res, const double* h1,
                                    const double* h2, const double* wt, const double* mask,
                                    const double* tol, const int* maxit, const int* kmax,
                                    const int* null_space, int* niter, double* div0,
                                    double* rnorm) {
  Handle* H = handle_lookup(handle);
  if (!H) return handle_fail(nullptr, NEKGPU_EHANDLE, "unknown handle");
  if (handle_enter(*H) != cudaSuccess)
    return handle_fail(H, NEKGPU_ECUDA, "call entry failed");
  if (!H->has_mesh) return handle_fail(H, NEKGPU_ENOSETUP, "mesh not set up (nekgpu_setup)");
  if (!res || !h1 || !h2 || !wt || !mask || !tol || !maxit || !niter || !div0 || !rnorm)
    return handle_fail(H, NEKGPU_EINVAL, "null argument");
  const int m = kmax ? *kmax : 30;
  if (m < 1 || m > NEKGPU_GMRES_MAX)
    return handle_fail(H, NEKGPU_EINVAL, "restart length must be in [1, NEKGPU_GMRES_MAX]");
  if (*maxit < 1) return handle_fail(H, NEKGPU_EINVAL, "maxit must be positive");
  H->err.clear();
  const int rc = gmres_solve(*H, res, h1, h2, wt, mask, *tol, *maxit, m,
                             null_space && *null_space != 0, niter, div0, rnorm);
  handle_leave(*H);  // no kernel of the call runs after it returns
  if (rc == -5) return handle_fail(H, NEKGPU_ENOTCONV, H->err);
  if (rc) return handle_fail(H, rc == -4 ? NEKGPU_ENOMEM : NEKGPU_ECUDA,
                             H->err.empty() ? "gmres failed" : H->err);
  return NEKGPU_OK;
}

extern "C" int nekgpu_hmh_flex_cg_dev(const int64_t* handle, double* res, const double* h1,
                                      const double* h2, const double* wt, const double* mask,
                                      const double* tol, const int* maxit, const int* null_space,
                                      int* niter, double* div0, double* rnorm) {
  Handle* H = handle_lookup(handle);
  if (!H) return handle_fail(nullptr, NEKGPU_EHANDLE, "unknown handle");
  if (handle_enter(*H) != cudaSuccess)
    return handle_fail(H, NEKGPU_ECUDA, "call entry failed");
  if (!H->has_mesh) return handle_fail(H, NEKGPU_ENOSETUP, "mesh not set up (nekgpu_setup)");
  if (!res || !h1 || !h2 || !wt || !mask || !tol || !maxit || !niter || !div0 || !rnorm)
    return handle_fail(H, NEKGPU_EINVAL, "null argument");
  if (*maxit < 1) return handle_fail(H, NEKGPU_EINVAL, "maxit must be positive");
  H->err.clear();
  const int rc = flex_cg_solve(*H, res, h1, h2, wt, mask, *tol, *maxit,
                               null_space && *null_space != 0, niter, div0, rnorm);
  handle_leave(*H);  // no kernel of the call runs after it returns
  if (rc == -5) return handle_fail(H, NEKGPU_ENOTCONV, H->err);
  if (rc) return handle_fail(H, rc == -4 ? NEKGPU_ENOMEM : NEKGPU_ECUDA,
                             H->err.empty() ? "flex cg failed" : H->err);
  return NEKGPU_OK;
}
