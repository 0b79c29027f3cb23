// mixed.cu -- mixed-precision Helmholtz solve: FP32 inner Jacobi-PCG inside an
// FP64 defect-correction loop.
//
//   x = 0, r = f                                       (FP64)
//   repeat:  rbn = sqrt(sum r^2 mult binv / vol)       (FP64, cggo's norm)
//            stop when rbn <= tol (tin < 0: |tin| * rbn of r = f)
//            e = PCG32(A, r / s) to inner_tol (relative; s = power of two
//                near max|r|, so the FP32 iterate stays O(1))
//            x += s * e                                (FP64)
//            r = f - mask * dssum(A x)                 (FP64 operator)
//
// The inner solve stores G, D, the fields and the Jacobi diagonal in FP32 and
// runs the same fused three-kernel iteration as the FP64 solver; its dot
// products are accumulated with compensated FP32 sums per thread and FP64
// across threads and blocks.  The outer residual, the solution and the
// stopping test are FP64, so the result meets the same FP64 tolerance as the
// plain solve.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "impl.cuh"

namespace nekgpu {

namespace {

constexpr int kThreads = 256;
constexpr int kMaxOuter = 30;

inline int blocks(int64_t n) {
  int64_t b = (n + kThreads - 1) / kThreads;
  return (int)std::min<int64_t>(std::max<int64_t>(b, 1), 152 * 8);
}

template <typename TO, typename TI>
__global__ void cast_scale_kernel(TO* __restrict__ o, const TI* __restrict__ a, double sc,
                                  int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    o[i] = (TO)((double)a[i] * sc);
}

__global__ void axpy_kernel(double* __restrict__ x, const float* __restrict__ e, double sc,
                            int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    x[i] = fma(sc, (double)e[i], x[i]);
}

// r = f - mask*w ; partial sums of mult*binv*r^2
__global__ void residual_kernel(double* __restrict__ r, const double* __restrict__ f,
                                const double* __restrict__ w, const double* __restrict__ mask,
                                const double* __restrict__ mult, const double* __restrict__ binv,
                                int64_t n, double* __restrict__ partial) {
  __shared__ double red[32];
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const double ri = f[i] - mask[i] * w[i];
    r[i] = ri;
    acc += mult[i] * binv[i] * ri * ri;
  }
  acc = block_sum(acc, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

__global__ void norm_kernel(const double* __restrict__ r, const double* __restrict__ mult,
                            const double* __restrict__ binv, int64_t n,
                            double* __restrict__ partial) {
  __shared__ double red[32];
  double acc = 0.0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    acc += mult[i] * binv[i] * r[i] * r[i];
  acc = block_sum(acc, red);
  if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

__global__ void scale_kernel(float* __restrict__ a, float f, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    a[i] *= f;
}

// partial[b] = sum (r d) r mult, partial[nb + b] = sum mult binv r r (FP32 data)
__global__ void rz_kernel(const float* __restrict__ r, const float* __restrict__ d,
                          const float* __restrict__ mult, const float* __restrict__ binv,
                          int64_t n, double* __restrict__ partial) {
  __shared__ double red[32];
  CompAcc<float> a1, a2;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float ri = r[i], m = mult[i];
    a1.add(ri * d[i] * ri * m);
    a2.add(m * binv[i] * ri * ri);
  }
  const double b1 = block_sum_comp(a1, red);
  const double b2 = block_sum_comp(a2, red);
  if (threadIdx.x == 0) {
    partial[blockIdx.x] = b1;
    partial[gridDim.x + blockIdx.x] = b2;
  }
}

double host_sum(Handle& h, int nb, int* st) {
  std::vector<double> hp((size_t)nb);
  if (cudaMemcpyAsync(hp.data(), h.red.ptr, nb * sizeof(double), cudaMemcpyDeviceToHost,
                      h.stream) != cudaSuccess ||
      cudaStreamSynchronize(h.stream) != cudaSuccess) {
    *st = -3;
    return 0.0;
  }
  double s = 0.0;
  for (double v : hp) s += v;
  return s;
}

}  // namespace

int ensure_f32(Handle& h) {
  Mesh& m = h.mesh;
  if (m.has_f32) return 0;
  const int64_t n = m.n;
  if (cudaMalloc(&m.f32.G, 6 * n * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&m.f32.bm1, n * sizeof(float)) != cudaSuccess ||
      cudaMalloc(&m.f32.D, m.nx1 * m.nx1 * sizeof(float)) != cudaSuccess) {
    m.f32.release();
    return -4;
  }
  count_launch();
  cast_scale_kernel<float, double><<<blocks(6 * n), kThreads, 0, h.stream>>>(m.f32.G, m.f64.G, 1.0,
                                                                            6 * n);
  count_launch();
  cast_scale_kernel<float, double><<<blocks(n), kThreads, 0, h.stream>>>(m.f32.bm1, m.f64.bm1, 1.0,
                                                                        n);
  count_launch();
  cast_scale_kernel<float, double><<<1, kThreads, 0, h.stream>>>(m.f32.D, m.f64.D, 1.0,
                                                                 m.nx1 * m.nx1);
  if (cudaStreamSynchronize(h.stream) != cudaSuccess) return -3;
  m.has_f32 = true;
  return 0;
}


void cast_to_f32(Handle& h, float* o, const double* a, double scale, int64_t n) {
  count_launch();
  cast_scale_kernel<float, double><<<blocks(n), kThreads, 0, h.stream>>>(o, a, scale, n);
}

void axpy_f32(Handle& h, double* x, const float* e, double scale, int64_t n) {
  count_launch();
  axpy_kernel<<<blocks(n), kThreads, 0, h.stream>>>(x, e, scale, n);
}

double norm64(Handle& h, const double* r, const double* mult, const double* binv) {
  const int64_t n = h.mesh.n;
  const int nb = blocks(n);
  if (h.red.ensure(nb)) return -1.0;
  count_launch();
  norm_kernel<<<nb, kThreads, 0, h.stream>>>(r, mult, binv, n, h.red.ptr);
  int st = 0;
  const double s2 = host_sum(h, nb, &st);
  return st ? -1.0 : std::sqrt(s2 / h.mesh.vol);
}

double outer_residual(Handle& h, double* r, const double* f, const double* x,
                      const Coef<double>& c, const double* mask, const double* mult,
                      const double* binv, double* w) {
  Mesh& m = h.mesh;
  const int64_t n = m.n;
  const int nb = blocks(n);
  if (h.red.ensure(nb)) return -1.0;
  cudaError_t e = launch_axhelm<double, false>(m, m.f64, w, x, c, h.stream);
  if (e != cudaSuccess) {
    set_error(h, std::string("outer residual: axhelm ") + cudaGetErrorString(e));
    return -1.0;
  }
  gs_op<double>(m.gs, w, 0, h.stream);
  count_launch();
  residual_kernel<<<nb, kThreads, 0, h.stream>>>(r, f, w, mask, mult, binv, n, h.red.ptr);
  int st = 0;
  const double s2 = host_sum(h, nb, &st);
  return st ? -1.0 : std::sqrt(s2 / m.vol);
}

// Residual replacement: t.r64 (h.w64.r for mixed_replace) holds r = f - A x
// (FP64).  It becomes the residual of the running FP32 PCG (t's vectors and
// scalars; h.w32 and h.cg for mixed_replace), rescaled by a power of two near
// max |r| (*scale: old in, new out; the ratio of two powers of two is exact,
// so p is rescaled exactly), x32 is zeroed (its old content is already in x),
// and the scalars after the last check (h.cg_host) are updated for the new r:
// r.z, norm and tolerance recomputed, rtz of the previous iterate rescaled,
// beta = (r.z)_new / (r.z)_old.  The direction restarts (beta = 0, p = z,
// counted in *restarts) when the true norm exceeds twice the recurrence norm,
// i.e. FP32 drift dominates and p no longer fits r.  Returns 0, 1 when r is
// zero (nothing to iterate on), or a negative status.
int mixed_replace(Handle& h, double& scale, double inner_tol, int* restarts, const int* perm) {
  PcgWork<float>& wk = h.w32;
  ReplaceTarget t{wk.r.ptr, wk.p.ptr, wk.x.ptr, wk.d.ptr, wk.mult.ptr, wk.binv.ptr,
                  h.w64.r.ptr, h.cg, h.cg_host, perm};
  return mixed_replace_into(h, t, scale, inner_tol, restarts);
}

int mixed_replace_into(Handle& h, const ReplaceTarget& t, double& scale, double inner_tol,
                       int* restarts) {
  const Mesh& m = h.mesh;
  const int64_t n = m.n;
  cudaStream_t s = h.stream;
  const int nb = blocks(n);
  int st = 0;
  const double amax = device_absmax<double>(h, t.r64, n, &st);
  if (st) return -3;
  if (amax == 0.0) return 1;
  const double s_new = std::ldexp(1.0, std::ilogb(amax));
  const double ratio = scale / s_new;
  count_launch(2);
  if (t.perm) perm_cast(h, t.r32, t.r64, 1.0 / s_new);
  else cast_scale_kernel<float, double><<<nb, kThreads, 0, s>>>(t.r32, t.r64, 1.0 / s_new, n);
  scale_kernel<<<nb, kThreads, 0, s>>>(t.p32, (float)ratio, n);
  cudaMemsetAsync(t.x32, 0, n * sizeof(float), s);
  rz_kernel<<<nb, kThreads, 0, s>>>(t.r32, t.d32, t.mult32, t.binv32, n, h.red.ptr);
  std::vector<double> hp(2 * (size_t)nb);
  cudaMemcpyAsync(hp.data(), h.red.ptr, hp.size() * sizeof(double), cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) {
    set_error(h, std::string("mixed: ") + cudaGetErrorString(cudaGetLastError()));
    return -3;
  }
  double s1 = 0.0, s2 = 0.0;
  for (int b = 0; b < nb; ++b) {
    s1 += hp[b];
    s2 += hp[nb + b];
  }
  CgScalars& c = *t.cg_host;  // state after the last (iterated) check
  const double rec = c.rbn2 * ratio;  // FP32 recurrence norm, new scaling
  c.rtz2 = c.rtz2 * ratio * ratio;
  c.rtz1 = s1;
  c.rbn0 = std::sqrt(s2 / m.vol);
  c.beta = (c.rbn0 <= 2.0 * rec) ? s1 / c.rtz2 : 0.0;
  if (c.beta == 0.0 && restarts) ++*restarts;
  c.rbn2 = c.rbn0;
  c.tol = inner_tol * c.rbn0;
  c.done = 0;
  c.counter[0] = c.counter[1] = c.counter[2] = c.counter[3] = 0u;
  cudaMemcpyAsync(t.cg_dev, &c, sizeof(CgScalars), cudaMemcpyHostToDevice, s);
  scale = s_new;
  return 0;
}

// Residual-replacement mode with the FP32 inner PCG in the assembled-boundary
// layout (split.cu): the same outer loop as the element-local form below, on
// the layout's vectors.  h.w64.r holds r = f on entry, h.w64.d the FP64
// Jacobi diagonal, h.w32 the FP32 mask and mult.
MixedResult mixed_split(Handle& h, MixedResult res, double* x, const double* f,
                        const Coef<double>& c64, const Coef<float>& c32, const double* mask,
                        const double* mult, const double* binv, double tol, double rbn,
                        int maxit, double inner_tol, double scale) {
  Mesh& m = h.mesh;
  const int64_t n = m.n;
  cudaStream_t s = h.stream;
  PcgWork<float>& wk = h.w32;
  PcgWork<double>& w64 = h.w64;
  // the element-local solver's checks: one mask value per shared node, mask
  // and mult 1 inside the elements
  if (wk.segmask.ensure(m.gs.nbseg) || wk.segmsum.ensure(m.gs.nbseg)) {
    res.status = -4;
    set_error(h, "mixed: device allocation failed");
    return res;
  }
  cudaMemsetAsync(h.flag, 0, 2 * sizeof(int), s);
  gs_cg_weights<float>(m.gs, wk.mask.ptr, wk.mult.ptr, wk.segmask.ptr, wk.segmsum.ptr, h.flag, s);
  launch_interior_check(h, wk.mask.ptr, wk.mult.ptr, h.flag + 1);
  int flags[2] = {0, 0};
  cudaMemcpyAsync(flags, h.flag, 2 * sizeof(int), cudaMemcpyDeviceToHost, s);
  if (split_load(h, w64.r.ptr, 1.0 / scale, w64.d.ptr, binv, mask)) {
    res.status = -3;
    return res;
  }
  CgScalars& hc = *h.cg_host;
  memset(&hc, 0, sizeof(CgScalars));
  hc.rtz1 = 1.0;
  hc.tin = -inner_tol;
  hc.tol = inner_tol;
  hc.vol = m.vol;
  hc.maxiter = maxit;
  hc.istep = 0;
  if (maxit < 1) {
    hc.done = 1;
    hc.niter = 0;
  }
  cudaMemcpyAsync(h.cg, &hc, sizeof(CgScalars), cudaMemcpyHostToDevice, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) {
    res.status = -3;
    set_error(h, std::string("mixed: ") + cudaGetErrorString(cudaGetLastError()));
    return res;
  }
  if (flags[0] || flags[1]) {
    res.status = -1;
    set_error(h, flags[0] ? "pcg: mask differs between copies of a shared node (apply dsop '*' first)"
                          : "pcg: an element-interior point has mask or multiplicity other than 1");
    return res;
  }
  if (split_first_check(h, c32)) {
    res.status = -3;
    return res;
  }
  for (int upd = 1; upd <= 100000; ++upd) {
    PcgResult pr = split_iterate(h, c32);
    if (pr.status && pr.status != -5) {
      res.status = pr.status;
      return res;
    }
    res.outer = upd;
    res.inner = h.cg_host->niter;
    const bool capped = h.cg_host->iter > h.cg_host->maxiter;
    split_axpy(h, x, scale);
    const double rnew = outer_residual(h, w64.r.ptr, f, x, c64, mask, mult, binv, w64.w.ptr);
    if (!(rnew >= 0.0) || !std::isfinite(rnew)) {
      res.status = -7;
      set_error(h, "mixed: non-finite outer residual");
      return res;
    }
    const bool progress = rnew < rbn;
    rbn = rnew;
    if (rbn <= tol || capped || !progress) break;
    const int rr = split_replace(h, w64.r.ptr, scale, inner_tol, &res.restarts);
    if (rr < 0) {
      res.status = rr;
      return res;
    }
    if (rr == 1) break;
  }
  res.rbn2 = rbn;
  if (!(rbn <= tol)) {
    res.status = -5;
    set_error(h, "mixed: defect correction did not reach the tolerance");
  }
  return res;
}

MixedResult mixed_solve(Handle& h, double* x, const double* f, const double* h1,
                        const double* h2, const double* mask, const double* mult,
                        const double* binv, double tin, int maxit, double inner_tol, int mode) {
  MixedResult res;
  Mesh& m = h.mesh;
  const int64_t n = m.n;
  cudaStream_t s = h.stream;
  const int nb = blocks(n);
  if ((res.status = ensure_f32(h))) {
    set_error(h, "mixed: FP32 operator data allocation failed");
    return res;
  }
  PcgWork<float>& wk = h.w32;
  PcgWork<double>& w64 = h.w64;
  if (wk.mask.ensure(n) || wk.mult.ensure(n) || wk.binv.ensure(n) || wk.x.ensure(n) ||
      wk.f.ensure(n) || wk.d.ensure(n) || wk.h1.ensure(n) || wk.h2.ensure(n) || w64.r.ensure(n) ||
      w64.w.ensure(n) || w64.d.ensure(n) || h.red.ensure(nb)) {
    res.status = -4;
    set_error(h, "mixed: device allocation failed");
    return res;
  }
  Coef<double> c64;
  if (detect_coef<double>(h, h1, h2, n, c64)) {
    res.status = -3;
    set_error(h, "mixed: coefficient scan failed");
    return res;
  }
  if (c64.h2mode == 0) {  // no Dirichlet point and h2 = 0: a null space
    int st0 = 0;
    const double skmin = device_sum(h, 6, mask, nullptr, nullptr, n, &st0);
    if (!st0 && skmin > 0.0) {
      res.status = -1;
      set_error(h, "mixed: singular operator (no Dirichlet point and h2 = 0): use the FP64 "
                   "solve, which applies cggo's null-space correction");
      return res;
    }
  }
  Coef<float> c32;
  c32.h1mode = c64.h1mode;
  c32.h2mode = c64.h2mode;
  c32.h1s = (float)c64.h1s;
  c32.h2s = (float)c64.h2s;
  auto cast = [&](float* o, const double* a, double sc) {
    count_launch();
    cast_scale_kernel<float, double><<<nb, kThreads, 0, s>>>(o, a, sc, n);
  };
  if (c64.h1mode) {
    cast(wk.h1.ptr, h1, 1.0);
    c32.h1 = wk.h1.ptr;
  }
  if (c64.h2mode == 2) {
    cast(wk.h2.ptr, h2, 1.0);
    c32.h2 = wk.h2.ptr;
  }
  cast(wk.mask.ptr, mask, 1.0);
  cast(wk.mult.ptr, mult, 1.0);
  cast(wk.binv.ptr, binv, 1.0);
  // Jacobi diagonal once, in FP64, then FP32
  if (setprec_f64(h, w64.d.ptr, c64)) {
    res.status = -3;
    set_error(h, "mixed: setprec failed");
    return res;
  }
  cast(wk.d.ptr, w64.d.ptr, 1.0);
  // x = 0, r = f
  cudaMemsetAsync(x, 0, n * sizeof(double), s);
  cudaMemcpyAsync(w64.r.ptr, f, n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  int st = 0;
  count_launch();
  norm_kernel<<<nb, kThreads, 0, s>>>(w64.r.ptr, mult, binv, n, h.red.ptr);
  const double rbn0 = std::sqrt(host_sum(h, nb, &st) / m.vol);
  if (st) {
    res.status = st;
    set_error(h, "mixed: reduction failed");
    return res;
  }
  res.rbn0 = res.rbn2 = rbn0;
  if (rbn0 == 0.0) return res;
  if (!std::isfinite(rbn0)) {
    res.status = -7;
    set_error(h, "mixed: non-finite residual norm");
    return res;
  }
  const double tol = tin < 0 ? std::fabs(tin) * rbn0 : std::fabs(tin);
  double rbn = rbn0;
  const bool exact = false;
  if (mode == 1) {
    // One FP32 PCG; whenever its residual has dropped by inner_tol the
    // correction joins x in FP64, r = f - A x is recomputed in FP64 and put
    // back (rescaled) as the FP32 residual, and the search direction p and
    // beta are kept (rescaled), so the Krylov space built so far is not lost.
    int st2 = 0;
    double amax = device_absmax<double>(h, w64.r.ptr, n, &st2);
    if (st2 || amax == 0.0) {
      res.status = st2 ? -3 : 0;
      return res;
    }
    double scale = std::ldexp(1.0, std::ilogb(amax));
    if (h.use_split && split_eligible(h)) {
      const int sst = split_setup(h);
      if (sst) {
        res.status = sst;
        return res;
      }
      return mixed_split(h, res, x, f, c64, c32, mask, mult, binv, tol, rbn, maxit, inner_tol,
                         scale);
    }
    // face-ordered FP32 vectors (perm.cu): the maps, position map and the
    // vectors cast in that order; the guard puts the mesh's maps back
    struct Gs32Reset {
      Handle& h;
      ~Gs32Reset() { h.gs32 = nullptr; }
    } gs32_reset{h};
    const int* perm = nullptr;
    if (perm_eligible(h)) {
      const int pst = perm_setup(h);
      if (pst) {
        res.status = pst;
        return res;
      }
      perm = perm_pt_pos(h);
      h.gs32 = perm_maps(h);
      c32.perm = perm;
      perm_cast(h, wk.mask.ptr, mask, 1.0);
      perm_cast(h, wk.mult.ptr, mult, 1.0);
      perm_cast(h, wk.binv.ptr, binv, 1.0);
      perm_cast(h, wk.d.ptr, w64.d.ptr, 1.0);
      perm_cast(h, wk.f.ptr, w64.r.ptr, 1.0 / scale);
    } else {
      cast(wk.f.ptr, w64.r.ptr, 1.0 / scale);
    }
    bool trivial = false;
    PcgResult pr = pcg_prepare<float>(h, wk, wk.x.ptr, wk.f.ptr, c32, wk.mask.ptr, wk.mult.ptr,
                                      -inner_tol, maxit, 0, wk.d.ptr, &trivial);
    if (pr.status) {
      res.status = pr.status;
      return res;
    }
    if (pcg_first_check<float>(h, wk, wk.x.ptr, wk.mult.ptr, wk.binv.ptr, false)) {
      res.status = -4;
      return res;
    }
    for (int upd = 1; upd <= 100000; ++upd) {
      pr = pcg_iterate<float>(h, m.f32, wk, wk.x.ptr, c32, wk.mult.ptr, wk.binv.ptr, false);
      if (pr.status && pr.status != -5) {
        res.status = pr.status;
        return res;
      }
      res.outer = upd;
      res.inner = h.cg_host->niter;
      const bool capped = h.cg_host->iter > h.cg_host->maxiter;
      if (perm) {
        perm_axpy(h, x, wk.x.ptr, scale);
      } else {
        count_launch();
        axpy_kernel<<<nb, kThreads, 0, s>>>(x, wk.x.ptr, scale, n);
      }
      const double rnew = outer_residual(h, w64.r.ptr, f, x, c64, mask, mult, binv, w64.w.ptr);
      if (!(rnew >= 0.0) || !std::isfinite(rnew)) {
        res.status = -7;
        set_error(h, "mixed: non-finite outer residual");
        return res;
      }
      const bool progress = rnew < rbn;
      rbn = rnew;
      if (rbn <= tol || capped || !progress) break;
      const int rr = mixed_replace(h, scale, inner_tol, &res.restarts, perm);
      if (rr < 0) {
        res.status = rr;
        return res;
      }
      if (rr == 1) break;
    }
    res.rbn2 = rbn;
    if (!(rbn <= tol)) {
      res.status = -5;
      set_error(h, "mixed: defect correction did not reach the tolerance");
    }
    return res;
  }
  for (int outer = 1; outer <= kMaxOuter; ++outer) {
    if (rbn <= tol) break;
    const double amax = device_absmax<double>(h, w64.r.ptr, n, &st);
    if (st || amax == 0.0) break;
    const double scale = std::ldexp(1.0, std::ilogb(amax));  // power of two: exact rescale
    cast(wk.f.ptr, w64.r.ptr, 1.0 / scale);
    PcgResult pr = pcg_solve<float>(h, m.f32, wk, wk.x.ptr, wk.f.ptr, c32, wk.mask.ptr,
                                    wk.mult.ptr, wk.binv.ptr, -inner_tol, maxit, 0, exact,
                                    wk.d.ptr);
    if (pr.status && pr.status != -5) {
      res.status = pr.status;
      return res;
    }
    res.outer = outer;
    res.inner += pr.niter;
    count_launch();
    axpy_kernel<<<nb, kThreads, 0, s>>>(x, wk.x.ptr, scale, n);
    // r = f - mask * dssum(A x) in FP64
    cudaError_t e = launch_axhelm<double, false>(m, m.f64, w64.w.ptr, x, c64, s);
    if (e != cudaSuccess) {
      res.status = -3;
      set_error(h, std::string("mixed: axhelm ") + cudaGetErrorString(e));
      return res;
    }
    gs_op<double>(m.gs, w64.w.ptr, 0, s);
    count_launch();
    residual_kernel<<<nb, kThreads, 0, s>>>(w64.r.ptr, f, w64.w.ptr, mask, mult, binv, n,
                                            h.red.ptr);
    const double rnew = std::sqrt(host_sum(h, nb, &st) / m.vol);
    if (st || !std::isfinite(rnew)) {
      res.status = st ? st : -7;
      set_error(h, "mixed: non-finite outer residual");
      return res;
    }
    if (rnew >= rbn) {  // no progress: FP32 inner solve cannot reduce further
      rbn = rnew;
      break;
    }
    rbn = rnew;
  }
  res.rbn2 = rbn;
  if (!(rbn <= tol)) {
    res.status = -5;
    set_error(h, "mixed: outer defect correction did not reach the tolerance");
  }
  return res;
}

}  // namespace nekgpu
