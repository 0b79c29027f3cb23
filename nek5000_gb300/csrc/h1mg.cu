// h1mg.cu -- the pressure preconditioner h1mg_solve (core/hsmg.f:1855-1949,
// if_hybrid = .false.) on the device: additive multilevel overlapping
// Schwarz with fast-diagonalisation local solves, a Galerkin coarse solve on
// the vertices, and interpolation back up.  The host plan (h1mg_plan.cpp)
// holds the per-element eigenvectors, weights, masks and numberings; this
// file uploads it and applies z = M r with one block per element for every
// tensor-product step and the library's gather-scatter for every exchange:
//
//   top level  : Schwarz (mask, extend, exchange, FDM, sum back, dssum, W)
//   each level : restrict (1/mult weights, J^T (x) J^T (x) J^T, dssum), Schwarz
//   coarse     : restrict without dssum, gather by vertex, x = X (X^T b) with
//                the sparse factor A_c^-1 = X X^T (xxt.cpp; two row-parallel
//                sparse products), null-space pin and mean, scatter
//   unwind     : e_l += J e_{l-1}; z += J e_top-1; dsavg
//
// All FP64.  Sums are formed in a fixed order (no atomics), so the result
// does not change from run to run.
#include <algorithm>
#include <string>
#include <vector>

#include "h1mg.h"
#include "impl.cuh"

namespace nekgpu {

struct MgDevLevel {
  int nx = 0, nl = 0;
  int64_t n = 0, ne = 0;  // nx^3 nel, nl^3 nel
  GsMaps gs, gse;
  DevBuf<double> mask, rwt, swt, S, dinv, jh;
  DevBuf<double> e, r;  // correction and residual of the levels below the top
};

struct MgDev {
  int lmax = 0, nel = 0;
  bool null_space = false;
  MgDevLevel lev[kMgMaxLev];
  DevBuf<double> A, E, rtop, vmult;
  int64_t nc = 0, ns = 0;
  DevBuf<int> cstart, cidx, cid;
  DevBuf<double> cv, cy;
  // coarse factor A^-1 = X X^T in nested-dissection order (xxt.cpp)
  DevBuf<int> xperm, xcidx, xridx;
  DevBuf<int64_t> xcptr, xrptr;
  DevBuf<double> xcval, xrval, xb, xy;
  // or the AMG hierarchy of the same unknowns (amg.cu), when set up so
  std::unique_ptr<AmgDev, AmgDevDeleter> amg;
  ~MgDev() {
    for (auto& L : lev) {
      gs_free(L.gs);
      gs_free(L.gse);
    }
  }
};

void MgDevDeleter::operator()(MgDev* p) const { delete p; }

namespace {

constexpr int kMgT = 256;

__device__ __forceinline__ int border_count(int i, int j, int k, int nl) {
  return (i == 0 || i == nl - 1) + (j == 0 || j == nl - 1) + (k == 0 || k == nl - 1);
}

// r <- 0 on masked points (h1mg_mask); A <- r extended by one layer: the
// face regions of the border hold the element's own first interior layer
// (hsmg_schwarz_toext3d, then hsmg_extrude(A,0,0,A,2,1)), edges and corners 0.
__global__ void __launch_bounds__(kMgT) mg_toext_kernel(double* __restrict__ A,
                                                        double* __restrict__ r,
                                                        const double* __restrict__ mask, int nx) {
  const int nl = nx + 2;
  const int64_t nxyz = (int64_t)nx * nx * nx, nn = (int64_t)nl * nl * nl;
  const int64_t e = blockIdx.x;
  double* re = r + e * nxyz;
  const double* me = mask + e * nxyz;
  for (int p = threadIdx.x; p < nxyz; p += blockDim.x)
    if (me[p] == 0.0) re[p] = 0.0;
  __syncthreads();
  double* Ae = A + e * nn;
  for (int q = threadIdx.x; q < nn; q += blockDim.x) {
    int i = q % nl, j = (q / nl) % nl, k = q / (nl * nl);
    const int nb = border_count(i, j, k, nl);
    double v = 0.0;
    if (nb <= 1) {
      if (i == 0) i = 2;
      else if (i == nl - 1) i = nl - 3;
      if (j == 0) j = 2;
      else if (j == nl - 1) j = nl - 3;
      if (k == 0) k = 2;
      else if (k == nl - 1) k = nl - 3;
      v = re[(i - 1) + nx * ((j - 1) + nx * (k - 1))];
    }
    Ae[q] = v;
  }
}

// After the exchange (A summed over the extended numbering): the border
// face regions become the neighbours' values (A_b - own first layer); then
// E = S diag(dinv) S^T A on the element (hsmg_do_fast :897-930), and A's
// border face regions keep the element's own E there (the next exchange
// subtracts them).  smem: 2 nl^3 + 3 nl^2 doubles.
__global__ void __launch_bounds__(kMgT) mg_fdm_kernel(double* __restrict__ A,
                                                      double* __restrict__ E,
                                                      const double* __restrict__ S,
                                                      const double* __restrict__ dinv, int nl) {
  extern __shared__ __align__(128) unsigned char mg_smem[];
  double* u = reinterpret_cast<double*>(mg_smem);
  const int nn = nl * nl * nl, nl2 = nl * nl;
  double* v = u + nn;
  double* Ss = v + nn;  // [d][nl*nl], column j = eigenvector j
  const int64_t e = blockIdx.x;
  double* Ae = A + e * (int64_t)nn;
  for (int q = threadIdx.x; q < nn; q += blockDim.x) u[q] = Ae[q];
  for (int q = threadIdx.x; q < 3 * nl2; q += blockDim.x) Ss[q] = S[e * 3 * (int64_t)nl2 + q];
  __syncthreads();
  for (int q = threadIdx.x; q < nn; q += blockDim.x) {
    const int i = q % nl, j = (q / nl) % nl, k = q / nl2;
    if (border_count(i, j, k, nl) != 1) continue;
    int i2 = i, j2 = j, k2 = k;
    if (i == 0) i2 = 2;
    else if (i == nl - 1) i2 = nl - 3;
    else if (j == 0) j2 = 2;
    else if (j == nl - 1) j2 = nl - 3;
    else if (k == 0) k2 = 2;
    else k2 = nl - 3;
    v[q] = u[q] - u[i2 + nl * (j2 + nl * k2)];
  }
  __syncthreads();
  for (int q = threadIdx.x; q < nn; q += blockDim.x) {
    const int i = q % nl, j = (q / nl) % nl, k = q / nl2;
    if (border_count(i, j, k, nl) == 1) u[q] = v[q];
  }
  __syncthreads();
  const double *Sr = Ss, *Sd = Ss + nl2, *St = Ss + 2 * nl2;
  // v = S_r^T along r, u = S_s^T along s, v = S_t^T along t
  for (int q = threadIdx.x; q < nn; q += blockDim.x) {
    const int i = q % nl, jk = q / nl;
    double acc = 0.0;
    for (int l = 0; l < nl; ++l) acc += Sr[l + nl * i] * u[l + nl * jk];
    v[q] = acc;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < nn; q += blockDim.x) {
    const int i = q % nl, j = (q / nl) % nl, k = q / nl2;
    double acc = 0.0;
    for (int l = 0; l < nl; ++l) acc += Sd[l + nl * j] * v[i + nl * (l + nl * k)];
    u[q] = acc;
  }
  __syncthreads();
  const double* de = dinv + e * (int64_t)nn;
  for (int q = threadIdx.x; q < nn; q += blockDim.x) {
    const int ij = q % nl2, k = q / nl2;
    double acc = 0.0;
    for (int l = 0; l < nl; ++l) acc += St[l + nl * k] * u[ij + nl2 * l];
    v[q] = de[q] * acc;
  }
  __syncthreads();
  // back: u = S_r along r, v = S_s along s, u = S_t along t
  for (int q = threadIdx.x; q < nn; q += blockDim.x) {
    const int i = q % nl, jk = q / nl;
    double acc = 0.0;
    for (int l = 0; l < nl; ++l) acc += Sr[i + nl * l] * v[l + nl * jk];
    u[q] = acc;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < nn; q += blockDim.x) {
    const int i = q % nl, j = (q / nl) % nl, k = q / nl2;
    double acc = 0.0;
    for (int l = 0; l < nl; ++l) acc += Sd[j + nl * l] * u[i + nl * (l + nl * k)];
    v[q] = acc;
  }
  __syncthreads();
  double* Ee = E + e * (int64_t)nn;
  for (int q = threadIdx.x; q < nn; q += blockDim.x) {
    const int i = q % nl, j = (q / nl) % nl, k = q / nl2, ij = q % nl2;
    double acc = 0.0;
    for (int l = 0; l < nl; ++l) acc += St[k + nl * l] * v[ij + nl2 * l];
    Ee[q] = acc;
    if (border_count(i, j, k, nl) == 1) Ae[q] = acc;
  }
}

// After the exchange of E: e (regular) = E's interior with the first layer
// next to every face raised by the neighbour's solution there (E_b - own
// E_b), faces r, s, t in turn (hsmg_extrude(E,0,1,A,0,-1) then (E,2,1,E,0,1)).
__global__ void __launch_bounds__(kMgT) mg_toreg_kernel(double* __restrict__ out,
                                                        const double* __restrict__ E,
                                                        const double* __restrict__ A, int nx) {
  const int nl = nx + 2;
  const int64_t nxyz = (int64_t)nx * nx * nx, nn = (int64_t)nl * nl * nl;
  const int64_t e = blockIdx.x;
  const double* Ee = E + e * nn;
  const double* Ae = A + e * nn;
  auto X = [nl](int i, int j, int k) { return i + nl * (j + nl * k); };
  for (int p = threadIdx.x; p < nxyz; p += blockDim.x) {
    const int I = p % nx + 1, J = (p / nx) % nx + 1, K = p / (nx * nx) + 1;
    double v = Ee[X(I, J, K)];
    if (I == 2) v = v + (Ee[X(0, J, K)] - Ae[X(0, J, K)]);
    if (I == nl - 3) v = v + (Ee[X(nl - 1, J, K)] - Ae[X(nl - 1, J, K)]);
    if (J == 2) v = v + (Ee[X(I, 0, K)] - Ae[X(I, 0, K)]);
    if (J == nl - 3) v = v + (Ee[X(I, nl - 1, K)] - Ae[X(I, nl - 1, K)]);
    if (K == 2) v = v + (Ee[X(I, J, 0)] - Ae[X(I, J, 0)]);
    if (K == nl - 3) v = v + (Ee[X(I, J, nl - 1)] - Ae[X(I, J, nl - 1)]);
    out[e * nxyz + p] = v;
  }
}

// e <- 0 on masked points, else e * swt (h1mg_mask, hsmg_schwarz_wt, sigma 1)
__global__ void mg_wt_kernel(double* __restrict__ e, const double* __restrict__ mask,
                             const double* __restrict__ swt, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    e[i] = mask[i] == 0.0 ? 0.0 : e[i] * swt[i];
}

// u (nc^3 per element) = [J^T (x) J^T (x) J^T] (rwt r) (nf^3 per element);
// J nf x nc column-major.  smem: 2 nf^3 + nf nc doubles.
__global__ void __launch_bounds__(kMgT) mg_rstr_kernel(double* __restrict__ u,
                                                       const double* __restrict__ r,
                                                       const double* __restrict__ rwt,
                                                       const double* __restrict__ J, int nf,
                                                       int nc) {
  extern __shared__ __align__(128) unsigned char mg_smem[];
  double* t0 = reinterpret_cast<double*>(mg_smem);
  const int nf3 = nf * nf * nf;
  double* t1 = t0 + nf3;
  double* Js = t1 + nf3;
  const int64_t e = blockIdx.x;
  for (int q = threadIdx.x; q < nf3; q += blockDim.x) t0[q] = r[e * nf3 + q] * rwt[e * nf3 + q];
  for (int q = threadIdx.x; q < nf * nc; q += blockDim.x) Js[q] = J[q];
  __syncthreads();
  for (int q = threadIdx.x; q < nc * nf * nf; q += blockDim.x) {  // r: (nf,nf,nf) -> (nc,nf,nf)
    const int a = q % nc, jk = q / nc;
    double acc = 0.0;
    for (int l = 0; l < nf; ++l) acc += Js[l + nf * a] * t0[l + nf * jk];
    t1[q] = acc;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < nc * nc * nf; q += blockDim.x) {  // s: -> (nc,nc,nf)
    const int a = q % nc, b = (q / nc) % nc, k = q / (nc * nc);
    double acc = 0.0;
    for (int l = 0; l < nf; ++l) acc += Js[l + nf * b] * t1[a + nc * (l + nf * k)];
    t0[q] = acc;
  }
  __syncthreads();
  const int nc3 = nc * nc * nc;
  for (int q = threadIdx.x; q < nc3; q += blockDim.x) {  // t: -> (nc,nc,nc)
    const int ab = q % (nc * nc), c = q / (nc * nc);
    double acc = 0.0;
    for (int l = 0; l < nf; ++l) acc += Js[l + nf * c] * t0[ab + nc * nc * l];
    u[e * nc3 + q] = acc;
  }
}

// ef (nf^3 per element) += [J (x) J (x) J] ec (nc^3 per element)
__global__ void __launch_bounds__(kMgT) mg_intp_add_kernel(double* __restrict__ ef,
                                                           const double* __restrict__ ec,
                                                           const double* __restrict__ J, int nf,
                                                           int nc) {
  extern __shared__ __align__(128) unsigned char mg_smem[];
  double* t0 = reinterpret_cast<double*>(mg_smem);
  const int nf3 = nf * nf * nf, nc3 = nc * nc * nc;
  double* t1 = t0 + nf3;
  double* Js = t1 + nf3;
  const int64_t e = blockIdx.x;
  for (int q = threadIdx.x; q < nc3; q += blockDim.x) t0[q] = ec[e * nc3 + q];
  for (int q = threadIdx.x; q < nf * nc; q += blockDim.x) Js[q] = J[q];
  __syncthreads();
  for (int q = threadIdx.x; q < nf * nc * nc; q += blockDim.x) {  // r: (nc,nc,nc) -> (nf,nc,nc)
    const int a = q % nf, jk = q / nf;
    double acc = 0.0;
    for (int l = 0; l < nc; ++l) acc += Js[a + nf * l] * t0[l + nc * jk];
    t1[q] = acc;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < nf * nf * nc; q += blockDim.x) {  // s: -> (nf,nf,nc)
    const int a = q % nf, b = (q / nf) % nf, k = q / (nf * nf);
    double acc = 0.0;
    for (int l = 0; l < nc; ++l) acc += Js[b + nf * l] * t1[a + nf * (l + nc * k)];
    t0[q] = acc;
  }
  __syncthreads();
  for (int q = threadIdx.x; q < nf3; q += blockDim.x) {  // t: -> (nf,nf,nf), added
    const int ab = q % (nf * nf), c = q / (nf * nf);
    double acc = 0.0;
    for (int l = 0; l < nc; ++l) acc += Js[c + nf * l] * t0[ab + nf * nf * l];
    ef[e * nf3 + q] = ef[e * nf3 + q] + acc;
  }
}

// coarse right-hand side: v[c] = sum of r over the level-0 points of
// unknown c, in ascending point order (crs_solve's vc[p] += b[i])
__global__ void mg_cgather_kernel(double* __restrict__ v, const double* __restrict__ r,
                                  const int* __restrict__ start, const int* __restrict__ idx,
                                  int64_t nc) {
  const int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (c >= nc) return;
  double s = 0.0;
  for (int q = start[c]; q < start[c + 1]; ++q) s += r[idx[q]];
  v[c] = s;
}

// out[r] = sum over the row's entries val * in[idx], r < nrows; one warp per
// row, lanes strided, then a fixed shuffle tree (the same order every run)
__global__ void mg_spmv_kernel(double* __restrict__ out, const int64_t* __restrict__ ptr,
                               const int* __restrict__ idx, const double* __restrict__ val,
                               const double* __restrict__ in, int64_t nrows) {
  const int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (row >= nrows) return;
  double acc = 0.0;
  for (int64_t q = ptr[row] + lane; q < ptr[row + 1]; q += 32) acc += val[q] * in[idx[q]];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
  if (lane == 0) out[row] = acc;
}

// b[k] = v[perm[k]] (into the factor's order), k < n
__global__ void mg_perm_gather_kernel(double* __restrict__ b, const double* __restrict__ v,
                                      const int* __restrict__ perm, int64_t n) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x)
    b[k] = v[perm[k]];
}

// v[perm[k]] = x[k] (back to the unknowns' order), k < n
__global__ void mg_perm_scatter_kernel(double* __restrict__ v, const double* __restrict__ x,
                                       const int* __restrict__ perm, int64_t n) {
  for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
       k += (int64_t)gridDim.x * blockDim.x)
    v[perm[k]] = x[k];
}

// null space: the pinned unknown is 0, then the mean over all unknowns is
// removed (crs_xxt.c:940-957).  One block.
__global__ void __launch_bounds__(1024) mg_cmean_kernel(double* __restrict__ y, int64_t nc) {
  __shared__ double red[32];
  if (threadIdx.x == 0) y[nc - 1] = 0.0;
  __syncthreads();
  const double sw = 1.0 / (double)nc;
  double s = 0.0;
  for (int64_t i = threadIdx.x; i < nc; i += blockDim.x) s += sw * y[i];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    red[0] = t;
  }
  __syncthreads();
  const double mean = red[0];
  for (int64_t i = threadIdx.x; i < nc; i += blockDim.x) y[i] -= mean;
}

__global__ void mg_cscatter_kernel(double* __restrict__ e, const double* __restrict__ y,
                                   const int* __restrict__ cid, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    e[i] = cid[i] >= 0 ? y[cid[i]] : 0.0;
}

__global__ void mg_mul_kernel(double* __restrict__ z, const double* __restrict__ w, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    z[i] = z[i] * w[i];
}

__global__ void mg_fill_kernel(double* __restrict__ z, double v, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    z[i] = v;
}

__global__ void mg_recip_kernel(double* __restrict__ z, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    z[i] = 1.0 / z[i];
}

inline int grid_for(int64_t n) {
  return (int)std::min<int64_t>(std::max<int64_t>((n + kMgT - 1) / kMgT, 1), 152 * 8);
}

size_t fdm_smem(int nl) { return sizeof(double) * (2 * (size_t)nl * nl * nl + 3 * (size_t)nl * nl); }
size_t tnsr_smem(int nf, int nc) { return sizeof(double) * (2 * (size_t)nf * nf * nf + (size_t)nf * nc); }

}  // namespace

namespace {

template <typename T>
int upload(DevBuf<T>& b, const std::vector<T>& h, cudaStream_t s) {
  if (b.ensure(std::max<size_t>(h.size(), 1)) != cudaSuccess) return -4;
  if (!h.empty() &&
      cudaMemcpyAsync(b.ptr, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s) != cudaSuccess)
    return -3;
  return 0;
}

// Schwarz on level l: e = W (sum over extended elements of their local
// solves) r; r is masked in place.
void schwarz(MgDev& m, int l, double* e, double* r, cudaStream_t s) {
  MgDevLevel& L = m.lev[l];
  count_launch(4);
  mg_toext_kernel<<<m.nel, kMgT, 0, s>>>(m.A.ptr, r, L.mask.ptr, L.nx);
  gs_op<double>(L.gse, m.A.ptr, 0, s);
  mg_fdm_kernel<<<m.nel, kMgT, fdm_smem(L.nl), s>>>(m.A.ptr, m.E.ptr, L.S.ptr, L.dinv.ptr, L.nl);
  gs_op<double>(L.gse, m.E.ptr, 0, s);
  mg_toreg_kernel<<<m.nel, kMgT, 0, s>>>(e, m.E.ptr, m.A.ptr, L.nx);
  gs_op<double>(L.gs, e, 0, s);
  mg_wt_kernel<<<grid_for(L.n), kMgT, 0, s>>>(e, L.mask.ptr, L.swt.ptr, L.n);
}

}  // namespace

int h1mg_apply(Handle& h, double* z, double* rhs) {
  if (!h.mg) return -6;
  MgDev& m = *h.mg;
  cudaStream_t s = h.stream;
  const int top = m.lmax - 1;
  MgDevLevel& T = m.lev[top];
  schwarz(m, top, z, rhs, s);
  cudaMemcpyAsync(m.rtop.ptr, rhs, T.n * sizeof(double), cudaMemcpyDeviceToDevice, s);
  double* rc = m.rtop.ptr;
  for (int l = top; l >= 1; --l) {  // restrict to l - 1; Schwarz there unless coarsest
    MgDevLevel &F = m.lev[l], &C = m.lev[l - 1];
    count_launch();
    mg_rstr_kernel<<<m.nel, kMgT, tnsr_smem(F.nx, C.nx), s>>>(C.r.ptr, rc, F.rwt.ptr, F.jh.ptr,
                                                              F.nx, C.nx);
    if (l - 1 >= 1) {
      gs_op<double>(C.gs, C.r.ptr, 0, s);
      schwarz(m, l - 1, C.e.ptr, C.r.ptr, s);
    }
    rc = C.r.ptr;
  }
  MgDevLevel& L0 = m.lev[0];
  count_launch(2);
  if (m.nc > 0) {  // no coarse unknown (every vertex Dirichlet): the coarse correction is 0
    count_launch();
    mg_cgather_kernel<<<(int)((m.nc + 255) / 256), 256, 0, s>>>(m.cv.ptr, L0.r.ptr, m.cstart.ptr,
                                                               m.cidx.ptr, m.nc);
  }
  if (m.ns > 0 && m.amg) {  // cy = one AMG V-cycle on cv (crs_amg_solve)
    amg_apply_dev(*m.amg, m.cy.ptr, m.cv.ptr, s);
  } else if (m.ns > 0) {  // cy = X (X^T cv) on the first ns unknowns
    const int gw = (int)((m.ns * 32 + 255) / 256);
    count_launch(4);
    mg_perm_gather_kernel<<<grid_for(m.ns), kMgT, 0, s>>>(m.xb.ptr, m.cv.ptr, m.xperm.ptr, m.ns);
    mg_spmv_kernel<<<gw, 256, 0, s>>>(m.xy.ptr, m.xcptr.ptr, m.xcidx.ptr, m.xcval.ptr, m.xb.ptr,
                                      m.ns);
    mg_spmv_kernel<<<gw, 256, 0, s>>>(m.xb.ptr, m.xrptr.ptr, m.xridx.ptr, m.xrval.ptr, m.xy.ptr,
                                      m.ns);
    mg_perm_scatter_kernel<<<grid_for(m.ns), kMgT, 0, s>>>(m.cy.ptr, m.xb.ptr, m.xperm.ptr, m.ns);
  }
  if (m.null_space && m.nc > 0) {
    count_launch();
    mg_cmean_kernel<<<1, 1024, 0, s>>>(m.cy.ptr, m.nc);
  }
  mg_cscatter_kernel<<<grid_for(L0.n), kMgT, 0, s>>>(L0.e.ptr, m.cy.ptr, m.cid.ptr, L0.n);
  for (int l = 1; l <= top; ++l) {  // unwind: e_l += J e_{l-1}; the top adds into z
    MgDevLevel &F = m.lev[l], &C = m.lev[l - 1];
    count_launch();
    mg_intp_add_kernel<<<m.nel, kMgT, tnsr_smem(F.nx, C.nx), s>>>(l == top ? z : F.e.ptr,
                                                                  C.e.ptr, F.jh.ptr, F.nx, C.nx);
  }
  gs_op<double>(h.mesh.gs, z, 0, s);  // dsavg
  count_launch();
  mg_mul_kernel<<<grid_for(T.n), kMgT, 0, s>>>(z, m.vmult.ptr, T.n);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error(h, std::string("h1mg: ") + cudaGetErrorString(e));
    return -3;
  }
  return 0;
}

// Build the plan on the host, the coarse Galerkin matrix with the device
// operator (h1 = 1, h2 = 0 as set_up_h1_crs uses), and upload.
int h1mg_setup(Handle& h, const double* x, const double* y, const double* z, const double* mask,
               const int64_t* glo, const int* fbc, bool null_space) {
  Mesh& msh = h.mesh;
  cudaStream_t s = h.stream;
  MgPlan p;
  std::string err;
  int rc = h1mg_plan(p, msh.nx1, msh.nel, glo, x, y, z, mask, fbc, null_space, err);
  if (rc) {
    set_error(h, err);
    return rc;
  }
  const int64_t n = msh.n, nxyz = (int64_t)msh.nx1 * msh.nx1 * msh.nx1;
  // element matrices b_i^T A_e b_j
  std::vector<double> basis;
  h1mg_coarse_basis(msh.nx1, basis);
  DevBuf<double> d1, d2, din, dout;
  if (d1.ensure(n) || d2.ensure(n) || din.ensure(n) || dout.ensure(n)) {
    set_error(h, "h1mg: device allocation failed");
    return NEKGPU_ENOMEM;
  }
  count_launch(2);
  mg_fill_kernel<<<grid_for(n), kMgT, 0, s>>>(d1.ptr, 1.0, n);
  mg_fill_kernel<<<grid_for(n), kMgT, 0, s>>>(d2.ptr, 0.0, n);
  Coef<double> c;
  if (detect_coef<double>(h, d1.ptr, d2.ptr, n, c)) {
    set_error(h, "h1mg: coefficient scan failed");
    return NEKGPU_ECUDA;
  }
  std::vector<double> hin((size_t)n), hout((size_t)n), elem((size_t)64 * msh.nel, 0.0);
  for (int j = 0; j < 8; ++j) {
    for (int e = 0; e < msh.nel; ++e)
      std::copy(basis.begin() + j * nxyz, basis.begin() + (j + 1) * nxyz, hin.begin() + e * nxyz);
    cudaMemcpyAsync(din.ptr, hin.data(), n * sizeof(double), cudaMemcpyHostToDevice, s);
    cudaError_t ce = h.exact ? launch_axhelm<double, true>(msh, msh.f64, dout.ptr, din.ptr, c, s)
                             : launch_axhelm<double, false>(msh, msh.f64, dout.ptr, din.ptr, c, s);
    if (ce == cudaSuccess)
      ce = cudaMemcpyAsync(hout.data(), dout.ptr, n * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(s);
    if (ce != cudaSuccess) {
      set_error(h, std::string("h1mg: coarse operator: ") + cudaGetErrorString(ce));
      return NEKGPU_ECUDA;
    }
    for (int e = 0; e < msh.nel; ++e)
      for (int i = 0; i < 8; ++i) {
        double a = 0.0;  // vlsc2
        const double* bi = basis.data() + i * nxyz;
        const double* we = hout.data() + e * nxyz;
        for (int64_t q = 0; q < nxyz; ++q) a = a + bi[q] * we[q];
        elem[64 * (size_t)e + i + 8 * j] = a;
      }
  }
  p.use_amg = h.coarse_amg;
  rc = h1mg_plan_coarse(p, elem.data(), err);
  if (rc) {
    set_error(h, err);
    return rc;
  }
  // upload
  std::unique_ptr<MgDev, MgDevDeleter> m(new MgDev());
  m->lmax = p.lmax;
  m->nel = p.nel;
  m->null_space = null_space;
  int64_t nemax = 0;
  for (int l = 0; l < p.lmax; ++l) {
    const MgLevelPlan& P = p.lev[l];
    MgDevLevel& L = m->lev[l];
    L.nx = P.nx;
    L.nl = P.nx + 2;
    L.n = P.n;
    L.ne = (int64_t)L.nl * L.nl * L.nl * p.nel;
    nemax = std::max(nemax, L.ne);
    if (gs_setup(L.gs, P.glo.data(), P.n, P.nx, err) ||
        (l > 0 && gs_setup(L.gse, P.glo_ext.data(), L.ne, L.nl, err))) {
      set_error(h, "h1mg: " + err);
      return NEKGPU_ENOMEM;
    }
    int u = upload(L.mask, P.mask, s);
    if (!u) u = upload(L.rwt, P.rwt, s);
    if (!u && l > 0) u = upload(L.swt, P.swt, s);
    if (!u && l > 0) u = upload(L.S, P.S, s);
    if (!u && l > 0) u = upload(L.dinv, P.dinv, s);
    if (!u && l > 0) u = upload(L.jh, P.jh, s);
    if (!u && l < p.lmax - 1 && (L.e.ensure(P.n) || L.r.ensure(P.n))) u = -4;
    if (u) {
      set_error(h, "h1mg: device upload failed");
      return u == -4 ? NEKGPU_ENOMEM : NEKGPU_ECUDA;
    }
  }
  m->nc = p.nc;
  m->ns = p.nsolve;
  {
    const int64_t n0 = p.lev[0].n;
    std::vector<int> start((size_t)p.nc + 1, 0), idx, cid(n0);
    for (int64_t i = 0; i < n0; ++i) {
      cid[i] = (int)p.cid[i];
      if (p.cid[i] >= 0) ++start[p.cid[i] + 1];
    }
    for (int64_t c2 = 0; c2 < p.nc; ++c2) start[c2 + 1] += start[c2];
    idx.resize(start[p.nc]);
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int64_t i = 0; i < n0; ++i)
      if (p.cid[i] >= 0) idx[fill[p.cid[i]]++] = (int)i;
    const XxtFactor& X = p.xxt;
    if (upload(m->cstart, start, s) || upload(m->cidx, idx, s) || upload(m->cid, cid, s) ||
        upload(m->xperm, X.perm, s) || upload(m->xcptr, X.cptr, s) ||
        upload(m->xcidx, X.cidx, s) || upload(m->xcval, X.cval, s) ||
        upload(m->xrptr, X.rptr, s) || upload(m->xridx, X.ridx, s) ||
        upload(m->xrval, X.rval, s) || m->xb.ensure(std::max<int64_t>(p.nsolve, 1)) ||
        m->xy.ensure(std::max<int64_t>(p.nsolve, 1)) ||
        m->cv.ensure(std::max<int64_t>(p.nc, 1)) || m->cy.ensure(std::max<int64_t>(p.nc, 1))) {
      set_error(h, "h1mg: device upload failed");
      return NEKGPU_ENOMEM;
    }
  }
  if (p.use_amg && p.nsolve > 0 && amg_upload(p.amg, m->amg, s)) {
    set_error(h, "h1mg: AMG upload failed");
    return NEKGPU_ENOMEM;
  }
  if (m->A.ensure(nemax) || m->E.ensure(nemax) || m->rtop.ensure(n) || m->vmult.ensure(n)) {
    set_error(h, "h1mg: device allocation failed");
    return NEKGPU_ENOMEM;
  }
  count_launch(2);
  mg_fill_kernel<<<grid_for(n), kMgT, 0, s>>>(m->vmult.ptr, 1.0, n);
  gs_op<double>(msh.gs, m->vmult.ptr, 0, s);
  mg_recip_kernel<<<grid_for(n), kMgT, 0, s>>>(m->vmult.ptr, n);
  // the largest extended element any handle can have (lx1 = 12)
  cudaFuncSetAttribute(mg_fdm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)fdm_smem(14));
  const cudaError_t ce = cudaStreamSynchronize(s);
  if (ce != cudaSuccess) {
    set_error(h, std::string("h1mg: setup: ") + cudaGetErrorString(ce));
    return NEKGPU_ECUDA;
  }
  h.mg = std::move(m);
  return NEKGPU_OK;
}

}  // namespace nekgpu

// ---------------------------------------------------------------------------
// C ABI
namespace nekgpu {
Handle* handle_lookup(const int64_t* h);
int handle_fail(Handle* H, int code, const std::string& msg);
}  // namespace nekgpu

using namespace nekgpu;

extern "C" int nekgpu_h1mg_setup(const int64_t* handle, const double* x, const double* y,
                                 const double* z, const double* mask, const int64_t* glo_num,
                                 const int* fbc, const int* null_space) {
  Handle* H = handle_lookup(handle);
  if (!H) return handle_fail(nullptr, NEKGPU_EHANDLE, "unknown handle");
  if (handle_enter(*H) != cudaSuccess)
    return handle_fail(H, NEKGPU_ECUDA, "call entry failed");
  if (!H->has_mesh) return handle_fail(H, NEKGPU_ENOSETUP, "mesh not set up (nekgpu_setup)");
  if (!x || !y || !z || !glo_num || (!mask && !fbc))
    return handle_fail(H, NEKGPU_EINVAL, "null argument");
  H->err.clear();
  H->mg.reset();
  const int rc = h1mg_setup(*H, x, y, z, mask, glo_num, fbc, null_space && *null_space != 0);
  handle_leave(*H);  // no kernel of the call runs after it returns
  if (rc) return handle_fail(H, rc, H->err.empty() ? "h1mg setup failed" : H->err);
  return NEKGPU_OK;
}

extern "C" int nekgpu_h1mg_free(const int64_t* handle) {
  Handle* H = handle_lookup(handle);
  if (!H) return handle_fail(nullptr, NEKGPU_EHANDLE, "unknown handle");
  if (handle_enter(*H) != cudaSuccess)
    return handle_fail(H, NEKGPU_ECUDA, "call entry failed");
  cudaStreamSynchronize(H->stream);
  H->mg.reset();
  return NEKGPU_OK;
}

extern "C" int nekgpu_h1mg_apply_dev(const int64_t* handle, double* z, double* rhs) {
  Handle* H = handle_lookup(handle);
  if (!H) return handle_fail(nullptr, NEKGPU_EHANDLE, "unknown handle");
  if (handle_enter(*H) != cudaSuccess)
    return handle_fail(H, NEKGPU_ECUDA, "call entry failed");
  if (!H->mg) return handle_fail(H, NEKGPU_ENOSETUP, "h1mg not set up (nekgpu_h1mg_setup)");
  if (!z || !rhs) return handle_fail(H, NEKGPU_EINVAL, "null argument");
  H->err.clear();
  int rc = h1mg_apply(*H, z, rhs);
  if (!rc && cudaStreamSynchronize(H->stream) != cudaSuccess) rc = -3;
  if (rc) return handle_fail(H, NEKGPU_ECUDA, H->err.empty() ? "h1mg apply failed" : H->err);
  return NEKGPU_OK;
}
