// gs.cu -- gather-scatter maps and kernels (see gs.cuh).
#include <algorithm>
#include <numeric>

#include "gs.cuh"

namespace nekgpu {

namespace {

template <typename T>
__global__ void gs_op_kernel(T* __restrict__ u, const int* __restrict__ start,
                             const int* __restrict__ idx, int nseg, int op) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  const int a = start[s], b = start[s + 1];
  T t = u[idx[a]];
  for (int c = a + 1; c < b; ++c) {
    const T v = u[idx[c]];
    if (op == 0) t = t + v;
    else if (op == 1) t = t * v;
    else if (op == 2) t = (v > t) ? v : t;
    else t = (v < t) ? v : t;
  }
  for (int c = a; c < b; ++c) u[idx[c]] = t;
}

// Grid-stride over boundary groups with a fixed, small grid; every block also
// folds a strided slice of the operator's interior partials into its own
// partial, so the last block sums only gridDim.x values.
template <typename T>
__global__ void __launch_bounds__(kGsThreads)
    gs_cg_kernel(T* __restrict__ w, const T* __restrict__ p, const int* __restrict__ start,
                 const int* __restrict__ idx, int nseg, const T* __restrict__ segmask,
                 const T* __restrict__ segmsum, CgScalars* cg,
                 const double* __restrict__ partialA, int nA, double* __restrict__ partialB) {
  __shared__ double red[32];
  __shared__ int am_last;
  if (cg->done) return;
  CompAcc<T> acc;
  const int stride = gridDim.x * blockDim.x;
  for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nseg; s += stride) {
    const int a = start[s], b = start[s + 1];
    T t = w[idx[a]];
    for (int c = a + 1; c < b; ++c) t = t + w[idx[c]];
    t = t * segmask[s];
    for (int c = a; c < b; ++c) w[idx[c]] = t;
    acc.add(t * p[idx[a]] * segmsum[s]);
  }
  double dot = block_sum_comp(acc, red);  // thread 0
  // this block's share of the interior partials: q = blockIdx.x + k*gridDim.x
  double pa = 0.0;
  for (int q = blockIdx.x + gridDim.x * threadIdx.x; q < nA; q += gridDim.x * blockDim.x)
    pa += __ldcg(partialA + q);
  pa = block_sum(pa, red);
  if (threadIdx.x == 0) {
    partialB[blockIdx.x] = dot + pa;
    __threadfence();
    const unsigned int ticket = atomicAdd(&cg->counter[0], 1u);
    am_last = (ticket == gridDim.x - 1);
  }
  __syncthreads();
  if (!am_last) return;
  double pb = 0.0;
  for (int q = threadIdx.x; q < (int)gridDim.x; q += blockDim.x) pb += __ldcg(partialB + q);
  const double rho = block_sum(pb, red);
  if (threadIdx.x == 0) {
    cg->rho = rho;
    cg->alpha = cg->rtz1 / rho;
    cg->counter[0] = 0u;
  }
}

template <typename T>
__global__ void gs_cg_weights_kernel(const int* __restrict__ start, const int* __restrict__ idx,
                                     int nseg, const T* __restrict__ mask,
                                     const T* __restrict__ mult, T* __restrict__ segmask,
                                     T* __restrict__ segmsum, int* nonuniform) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  const int a = start[s], b = start[s + 1];
  const T m0 = mask[idx[a]];
  double ms = 0.0;
  for (int c = a; c < b; ++c) {
    if (mask[idx[c]] != m0) atomicOr(nonuniform, 1);
    ms += (double)mult[idx[c]];
  }
  segmask[s] = m0;
  segmsum[s] = (T)ms;
}

}  // namespace

int gs_setup(GsMaps& gs, const int64_t* glo_num, int64_t n, std::string& err) {
  gs_free(gs);
  if (n >= (int64_t)INT32_MAX) {
    err = "gs_setup: more than 2^31-1 local points";
    return -1;
  }
  gs.n = n;
  std::vector<std::pair<int64_t, int>> pr;
  pr.reserve((size_t)(n / 2));
  for (int64_t i = 0; i < n; ++i)
    if (glo_num[i] != 0) pr.emplace_back(glo_num[i], (int)i);
  std::sort(pr.begin(), pr.end());
  std::vector<int> st, ix, bst, bix;
  st.reserve(pr.size() / 2 + 1);
  ix.reserve(pr.size());
  bst.reserve(pr.size() / 2 + 1);
  bix.reserve(pr.size());
  for (size_t a = 0; a < pr.size();) {
    size_t b = a + 1;
    while (b < pr.size() && pr[b].first == pr[a].first) ++b;
    bst.push_back((int)bix.size());
    for (size_t c = a; c < b; ++c) bix.push_back(pr[c].second);
    if (b - a >= 2) {
      st.push_back((int)ix.size());
      for (size_t c = a; c < b; ++c) ix.push_back(pr[c].second);
    }
    a = b;
  }
  st.push_back((int)ix.size());
  bst.push_back((int)bix.size());
  gs.nseg = (int)st.size() - 1;
  gs.nidx = (int)ix.size();
  gs.nbseg = (int)bst.size() - 1;
  gs.nbidx = (int)bix.size();
  gs.h_start.assign(st.begin(), st.end());
  gs.h_idx.assign(ix.begin(), ix.end());
  // The PCG-form maps are processed in order of each group's first local
  // index: neighbouring threads then gather and scatter within the same few
  // elements (the order of groups does not change any group's sum).
  {
    const size_t ns = bst.size() - 1;
    std::vector<int> ord(ns);
    std::iota(ord.begin(), ord.end(), 0);
    std::stable_sort(ord.begin(), ord.end(),
                     [&](int a, int b) { return bix[bst[a]] < bix[bst[b]]; });
    std::vector<int> nst, nix;
    nst.reserve(bst.size());
    nix.reserve(bix.size());
    for (int g : ord) {
      nst.push_back((int)nix.size());
      for (int c = bst[g]; c < bst[g + 1]; ++c) nix.push_back(bix[c]);
    }
    nst.push_back((int)nix.size());
    bst.swap(nst);
    bix.swap(nix);
  }
  auto up = [&](int** dst, const std::vector<int>& v) -> bool {
    size_t bytes = std::max<size_t>(v.size(), 1) * sizeof(int);
    if (cudaMalloc(dst, bytes) != cudaSuccess) return false;
    if (!v.empty() && cudaMemcpy(*dst, v.data(), v.size() * sizeof(int), cudaMemcpyHostToDevice) !=
                          cudaSuccess)
      return false;
    return true;
  };
  if (!up(&gs.start, st) || !up(&gs.idx, ix) || !up(&gs.bstart, bst) || !up(&gs.bidx, bix)) {
    err = "gs_setup: device allocation failed";
    gs_free(gs);
    return -4;
  }
  return 0;
}

void gs_free(GsMaps& gs) {
  cudaFree(gs.start);
  cudaFree(gs.idx);
  cudaFree(gs.bstart);
  cudaFree(gs.bidx);
  gs.start = gs.idx = gs.bstart = gs.bidx = nullptr;
  gs.nseg = gs.nidx = gs.nbseg = gs.nbidx = 0;
  gs.h_start.clear();
  gs.h_idx.clear();
}

template <typename T>
void gs_op(const GsMaps& gs, T* u, int op, cudaStream_t s) {
  if (gs.nseg == 0) return;
  count_launch();
  gs_op_kernel<T><<<(gs.nseg + kGsThreads - 1) / kGsThreads, kGsThreads, 0, s>>>(
      u, gs.start, gs.idx, gs.nseg, op);
}

template <typename T>
void gs_cg(const GsMaps& gs, T* w, const T* p, const T* segmask, const T* segmsum,
           CgScalars* cg, double* partialA, int nA, double* partialB, cudaStream_t s) {
  const int nb = gs_cg_blocks(gs);
  count_launch();
  gs_cg_kernel<T><<<nb, kGsThreads, 0, s>>>(w, p, gs.bstart, gs.bidx, gs.nbseg, segmask, segmsum,
                                            cg, partialA, nA, partialB);
}

template <typename T>
void gs_cg_weights(const GsMaps& gs, const T* mask, const T* mult, T* segmask, T* segmsum,
                   int* nonuniform, cudaStream_t s) {
  if (gs.nbseg == 0) return;
  count_launch();
  gs_cg_weights_kernel<T><<<(gs.nbseg + kGsThreads - 1) / kGsThreads, kGsThreads, 0, s>>>(
      gs.bstart, gs.bidx, gs.nbseg, mask, mult, segmask, segmsum, nonuniform);
}

template void gs_op<double>(const GsMaps&, double*, int, cudaStream_t);
template void gs_op<float>(const GsMaps&, float*, int, cudaStream_t);
template void gs_cg<double>(const GsMaps&, double*, const double*, const double*, const double*,
                            CgScalars*, double*, int, double*, cudaStream_t);
template void gs_cg<float>(const GsMaps&, float*, const float*, const float*, const float*,
                           CgScalars*, double*, int, double*, cudaStream_t);
template void gs_cg_weights<double>(const GsMaps&, const double*, const double*, double*, double*,
                                    int*, cudaStream_t);
template void gs_cg_weights<float>(const GsMaps&, const float*, const float*, float*, float*,
                                   int*, cudaStream_t);

}  // namespace nekgpu
