// gs.cu -- gather-scatter maps and kernels (see gs.cuh).
#include <algorithm>
#include <cstdint>
#include <numeric>

#include "gs_kernels.cuh"

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

template <typename T>
__global__ void gs_cg_weights_kernel(const int* __restrict__ start, const int* __restrict__ idx,
                                     int nseg, const GsClasses cls, const T* __restrict__ mask,
                                     const T* __restrict__ mult, T* __restrict__ segmask,
                                     T* __restrict__ segmsum, int* nonuniform) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nseg) return;
  // A group of the 1-, 2-, 4- or 8-copy classes has exactly that many copies:
  // the idx entries after the last group of a class up to the next 16-byte
  // boundary are padding and belong to no group.
  int k = 0;
  while (k < kGsClasses - 1 && s >= cls.soff[k] + cls.cnt[k]) ++k;
  const int a = start[s];
  const int b = k < kGsClasses - 1 ? a + (1 << k) : start[s + 1];
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

int gs_setup(GsMaps& gs, const int64_t* glo_num, int64_t n, int nx1, std::string& err,
             const int* pos_pt) {
  gs_free(gs);
  if (n < 0 || n >= (int64_t)INT32_MAX) {
    err = "gs_setup: more than 2^31-1 local points";
    return -1;
  }
  gs.n = n;
  // (id, local index) pairs of the numbered points in (id, index) order: a
  // counting sort by id when the ids are dense (set_vert's are), else a sort
  std::vector<std::pair<int64_t, int>> pr;
  {
    int64_t cnt_n = 0, gmin = INT64_MAX, gmax = INT64_MIN;
    for (int64_t i = 0; i < n; ++i)
      if (glo_num[i] != 0) {
        ++cnt_n;
        gmin = std::min(gmin, glo_num[i]);
        gmax = std::max(gmax, glo_num[i]);
      }
    pr.resize((size_t)cnt_n);
    const uint64_t span = cnt_n ? (uint64_t)gmax - (uint64_t)gmin : 0;
    if (cnt_n && span < (uint64_t)(4 * n)) {
      std::vector<int> bucket((size_t)span + 2, 0);
      for (int64_t i = 0; i < n; ++i)
        if (glo_num[i] != 0) ++bucket[(size_t)(glo_num[i] - gmin + 1)];
      for (size_t b = 1; b < bucket.size(); ++b) bucket[b] += bucket[b - 1];
      for (int64_t i = 0; i < n; ++i)  // ascending i: indices ascend within an id
        if (glo_num[i] != 0) pr[(size_t)bucket[(size_t)(glo_num[i] - gmin)]++] = {glo_num[i], (int)i};
    } else {
      size_t q = 0;
      for (int64_t i = 0; i < n; ++i)
        if (glo_num[i] != 0) pr[q++] = {glo_num[i], (int)i};
      std::sort(pr.begin(), pr.end());
    }
  }
  std::vector<int> st, ix, bst, bix;
  st.reserve(pr.size() / 2 + 1);
  ix.reserve(pr.size());
  bst.reserve(pr.size() / 2 + 1);
  bix.reserve(pr.size());
  const int P = nx1 * nx1 * nx1;
  auto interior = [&](int64_t i) {
    const int q = (int)(i % P), p = pos_pt ? pos_pt[q] : q;
    const int x = p % nx1, y = (p / nx1) % nx1, z = p / (nx1 * nx1);
    return x > 0 && x < nx1 - 1 && y > 0 && y < nx1 - 1 && z > 0 && z < nx1 - 1;
  };
  std::vector<unsigned char> skip;
  for (size_t a = 0; a < pr.size();) {
    size_t b = a + 1;
    while (b < pr.size() && pr[b].first == pr[a].first) ++b;
    bst.push_back((int)bix.size());
    for (size_t c = a; c < b; ++c) {
      bix.push_back(pr[c].second);
      if (interior(pr[c].second)) {
        if (skip.empty()) skip.assign((size_t)n, 0);
        skip[(size_t)pr[c].second] = 1;
      }
    }
    if (b - a >= 2) {
      st.push_back((int)ix.size());
      for (size_t c = a; c < b; ++c) ix.push_back(pr[c].second);
    }
    a = b;
  }
  // element-boundary points without an id: singleton groups of the PCG form
  for (int64_t i = 0; i < n; ++i)
    if (glo_num[i] == 0 && !interior(i)) {
      bst.push_back((int)bix.size());
      bix.push_back((int)i);
    }
  st.push_back((int)ix.size());
  bst.push_back((int)bix.size());
  gs.nseg = (int)st.size() - 1;
  gs.nidx = (int)ix.size();
  gs.h_start.assign(st.begin(), st.end());
  gs.h_idx.assign(ix.begin(), ix.end());
  {
    // PCG-form maps: by size class (1, 2, 4, 8, other), then first index;
    // each class's idx run starts on a 4-entry (16-byte) boundary.
    const size_t ns = bst.size() - 1;
    auto cls_of = [&](int g) {
      const int sz = bst[g + 1] - bst[g];
      return sz == 1 ? 0 : sz == 2 ? 1 : sz == 4 ? 2 : sz == 8 ? 3 : 4;
    };
    // groups by class, then by first index (first indices are distinct):
    // one pass over the local points per class
    std::vector<int> group_at((size_t)n, -1);
    for (size_t g = 0; g < ns; ++g) group_at[(size_t)bix[bst[g]]] = (int)g;
    std::vector<int> by_cls[kGsClasses];
    for (int64_t i = 0; i < n; ++i) {
      const int g = group_at[(size_t)i];
      if (g >= 0) by_cls[cls_of(g)].push_back(g);
    }
    std::vector<int> ord;
    ord.reserve(ns);
    for (int k = 0; k < kGsClasses; ++k) ord.insert(ord.end(), by_cls[k].begin(), by_cls[k].end());
    std::vector<int> nst, nix;
    nst.reserve(bst.size());
    nix.reserve(bix.size() + 16);
    GsClasses& C = gs.cls;
    for (int k = 0; k < kGsClasses; ++k) C.cnt[k] = 0;
    int cur = -1;
    for (size_t q = 0; q < ns; ++q) {
      const int g = ord[q];
      const int k = cls_of(g);
      while (cur < k) {  // open the next class region(s)
        ++cur;
        while (nix.size() % 4) nix.push_back(0);
        C.soff[cur] = (int)q;
        C.ioff[cur] = (int)nix.size();
      }
      ++C.cnt[k];
      nst.push_back((int)nix.size());
      for (int c = bst[g]; c < bst[g + 1]; ++c) nix.push_back(bix[c]);
    }
    while (cur < kGsClasses - 1) {
      ++cur;
      while (nix.size() % 4) nix.push_back(0);
      C.soff[cur] = (int)ns;
      C.ioff[cur] = (int)nix.size();
    }
    nst.push_back((int)nix.size());
    C = gs_shape(C, kGsThreads, 0);
    bst.swap(nst);
    bix.swap(nix);
  }
  gs.nbseg = (int)bst.size() - 1;
  gs.nbidx = (int)bix.size();
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
  if (!skip.empty()) {
    if (cudaMalloc(&gs.skip, (size_t)n) != cudaSuccess ||
        cudaMemcpy(gs.skip, skip.data(), (size_t)n, cudaMemcpyHostToDevice) != cudaSuccess) {
      err = "gs_setup: device allocation failed";
      gs_free(gs);
      return -4;
    }
  }
  return 0;
}

void gs_free(GsMaps& gs) {
  cudaFree(gs.start);
  cudaFree(gs.idx);
  cudaFree(gs.bstart);
  cudaFree(gs.bidx);
  cudaFree(gs.skip);
  gs.skip = nullptr;
  gs.start = gs.idx = gs.bstart = gs.bidx = nullptr;
  gs.nseg = gs.nidx = gs.nbseg = gs.nbidx = 0;
  gs.cls = GsClasses{};
  gs.cls_tuned[0] = gs.cls_tuned[1] = GsClasses{};  // tuned shapes belong to the old maps
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

GsClasses gs_shape(const GsClasses& cls, int threads, int gshift) {
  GsClasses C = cls;
  C.threads = threads;
  C.boff[0] = 0;
  for (int k = 0; k < kGsClasses; ++k) {
    C.g[k] = gs_groups_shifted(k, gshift);
    C.boff[k + 1] = C.boff[k] + (C.cnt[k] + threads * C.g[k] - 1) / (threads * C.g[k]);
  }
  return C;
}

template <typename T>
void gs_cg(const GsMaps& gs, T* w, const T* p, const T* segmask, const T* segmsum,
           CgScalars* cg, double* partialA, int nA, double* partialB, cudaStream_t s, bool rho,
           const GsClasses* shape) {
  const GsClasses& C = (shape && shape->threads > 0) ? *shape : gs.cls;
  const int nb = gs_cg_blocks(C);
  // the shape's groups-per-thread shift, recovered from class 0 (4 by default)
  const int g0 = C.g[0];
  auto kern = rho ? (g0 <= 2 ? gs_cg_kernel<T, -1, true>
                             : g0 >= 8 ? gs_cg_kernel<T, 1, true> : gs_cg_kernel<T, 0, true>)
                  : (g0 <= 2 ? gs_cg_kernel<T, -1, false>
                             : g0 >= 8 ? gs_cg_kernel<T, 1, false> : gs_cg_kernel<T, 0, false>);
  count_launch();
  kern<<<nb, C.threads, 0, s>>>(w, p, gs.bstart, gs.bidx, C, segmask, segmsum, cg, partialA, nA,
                                partialB);
}

template <typename T>
void gs_cg_weights(const GsMaps& gs, const T* mask, const T* mult, T* segmask, T* segmsum,
                   int* nonuniform, cudaStream_t s) {
  if (gs.nbseg == 0) return;
  count_launch();
  gs_cg_weights_kernel<T><<<(gs.nbseg + kGsThreads - 1) / kGsThreads, kGsThreads, 0, s>>>(
      gs.bstart, gs.bidx, gs.nbseg, gs.cls, mask, mult, segmask, segmsum, nonuniform);
}

template void gs_op<double>(const GsMaps&, double*, int, cudaStream_t);
template void gs_op<float>(const GsMaps&, float*, int, cudaStream_t);
template void gs_cg<double>(const GsMaps&, double*, const double*, const double*, const double*,
                            CgScalars*, double*, int, double*, cudaStream_t, bool,
                            const GsClasses*);
template void gs_cg<float>(const GsMaps&, float*, const float*, const float*, const float*,
                           CgScalars*, double*, int, double*, cudaStream_t, bool,
                           const GsClasses*);
template void gs_cg_weights<double>(const GsMaps&, const double*, const double*, double*, double*,
                                    int*, cudaStream_t);
template void gs_cg_weights<float>(const GsMaps&, const float*, const float*, float*, float*,
                                   int*, cudaStream_t);

}  // namespace nekgpu
