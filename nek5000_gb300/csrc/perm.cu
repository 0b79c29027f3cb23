// perm.cu -- the face-ordered element layout of the mixed solve's FP32 inner
// PCG.
//
// In the reference's layout an element's points are stored x fastest
// (core/hmholtz.f works on (lx1,ly1,lz1,nel) arrays), so the points of an
// element face normal to x lie lx1 values apart, and the direct-stiffness sum
// (dssum, core/dssum.f:79) that joins them with the neighbour's copies
// touches one 32-byte sector per value.  The FP32 inner vectors (r, p, x, w,
// the Jacobi diagonal and the weights) are private to the solve, so they are
// stored with each element's points in this order instead:
//
//   the interior points of the six faces (x-, x+, y-, y+, z-, z+), each face
//     in the order of its two free coordinates, the lower axis fastest;
//   the interior points of the twelve edges (along x, y, then z; each from
//     the low to the high end of its free coordinate);
//   the eight vertices; the element's interior points, x fastest.
//
// The two copies of a face point then sit in runs that match point for point
// in the two elements (structured neighbours share the face's orientation),
// the gather-scatter groups are numbered in the new order (gs_setup with the
// position map), and a warp's boundary groups read and write a few whole
// sectors in each element.  The operator keeps G, bm1, h1 and h2 in the
// natural order and maps positions when it stages the vectors (AxArgs::perm).
//
// Measured on GB300 at E=32^3, N=7 (mixed solve, per FP32 iteration): the
// boundary-group kernel drops from 0.071 to 0.061 ms, but the operator rises
// from 0.128 to 0.148 ms (the extra shared-memory pass and barrier, and p
// and w stored at scattered positions inside each element), 0.293 against
// 0.283 ms in all.  The layout stays an option (NEKGPU_OPT_FACE_ORDER), off
// by default.
#include <algorithm>
#include <vector>

#include "impl.cuh"

namespace nekgpu {

// pos_pt[q] = natural point (x fastest) stored at position q of an element.
std::vector<int> face_order(int nx) {
  std::vector<int> o;
  o.reserve((size_t)nx * nx * nx);
  const int a = 1, b = nx - 2, hi = nx - 1;
  auto pt = [&](int i, int j, int k) { return i + nx * (j + nx * k); };
  for (int f = 0; f < 2; ++f)  // x faces
    for (int k = a; k <= b; ++k)
      for (int j = a; j <= b; ++j) o.push_back(pt(f ? hi : 0, j, k));
  for (int f = 0; f < 2; ++f)  // y faces
    for (int k = a; k <= b; ++k)
      for (int i = a; i <= b; ++i) o.push_back(pt(i, f ? hi : 0, k));
  for (int f = 0; f < 2; ++f)  // z faces
    for (int j = a; j <= b; ++j)
      for (int i = a; i <= b; ++i) o.push_back(pt(i, j, f ? hi : 0));
  const int ends[4][2] = {{0, 0}, {1, 0}, {0, 1}, {1, 1}};
  for (auto& e : ends)  // edges along x
    for (int i = a; i <= b; ++i) o.push_back(pt(i, e[0] ? hi : 0, e[1] ? hi : 0));
  for (auto& e : ends)  // edges along y
    for (int j = a; j <= b; ++j) o.push_back(pt(e[0] ? hi : 0, j, e[1] ? hi : 0));
  for (auto& e : ends)  // edges along z
    for (int k = a; k <= b; ++k) o.push_back(pt(e[0] ? hi : 0, e[1] ? hi : 0, k));
  for (int k = 0; k < 2; ++k)  // vertices
    for (int j = 0; j < 2; ++j)
      for (int i = 0; i < 2; ++i) o.push_back(pt(i ? hi : 0, j ? hi : 0, k ? hi : 0));
  for (int k = a; k <= b; ++k)  // interior
    for (int j = a; j <= b; ++j)
      for (int i = a; i <= b; ++i) o.push_back(pt(i, j, k));
  return o;
}

struct PermLayout {
  int nx = 0, nel = 0;
  GsMaps gs;             // gather-scatter maps of the face-ordered layout
  DevBuf<int> pt_pos;    // [P] position of each natural point
  bool ready = false;
  ~PermLayout() { gs_free(gs); }
};

void PermLayoutDeleter::operator()(PermLayout* p) const { delete p; }

namespace {

// o[e P + pt_pos[pt]] = fl32(sc a[e P + pt])
__global__ void perm_cast_kernel(float* __restrict__ o, const double* __restrict__ a, double sc,
                                 const int* __restrict__ pt_pos, int P, int64_t n) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = t / P;
    const int pt = (int)(t - e * P);
    o[e * P + __ldg(pt_pos + pt)] = (float)(a[t] * sc);
  }
}

// x[e P + pt] += sc x32[e P + pt_pos[pt]]
__global__ void perm_axpy_kernel(double* __restrict__ x, const float* __restrict__ e32,
                                 double sc, const int* __restrict__ pt_pos, int P, int64_t n) {
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n;
       t += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = t / P;
    const int pt = (int)(t - e * P);
    x[t] = fma(sc, (double)e32[e * P + __ldg(pt_pos + pt)], x[t]);
  }
}

inline int grid_n(int64_t n) {
  return (int)std::min<int64_t>(std::max<int64_t>((n + 255) / 256, 1), 152 * 8);
}

}  // namespace

bool perm_eligible(const Handle& h) { return h.use_perm && h.has_mesh && h.mesh.nx1 >= 3; }

// Maps of the layout from the natural PCG-form maps (the same groups: every
// copy of group g gets the synthetic id g + 1, element interiors 0), once per
// mesh.
int perm_setup(Handle& h) {
  Mesh& m = h.mesh;
  if (!h.perm) h.perm.reset(new PermLayout());
  PermLayout& L = *h.perm;
  if (L.ready && L.nx == m.nx1 && L.nel == m.nel) return 0;
  L.ready = false;
  const int nx = m.nx1, P = nx * nx * nx;
  const int64_t n = m.n;
  const std::vector<int> pos_pt = face_order(nx);
  std::vector<int> pt_pos((size_t)P);
  for (int q = 0; q < P; ++q) pt_pos[(size_t)pos_pt[(size_t)q]] = q;
  std::vector<int> bst((size_t)m.gs.nbseg + 1), bix((size_t)m.gs.nbidx);
  if (cudaMemcpy(bst.data(), m.gs.bstart, bst.size() * sizeof(int), cudaMemcpyDeviceToHost) !=
          cudaSuccess ||
      (!bix.empty() && cudaMemcpy(bix.data(), m.gs.bidx, bix.size() * sizeof(int),
                                  cudaMemcpyDeviceToHost) != cudaSuccess)) {
    set_error(h, "face-ordered layout: map download failed");
    return -3;
  }
  std::vector<int64_t> gid((size_t)n, 0);
  for (int g = 0; g < m.gs.nbseg; ++g) {
    int k = 0;
    while (k < kGsClasses - 1 && g >= m.gs.cls.soff[k] + m.gs.cls.cnt[k]) ++k;
    const int a = bst[(size_t)g];
    const int b = k < kGsClasses - 1 ? a + (1 << k) : bst[(size_t)g + 1];
    for (int c = a; c < b; ++c) {
      const int li = bix[(size_t)c];
      const int64_t e = li / P;
      gid[(size_t)(e * P + pt_pos[(size_t)(li % P)])] = (int64_t)g + 1;
    }
  }
  std::string err;
  const int rc = gs_setup(L.gs, gid.data(), n, nx, err, pos_pt.data());
  if (rc) {
    set_error(h, "face-ordered layout: " + err);
    return rc == -4 ? -4 : -1;
  }
  // the element-local solver's tuned boundary-group shape carries over
  const GsClasses& t = m.gs.cls_tuned[1];
  if (t.threads > 0) L.gs.cls_tuned[1] = gs_shape(L.gs.cls, t.threads, m.gs_gshift[1]);
  if (L.pt_pos.ensure((size_t)P)) return -4;
  if (cudaMemcpy(L.pt_pos.ptr, pt_pos.data(), P * sizeof(int), cudaMemcpyHostToDevice) !=
      cudaSuccess)
    return -3;
  L.nx = nx;
  L.nel = m.nel;
  L.ready = true;
  return 0;
}

const int* perm_pt_pos(const Handle& h) { return h.perm ? h.perm->pt_pos.ptr : nullptr; }
const GsMaps* perm_maps(const Handle& h) { return h.perm ? &h.perm->gs : nullptr; }

void perm_cast(Handle& h, float* o, const double* a, double scale) {
  const int P = h.mesh.nx1 * h.mesh.nx1 * h.mesh.nx1;
  count_launch();
  perm_cast_kernel<<<grid_n(h.mesh.n), 256, 0, h.stream>>>(o, a, scale, h.perm->pt_pos.ptr, P,
                                                           h.mesh.n);
}

void perm_axpy(Handle& h, double* x, const float* e32, double scale) {
  const int P = h.mesh.nx1 * h.mesh.nx1 * h.mesh.nx1;
  count_launch();
  perm_axpy_kernel<<<grid_n(h.mesh.n), 256, 0, h.stream>>>(x, e32, scale, h.perm->pt_pos.ptr, P,
                                                           h.mesh.n);
}

}  // namespace nekgpu
