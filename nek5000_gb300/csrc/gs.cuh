// gs.cuh -- direct-stiffness summation (gslib gs_setup / gs_op semantics).
//
// gs_setup (called from core/dssum.f:20) groups the local copies of every
// non-zero global id; gs_op(+) (core/dssum.f:79) replaces each copy by the
// sum over its group.  Ids of 0 (element interiors, core/navier8.f:2317-2346)
// are never touched.  Here the groups are sorted segments: the (id, local
// index) pairs sorted by id then index give CSR maps
//   start[s] .. start[s+1]-1  ->  idx[]  (ascending local index)
// and one thread owns one segment: gather in ascending index order, reduce,
// scatter back.  Two map sets are kept:
//   shared  -- groups with >= 2 copies (what dssum/dsop changes)
//   bound   -- every non-zero id, singletons included (the PCG form, which
//              also applies the Dirichlet mask and forms the element-boundary
//              part of rho = sum w*p*mult there)
#pragma once
#include <vector>

#include "common.cuh"

namespace nekgpu {

// The PCG-form ("bound") maps are ordered by size class -- groups of 1, 2, 4
// and 8 copies, then all other sizes -- and inside a class by first local
// index.  A class's copies form one packed, 16-byte aligned run of idx, so a
// thread loads its group's indices with one vector access and issues every
// gather at once.
constexpr int kGsClasses = 5;  // sizes 1, 2, 4, 8, other
struct GsClasses {
  int cnt[kGsClasses];      // groups per class
  int soff[kGsClasses];     // first group index of the class
  int ioff[kGsClasses];     // first idx entry of the class (multiple of 4)
  int boff[kGsClasses + 1]; // first block of the class in the launch
  int g[kGsClasses];        // groups per thread of the class (1, 2, 4 or 8)
  int threads;              // threads per block
};

struct GsMaps {
  int64_t n = 0;
  int nseg = 0, nidx = 0;    // shared groups
  int* start = nullptr;      // device, nseg+1
  int* idx = nullptr;        // device, nidx
  int nbseg = 0, nbidx = 0;  // all boundary groups
  int* bstart = nullptr;
  int* bidx = nullptr;
  GsClasses cls{};          // launch shape of the batched solver and the default
  GsClasses cls_tuned[2]{};  // [0] FP64, [1] FP32 single-problem PCG (threads 0: = cls)
  // 1 for element-interior points that the caller's numbering shares (id != 0):
  // the fused operator must leave them to the boundary-group kernel.
  // nullptr when there are none (the reference's numbering).
  unsigned char* skip = nullptr;
  std::vector<int64_t> h_start, h_idx;  // host copy of the shared maps (export)
};

// Host: build maps from glo_num (sort by (id, local index)).  nx1 classifies
// element-interior points: element-boundary points with id 0 join the PCG-form
// maps as singletons (so that masks reach them).  Returns 0 or an error code.
// pos_pt (optional, nx1^3 entries): the natural point (x fastest) held at
// each position of an element when the vectors these maps serve store an
// element's points in another order (the FP32 inner PCG's face-ordered
// layout); nullptr: natural order.
int gs_setup(GsMaps& gs, const int64_t* glo_num, int64_t n, int nx1, std::string& err,
             const int* pos_pt = nullptr);
void gs_free(GsMaps& gs);

// u <- gs_op(u, op): op 0 '+', 1 '*', 2 max, 3 min
template <typename T>
void gs_op(const GsMaps& gs, T* u, int op, cudaStream_t s);

// PCG form: for every boundary group g, s = mask_g * sum w; w <- s on all
// copies; rho partial += s * p_g * msum_g (rho = true).  The last block adds
// these partials to the per-element partials left by the fused axhelm (nA of
// them) and sets rho, alpha = rtz1/rho.  rho = false: the operator's
// partials already hold all of rho (AxArgs::allrho).
template <typename T>
void gs_cg(const GsMaps& gs, T* w, const T* p, const T* segmask, const T* segmsum,
           CgScalars* cg, double* partialA, int nA, double* partialB, cudaStream_t s,
           bool rho = true, const GsClasses* shape = nullptr);

// Per-segment mask value (mask at the first copy) and sum of mult over the
// copies, for the bound maps.  Returns via `nonuniform` (device int) whether
// any group has copies with different mask values.
template <typename T>
void gs_cg_weights(const GsMaps& gs, const T* mask, const T* mult, T* segmask, T* segmsum,
                   int* nonuniform, cudaStream_t s);

constexpr int kGsThreads = 256;     // default block of the PCG-form kernel
constexpr int kGsMaxThreads = 512;  // largest block the autotuner tries
// Default groups per thread in the PCG-form kernel, by class (1, 2, 4, 8
// copies, other): about 8 gathers in flight per thread.
__host__ __device__ constexpr int gs_groups_per_thread(int cls) {
  return cls <= 1 ? 4 : cls == 2 ? 2 : 1;
}
// Launch shape of the PCG-form kernel: `threads` per block and the default
// groups per thread scaled by 2^gshift (clamped to 1..8; the "other" class
// keeps 1), classes block-aligned.  Returns the shape; cls's counts and
// offsets are kept.
GsClasses gs_shape(const GsClasses& cls, int threads, int gshift);
// Blocks of the PCG-form kernel for a shape.
inline int gs_cg_blocks(const GsClasses& c) { return c.boff[kGsClasses] > 0 ? c.boff[kGsClasses] : 1; }
inline int gs_cg_blocks(const GsMaps& gs) { return gs_cg_blocks(gs.cls); }

}  // namespace nekgpu
