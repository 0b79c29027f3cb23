// capi.cu -- the extern "C" entry points declared in include/nekgpu.h.
//
// Handles are small integers mapped to Handle objects; every call validates
// its handle and arguments, records a message on failure and returns a
// negative status.  Nothing here exits or traps.
#include <cmath>
#include <cstring>
#include <map>
#include <mutex>

#include "impl.cuh"
#include "nekgpu.h"

using namespace nekgpu;

namespace {

std::mutex g_mu;
std::map<int64_t, std::unique_ptr<Handle>> g_handles;
int64_t g_next = 1;
thread_local std::string g_orphan_err;

Handle* get(const int64_t* h) {
  if (!h) return nullptr;
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_handles.find(*h);
  return it == g_handles.end() ? nullptr : it->second.get();
}

int fail(Handle* H, int code, const std::string& msg) {
  if (H) H->err = msg;
  else g_orphan_err = msg;
  return code;
}

int cuda_fail(Handle* H, cudaError_t e, const char* where) {
  return fail(H, NEKGPU_ECUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// Every call on a handle: look it up, wait for the caller's queued work
// (handle_enter), and wait for the handle's stream when the call returns, on
// every return path, so that no kernel of the call is still running then.
// The paths that read results back already synchronize and report errors;
// the guard only makes the completion promise hold on all of them.
struct LeaveGuard {
  Handle* h;
  ~LeaveGuard() {
    if (h && h->stream) cudaStreamSynchronize(h->stream);
  }
};

#define GET_HANDLE(hp)                                                   \
  Handle* H = get(hp);                                                   \
  if (!H) return fail(nullptr, NEKGPU_EHANDLE, "unknown handle");        \
  if (cudaError_t e_ = handle_enter(*H))                                 \
    return cuda_fail(H, e_, "call entry");                               \
  LeaveGuard leave_guard_{H};

#define NEED_MESH()                                                      \
  if (!H->has_mesh) return fail(H, NEKGPU_ENOSETUP, "mesh not set up (nekgpu_setup)");

__global__ void pack_g_kernel(double* __restrict__ G, const double* __restrict__ gm, int m, int P,
                              int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t e = i / P;
    const int p = (int)(i % P);
    G[(e * 6 + m) * P + p] = gm[i];
  }
}

__global__ void mul_kernel(double* __restrict__ a, const double* __restrict__ b, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    a[i] = a[i] * b[i];
}

__global__ void fill_kernel(double* __restrict__ a, double v, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x)
    a[i] = v;
}

inline int nblk(int64_t n) {
  int64_t b = (n + 255) / 256;
  return (int)std::min<int64_t>(std::max<int64_t>(b, 1), 152 * 16);
}

// Device-side coefficient descriptor for host or device h1/h2.
int make_coef(Handle* H, const double* h1, const double* h2, Coef<double>& c) {
  if (!h1 || !h2) return fail(H, NEKGPU_EINVAL, "h1/h2 must not be null");
  int st = detect_coef<double>(*H, h1, h2, H->mesh.n, c);
  if (st) return fail(H, NEKGPU_ECUDA, "coefficient scan failed");
  return 0;
}

int axhelm_dev(Handle* H, double* au, const double* u, const Coef<double>& c) {
  cudaError_t e = H->exact ? launch_axhelm<double, true>(H->mesh, H->mesh.f64, au, u, c, H->stream)
                           : launch_axhelm<double, false>(H->mesh, H->mesh.f64, au, u, c, H->stream);
  if (e != cudaSuccess) return cuda_fail(H, e, "axhelm launch");
  e = cudaStreamSynchronize(H->stream);
  if (e != cudaSuccess) return cuda_fail(H, e, "axhelm");
  return 0;
}

int h2d(Handle* H, DevBuf<double>& b, const double* src, int64_t n) {
  if (b.ensure(n) != cudaSuccess) return fail(H, NEKGPU_ENOMEM, "staging allocation failed");
  cudaError_t e = cudaMemcpyAsync(b.ptr, src, n * sizeof(double), cudaMemcpyHostToDevice, H->stream);
  if (e != cudaSuccess) return cuda_fail(H, e, "host to device copy");
  return 0;
}

int d2h(Handle* H, double* dst, const double* src, int64_t n) {
  cudaError_t e = cudaMemcpyAsync(dst, src, n * sizeof(double), cudaMemcpyDeviceToHost, H->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
  if (e != cudaSuccess) return cuda_fail(H, e, "device to host copy");
  return 0;
}

// chktcg1 (core/hmholtz.f:527-609) on device arrays; EIGAA = 0 -> ACONDNO = 10
int chktcg1_dev(Handle* H, double* tol, const double* res, const Coef<double>& c,
                const double* mask, const double* mult, const double* binv) {
  const int64_t n = H->mesh.n;
  const double eps = 1.0e-13, acondno = 10.0, vol = H->mesh.vol;
  int st = 0;
  const double r2 = device_sum(*H, 4, binv, res, mult, n, &st);
  if (st) return fail(H, st, "chktcg1: reduction failed");
  const double rinit = std::sqrt(r2 / vol);
  const double rmin = eps * rinit;
  if (*tol < rmin) *tol = rmin;
  const double bcneu1 = device_sum(*H, 5, mask, mult, nullptr, n, &st);
  const double bcneu2 = device_sum(*H, 0, mult, nullptr, nullptr, n, &st);
  const double bctest = std::fabs(bcneu1 - bcneu2);
  DevBuf<double>& w1 = H->io5;
  DevBuf<double>& w2 = H->io6;
  if (w1.ensure(n) || w2.ensure(n)) return fail(H, NEKGPU_ENOMEM, "chktcg1: allocation failed");
  count_launch();
  fill_kernel<<<nblk(n), 256, 0, H->stream>>>(w1.ptr, 1.0, n);
  int rc = axhelm_dev(H, w2.ptr, w1.ptr, c);
  if (rc) return rc;
  const double s = device_sum(*H, 2, w2.ptr, H->mesh.f64.bm1, nullptr, n, &st);
  if (st) return fail(H, st, "chktcg1: reduction failed");
  const double bcrob = std::sqrt(s / vol);
  if (bctest < 0.1 && bcrob < eps * acondno) {
    const double tolmin = rinit * eps * 10.0;
    if (*tol < tolmin) *tol = tolmin;
  }
  return 0;
}

// cggo on device arrays.  Returns status; outputs niter/rbn0/rbn2.
int cggo_dev(Handle* H, double* x, const double* f, const double* h1, const double* h2,
             const double* mask, const double* mult, double tin, int maxit, int maxcg,
             const double* binv, int* niter, double* rbn0, double* rbn2) {
  H->err.clear();
  Coef<double> c;
  int rc = make_coef(H, h1, h2, c);
  if (rc) return rc;
  if (cuda_pending(*H, "cggo: coefficient scan")) return NEKGPU_ECUDA;
  // a non-trivial null space (no Dirichlet point, h2 == 0) gets cggo's mean
  // correction (hmholtz.f:705-750) inside the FP64 solve
  const int maxiter = std::min(maxit, maxcg);
  PcgResult r = pcg_solve<double>(*H, H->mesh.f64, H->w64, x, f, c, mask, mult, binv, tin,
                                  maxiter, H->istep, H->exact);
  if (niter) *niter = r.niter;
  if (rbn0) *rbn0 = r.rbn0;
  if (rbn2) *rbn2 = r.rbn2;
  if (r.status == -5) return NEKGPU_ENOTCONV;
  if (r.status == -7) return NEKGPU_ENAN;
  if (r.status) return fail(H, r.status, H->err.empty() ? "pcg failed" : H->err);
  return 0;
}

int hmholtz_dev(Handle* H, double* u, double* rhs, const double* h1, const double* h2,
                const double* mask, const double* mult, double tli, int maxit, int maxcg,
                const double* binv, int* niter, double* rbn0, double* rbn2) {
  const int64_t n = H->mesh.n;
  double tol = std::fabs(tli);
  gs_op<double>(H->mesh.gs, rhs, 0, H->stream);                       // dssum(rhs)
  count_launch();
  mul_kernel<<<nblk(n), 256, 0, H->stream>>>(rhs, mask, n);           // col2(rhs,mask)
  Coef<double> c;
  int rc = make_coef(H, h1, h2, c);
  if (rc) return rc;
  rc = chktcg1_dev(H, &tol, rhs, c, mask, mult, binv);
  if (rc) return rc;
  if (tli < 0) tol = tli;
  return cggo_dev(H, u, rhs, h1, h2, mask, mult, tol, maxit, maxcg, binv, niter, rbn0, rbn2);
}

int check_n(Handle* H, const void* p) {
  if (!p) return fail(H, NEKGPU_EINVAL, "null array argument");
  return 0;
}

}  // namespace

namespace nekgpu {

int handle_open(Handle& H, int device, cudaStream_t shared, std::string& err) {
  cudaError_t e;
  H.device = device;
  if ((e = cudaSetDevice(device)) != cudaSuccess) {
    err = std::string("cudaSetDevice: ") + cudaGetErrorString(e);
    return -3;
  }
  if (shared) {
    H.stream = shared;
    H.own_stream = false;
  } else if ((e = cudaStreamCreateWithFlags(&H.stream, cudaStreamNonBlocking)) != cudaSuccess) {
    err = std::string("stream: ") + cudaGetErrorString(e);
    return -3;
  }
  if (cudaMalloc(&H.cg, sizeof(CgScalars)) != cudaSuccess ||
      cudaMallocHost(&H.cg_host, sizeof(CgScalars)) != cudaSuccess ||
      cudaMalloc(&H.flag, sizeof(int) * 4) != cudaSuccess) {
    err = "handle allocation failed";
    return -4;
  }
  cudaMemset(H.cg, 0, sizeof(CgScalars));
  cudaEventCreate(&H.ev0);
  cudaEventCreate(&H.ev1);
  cudaEventCreate(&H.evt0);
  cudaEventCreate(&H.evt1);
  if ((e = cudaEventCreateWithFlags(&H.ev_enter, cudaEventDisableTiming)) != cudaSuccess) {
    err = std::string("event: ") + cudaGetErrorString(e);
    return -3;
  }
  return 0;
}

cudaError_t handle_enter(Handle& H) {
  cudaError_t e = cudaSetDevice(H.device);
  if (e != cudaSuccess) return e;
  e = cudaEventRecord(H.ev_enter, cudaStreamLegacy);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(H.stream, H.ev_enter, 0);
  return e;
}

cudaError_t handle_leave(Handle& H) {
  cudaError_t e = cudaStreamSynchronize(H.stream);
  if (e == cudaSuccess) e = cudaGetLastError();
  return e;
}

void handle_close(Handle& H) {
  cudaSetDevice(H.device);
  if (H.stream) cudaStreamSynchronize(H.stream);
  H.mg.reset();
  H.split.reset();
  H.perm.reset();
  H.crs_amg.reset();
  H.iface.reset();
  H.dealias.reset();
  gs_free(H.mesh.gs);
  H.mesh.f64.release();
  H.mesh.f32.release();
  cudaFree(H.mesh.dev_err);
  H.mesh.dev_err = nullptr;
  for (cudaEvent_t e : H.ax_ev) cudaEventDestroy(e);
  H.ax_ev.clear();
  if (H.gexec) cudaGraphExecDestroy(H.gexec);
  H.gexec = nullptr;
  cudaFree(H.cg);
  cudaFreeHost(H.cg_host);
  cudaFree(H.flag);
  H.cg = nullptr;
  H.cg_host = nullptr;
  H.flag = nullptr;
  cudaEventDestroy(H.ev0);
  cudaEventDestroy(H.ev1);
  cudaEventDestroy(H.evt0);
  cudaEventDestroy(H.evt1);
  if (H.ev_enter) cudaEventDestroy(H.ev_enter);
  H.ev_enter = nullptr;
  if (H.own_stream && H.stream) cudaStreamDestroy(H.stream);
  H.stream = nullptr;
}

// Mesh sizes, D, and the device arrays of the geometry (old mesh dropped).
static int mesh_prepare(Handle& H, int lx1, int nel, const double* dxm1, std::string& err) {
  if (lx1 < 2 || lx1 > NEKGPU_MAX_LX1) {
    err = "lx1 out of range [2, " + std::to_string(NEKGPU_MAX_LX1) + "]";
    return NEKGPU_EINVAL;
  }
  if (nel < 1) {
    err = "nel must be positive";
    return NEKGPU_EINVAL;
  }
  cudaStreamSynchronize(H.stream);
  H.split.reset();  // maps of the old mesh
  H.perm.reset();
  Mesh& m = H.mesh;
  gs_free(m.gs);
  m.f64.release();
  m.f32.release();
  m.has_f32 = false;
  m.has_df = false;
  m.ax_sel[0] = m.ax_sel[1] = AxShapeSel();
  m.has_rst = false;  // metric terms only come with coordinates (geom.cu)
  H.proj.clear();  // projection spaces belong to the old mesh
  H.mg.reset();    // and so does the pressure preconditioner
  H.iface.reset();  // and the shard's interface maps
  H.dealias.reset();  // and the dealiasing grid
  H.has_mesh = false;
  if (H.gexec) cudaGraphExecDestroy(H.gexec);
  H.gexec = nullptr;
  m.nx1 = lx1;
  m.nel = nel;
  const int P = m.nx1 * m.nx1 * m.nx1;
  m.n = (int64_t)P * m.nel;
  const int64_t n = m.n;
  if (cudaMalloc(&m.f64.G, 6 * n * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&m.f64.bm1, n * sizeof(double)) != cudaSuccess ||
      cudaMalloc(&m.f64.D, m.nx1 * m.nx1 * sizeof(double)) != cudaSuccess) {
    m.f64.release();
    err = "mesh allocation failed";
    return NEKGPU_ENOMEM;
  }
  // D row-major from the Fortran-ordered dxm1(i,j) = dxm1[i + j*lx1]
  m.h_D.assign((size_t)m.nx1 * m.nx1, 0.0);
  for (int i = 0; i < m.nx1; ++i)
    for (int j = 0; j < m.nx1; ++j) m.h_D[i * m.nx1 + j] = dxm1[i + j * m.nx1];
  cudaMemcpy(m.f64.D, m.h_D.data(), m.h_D.size() * sizeof(double), cudaMemcpyHostToDevice);
  return 0;
}

// Numbering-side setup once the geometry is in place.
static int mesh_finish(Handle& H, const int64_t* glo_num, std::string& err) {
  Mesh& m = H.mesh;
  const int64_t n = m.n;
  cudaError_t e;
  if (!m.dev_err && cudaMalloc(&m.dev_err, sizeof(int)) != cudaSuccess) {
    err = "flag allocation failed";
    return NEKGPU_ENOMEM;
  }
  cudaMemset(m.dev_err, 0, sizeof(int));
  const int rc = gs_setup(m.gs, glo_num, n, m.nx1, err);
  if (rc) return rc == -4 ? NEKGPU_ENOMEM : NEKGPU_EINVAL;
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    err = std::string("setup: ") + cudaGetErrorString(e);
    return NEKGPU_ECUDA;
  }
  H.has_mesh = true;
  if (m.use_df && build_df(H)) {
    err = "setup: double-float geometric factors failed";
    return NEKGPU_ECUDA;
  }
  return 0;
}

int handle_setup(Handle& H, int lx1, int nel, const double* dxm1, const double* const* g6,
                 const double* bm1, const int64_t* glo_num, std::string& err) {
  int rc0 = mesh_prepare(H, lx1, nel, dxm1, err);
  if (rc0) return rc0;
  Mesh& m = H.mesh;
  const int64_t n = m.n;
  const int P = m.nx1 * m.nx1 * m.nx1;
  cudaError_t e;
  DevBuf<double> stage;
  if (stage.ensure(n)) {
    err = "staging allocation failed";
    return NEKGPU_ENOMEM;
  }
  for (int q = 0; q < 6; ++q) {
    if ((e = cudaMemcpy(stage.ptr, g6[q], n * sizeof(double), cudaMemcpyHostToDevice)) !=
        cudaSuccess) {
      err = std::string("geometry upload: ") + cudaGetErrorString(e);
      return NEKGPU_ECUDA;
    }
    count_launch();
    pack_g_kernel<<<nblk(n), 256, 0, H.stream>>>(m.f64.G, stage.ptr, q, P, n);
    if ((e = cudaStreamSynchronize(H.stream)) != cudaSuccess) {
      err = std::string("geometry pack: ") + cudaGetErrorString(e);
      return NEKGPU_ECUDA;
    }
  }
  if ((e = cudaMemcpy(m.f64.bm1, bm1, n * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess) {
    err = std::string("mass upload: ") + cudaGetErrorString(e);
    return NEKGPU_ECUDA;
  }
  // volvm1 = glsum(bm1): serial left-to-right, as one rank of the reference
  double vol = 0.0;
  for (int64_t i = 0; i < n; ++i) vol = vol + bm1[i];
  m.vol = vol;
  return mesh_finish(H, glo_num, err);
}

int geom_from_xyz(Handle& H, const double* x, const double* y, const double* z, const double* w,
                  std::string& err);

// As handle_setup, with G and bm1 computed on the device from the GLL
// coordinates (host arrays) and weights.
int handle_setup_xyz(Handle& H, int lx1, int nel, const double* dxm1, const double* wxm1,
                     const double* xm1, const double* ym1, const double* zm1,
                     const int64_t* glo_num, std::string& err) {
  int rc0 = mesh_prepare(H, lx1, nel, dxm1, err);
  if (rc0) return rc0;
  const int64_t n = H.mesh.n;
  if (H.io0.ensure(n) || H.io1.ensure(n) || H.io2.ensure(n)) {
    err = "staging allocation failed";
    return NEKGPU_ENOMEM;
  }
  const double* src[3] = {xm1, ym1, zm1};
  double* dst[3] = {H.io0.ptr, H.io1.ptr, H.io2.ptr};
  for (int q = 0; q < 3; ++q) {
    cudaError_t e = cudaMemcpy(dst[q], src[q], n * sizeof(double), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      err = std::string("coordinate upload: ") + cudaGetErrorString(e);
      return NEKGPU_ECUDA;
    }
  }
  rc0 = geom_from_xyz(H, H.io0.ptr, H.io1.ptr, H.io2.ptr, wxm1, err);
  if (rc0) return rc0;
  return mesh_finish(H, glo_num, err);
}

Handle* handle_lookup(const int64_t* h) { return get(h); }
int handle_fail(Handle* H, int code, const std::string& msg) { return fail(H, code, msg); }

}  // namespace nekgpu

extern "C" {

int nekgpu_init(const int* device, int64_t* handle) {
  if (!device || !handle) return fail(nullptr, NEKGPU_EINVAL, "null argument");
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev == 0) return fail(nullptr, NEKGPU_ECUDA, "no CUDA device");
  if (*device < 0 || *device >= ndev) return fail(nullptr, NEKGPU_EINVAL, "device out of range");
  auto H = std::make_unique<Handle>();
  std::string err;
  if (handle_open(*H, *device, nullptr, err)) return fail(nullptr, NEKGPU_ECUDA, err);
  std::lock_guard<std::mutex> lk(g_mu);
  *handle = g_next++;
  g_handles[*handle] = std::move(H);
  return NEKGPU_OK;
}

int nekgpu_finalize(int64_t* handle) {
  Handle* H = get(handle);
  if (!H) return fail(nullptr, NEKGPU_EHANDLE, "unknown handle");
  handle_close(*H);
  std::lock_guard<std::mutex> lk(g_mu);
  g_handles.erase(*handle);
  *handle = 0;
  return NEKGPU_OK;
}

int nekgpu_last_error(const int64_t* handle, char* buf, const int* buflen) {
  if (!buf || !buflen || *buflen <= 0) return NEKGPU_EINVAL;
  Handle* H = get(handle);
  const std::string& m = H ? H->err : g_orphan_err;
  const size_t k = std::min<size_t>(m.size(), (size_t)*buflen - 1);
  std::memcpy(buf, m.data(), k);
  buf[k] = '\0';
  return NEKGPU_OK;
}

int nekgpu_set_option(const int64_t* handle, const int* key, const int* value) {
  GET_HANDLE(handle);
  if (!key || !value) return fail(H, NEKGPU_EINVAL, "null argument");
  switch (*key) {
    case NEKGPU_OPT_EXACT: H->exact = (*value != 0); break;
    case NEKGPU_OPT_TIMING: H->timing = (*value != 0); break;
    case NEKGPU_OPT_CHUNK:
      if (*value < 1) return fail(H, NEKGPU_EINVAL, "chunk must be >= 1");
      H->graph_chunk = *value;
      break;
    case NEKGPU_OPT_ISTEP: H->istep = *value; break;
    case NEKGPU_OPT_TMA:
      H->mesh.use_tma = (*value != 0);
      H->mesh.ax_sel[1] = AxShapeSel();  // FP32 shape: tuned again (or built-in)
      break;
    case NEKGPU_OPT_AUTOTUNE:
      H->autotune = (*value != 0);
      H->mesh.ax_sel[0] = H->mesh.ax_sel[1] = AxShapeSel();
      H->mesh.gs.cls_tuned[0] = H->mesh.gs.cls_tuned[1] = GsClasses{};
      H->mesh.gs_gshift[0] = H->mesh.gs_gshift[1] = 0;
      H->mesh.gs_ms[0] = H->mesh.gs_ms[1] = 0.f;
      break;
    case NEKGPU_OPT_GRAPH: H->use_graph = (*value != 0); break;
    case NEKGPU_OPT_SPLIT: H->use_split = (*value != 0); break;
    case NEKGPU_OPT_FACE_ORDER: H->use_perm = (*value != 0); break;
    case NEKGPU_OPT_COARSE:
      if (*value != 0 && *value != 1) return fail(H, NEKGPU_EINVAL, "coarse must be 0 or 1");
      H->coarse_amg = (*value == 1);
      break;
    case NEKGPU_OPT_DF:
      H->mesh.use_df = (*value != 0);
      if (H->mesh.use_df && H->has_mesh && !H->mesh.has_df && build_df(*H))
        return fail(H, NEKGPU_ECUDA, "double-float geometric factors failed");
      if (H->gexec) {  // captured FP64 iterations launch the other kernel now
        cudaGraphExecDestroy(H->gexec);
        H->gexec = nullptr;
      }
      break;
    case NEKGPU_OPT_MIXED_MODE:
      if (*value != 0 && *value != 1) return fail(H, NEKGPU_EINVAL, "mixed mode must be 0 or 1");
      H->mixed_mode = *value;
      break;
    default: return fail(H, NEKGPU_EINVAL, "unknown option");
  }
  return NEKGPU_OK;
}

int nekgpu_setup(const int64_t* handle, const int* lx1, const int* nel, const double* dxm1,
                 const double* g1, const double* g2, const double* g3, const double* g4,
                 const double* g5, const double* g6, const double* bm1, const int64_t* glo_num) {
  GET_HANDLE(handle);
  if (!lx1 || !nel || !dxm1 || !g1 || !g2 || !g3 || !g4 || !g5 || !g6 || !bm1 || !glo_num)
    return fail(H, NEKGPU_EINVAL, "null argument");
  const double* g[6] = {g1, g2, g3, g4, g5, g6};
  std::string err;
  const int rc = handle_setup(*H, *lx1, *nel, dxm1, g, bm1, glo_num, err);
  if (rc) return fail(H, rc, err);
  return NEKGPU_OK;
}

int nekgpu_setup_xyz(const int64_t* handle, const int* lx1, const int* nel, const double* dxm1,
                     const double* wxm1, const double* xm1, const double* ym1, const double* zm1,
                     const int64_t* glo_num) {
  GET_HANDLE(handle);
  if (!lx1 || !nel || !dxm1 || !wxm1 || !xm1 || !ym1 || !zm1 || !glo_num)
    return fail(H, NEKGPU_EINVAL, "null argument");
  std::string err;
  const int rc = handle_setup_xyz(*H, *lx1, *nel, dxm1, wxm1, xm1, ym1, zm1, glo_num, err);
  if (rc) return fail(H, rc, err);
  return NEKGPU_OK;
}

int nekgpu_geom_update_dev(const int64_t* handle, const double* wxm1, const double* xm1,
                           const double* ym1, const double* zm1) {
  GET_HANDLE(handle);
  NEED_MESH();
  if (!wxm1 || !xm1 || !ym1 || !zm1) return fail(H, NEKGPU_EINVAL, "null argument");
  std::string err;
  const int rc = geom_from_xyz(*H, xm1, ym1, zm1, wxm1, err);
  if (rc) return fail(H, rc, err);
  if (H->mesh.use_df && build_df(*H)) return fail(H, NEKGPU_ECUDA, "double-float geometric factors failed");
  return NEKGPU_OK;
}

int nekgpu_geometry(const int64_t* handle, double* g1, double* g2, double* g3, double* g4,
                    double* g5, double* g6, double* bm1) {
  GET_HANDLE(handle);
  NEED_MESH();
  const Mesh& m = H->mesh;
  const int64_t n = m.n;
  const int P = m.nx1 * m.nx1 * m.nx1;
  std::vector<double> packed((size_t)(6 * n));
  if (cudaMemcpy(packed.data(), m.f64.G, 6 * n * sizeof(double), cudaMemcpyDeviceToHost) !=
          cudaSuccess ||
      (bm1 && cudaMemcpy(bm1, m.f64.bm1, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess))
    return fail(H, NEKGPU_ECUDA, "geometry download failed");
  double* out[6] = {g1, g2, g3, g4, g5, g6};
  for (int q = 0; q < 6; ++q)
    if (out[q])
      for (int64_t e = 0; e < m.nel; ++e)
        std::memcpy(out[q] + e * P, packed.data() + (e * 6 + q) * P, P * sizeof(double));
  return NEKGPU_OK;
}

int nekgpu_gs_maps(const int64_t* handle, int64_t* nseg, int64_t* nidx, int64_t* seg_start,
                   int64_t* idx) {
  GET_HANDLE(handle);
  NEED_MESH();
  const GsMaps& g = H->mesh.gs;
  if (nseg) *nseg = g.nseg;
  if (nidx) *nidx = g.nidx;
  if (seg_start) std::memcpy(seg_start, g.h_start.data(), g.h_start.size() * sizeof(int64_t));
  if (idx) std::memcpy(idx, g.h_idx.data(), g.h_idx.size() * sizeof(int64_t));
  return NEKGPU_OK;
}

int nekgpu_axhelm_dev(const int64_t* handle, double* au, const double* u, const double* h1,
                      const double* h2, const int* imesh, const int* isd) {
  GET_HANDLE(handle);
  NEED_MESH();
  (void)imesh;
  (void)isd;
  if (check_n(H, au) || check_n(H, u)) return NEKGPU_EINVAL;
  Coef<double> c;
  int rc = make_coef(H, h1, h2, c);
  if (rc) return rc;
  if (H->timing) cudaEventRecord(H->evt0, H->stream);
  rc = axhelm_dev(H, au, u, c);
  if (H->timing && !rc) {
    cudaEventRecord(H->evt1, H->stream);
    cudaEventSynchronize(H->evt1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, H->evt0, H->evt1);
    H->ms_total = ms;
    H->ms_axhelm = ms;
    H->n_axhelm = 1;
  }
  return rc;
}

int nekgpu_axhelm(const int64_t* handle, double* au, const double* u, const double* h1,
                  const double* h2, const int* imesh, const int* isd) {
  GET_HANDLE(handle);
  NEED_MESH();
  if (check_n(H, au) || check_n(H, u) || check_n(H, h1) || check_n(H, h2)) return NEKGPU_EINVAL;
  const int64_t n = H->mesh.n;
  int rc;
  if ((rc = h2d(H, H->io0, u, n)) || (rc = h2d(H, H->io1, h1, n)) || (rc = h2d(H, H->io2, h2, n)))
    return rc;
  if (H->io3.ensure(n)) return fail(H, NEKGPU_ENOMEM, "staging allocation failed");
  rc = nekgpu_axhelm_dev(handle, H->io3.ptr, H->io0.ptr, H->io1.ptr, H->io2.ptr, imesh, isd);
  if (rc) return rc;
  return d2h(H, au, H->io3.ptr, n);
}

int nekgpu_dssum_dev(const int64_t* handle, double* u) {
  GET_HANDLE(handle);
  NEED_MESH();
  if (check_n(H, u)) return NEKGPU_EINVAL;
  gs_op<double>(H->mesh.gs, u, 0, H->stream);
  cudaError_t e = cudaStreamSynchronize(H->stream);
  if (e != cudaSuccess) return cuda_fail(H, e, "dssum");
  return NEKGPU_OK;
}

int nekgpu_dssum(const int64_t* handle, double* u) {
  GET_HANDLE(handle);
  NEED_MESH();
  if (check_n(H, u)) return NEKGPU_EINVAL;
  int rc = h2d(H, H->io0, u, H->mesh.n);
  if (rc) return rc;
  rc = nekgpu_dssum_dev(handle, H->io0.ptr);
  if (rc) return rc;
  return d2h(H, u, H->io0.ptr, H->mesh.n);
}

int nekgpu_dsop_dev(const int64_t* handle, double* u, const char* op) {
  GET_HANDLE(handle);
  NEED_MESH();
  if (check_n(H, u) || !op) return fail(H, NEKGPU_EINVAL, "null argument");
  int code;
  switch (op[0]) {
    case '+': code = 0; break;
    case '*': code = 1; break;
    case 'M': code = 2; break;
    case 'm': code = 3; break;
    default: return fail(H, NEKGPU_EINVAL, "dsop: op must be one of + * M m");
  }
  gs_op<double>(H->mesh.gs, u, code, H->stream);
  cudaError_t e = cudaStreamSynchronize(H->stream);
  if (e != cudaSuccess) return cuda_fail(H, e, "dsop");
  return NEKGPU_OK;
}

int nekgpu_setprec_dev(const int64_t* handle, double* d, const double* h1, const double* h2,
                       const int* imsh, const int* isd) {
  GET_HANDLE(handle);
  NEED_MESH();
  (void)imsh;
  (void)isd;
  if (check_n(H, d)) return NEKGPU_EINVAL;
  Coef<double> c;
  int rc = make_coef(H, h1, h2, c);
  if (rc) return rc;
  if (setprec_f64(*H, d, c)) return fail(H, NEKGPU_ECUDA, "setprec launch");
  cudaError_t e = cudaStreamSynchronize(H->stream);
  if (e != cudaSuccess) return cuda_fail(H, e, "setprec");
  return NEKGPU_OK;
}

int nekgpu_setprec(const int64_t* handle, double* d, const double* h1, const double* h2,
                   const int* imsh, const int* isd) {
  GET_HANDLE(handle);
  NEED_MESH();
  if (check_n(H, d) || check_n(H, h1) || check_n(H, h2)) return NEKGPU_EINVAL;
  const int64_t n = H->mesh.n;
  int rc;
  if ((rc = h2d(H, H->io1, h1, n)) || (rc = h2d(H, H->io2, h2, n))) return rc;
  if (H->io3.ensure(n)) return fail(H, NEKGPU_ENOMEM, "staging allocation failed");
  rc = nekgpu_setprec_dev(handle, H->io3.ptr, H->io1.ptr, H->io2.ptr, imsh, isd);
  if (rc) return rc;
  return d2h(H, d, H->io3.ptr, n);
}

int nekgpu_cggo_dev(const int64_t* handle, double* x, const double* f, const double* h1,
                    const double* h2, const double* mask, const double* mult, const int* imsh,
                    const double* tin, const int* maxit, const int* isd, const double* binv,
                    const int* maxcg, int* niter, double* rbn0, double* rbn2) {
  GET_HANDLE(handle);
  NEED_MESH();
  (void)imsh;
  (void)isd;
  if (check_n(H, x) || check_n(H, f) || check_n(H, mask) || check_n(H, mult) ||
      check_n(H, binv) || !tin || !maxit)
    return fail(H, NEKGPU_EINVAL, "null argument");
  H->ms_axhelm = H->ms_gs = H->ms_update = 0.0;
  H->n_axhelm = 0;
  if (cuda_pending(*H, "cggo: on entry")) return NEKGPU_ECUDA;
  if (H->timing) cudaEventRecord(H->evt0, H->stream);
  if (cuda_pending(*H, "cggo: timing event")) return NEKGPU_ECUDA;
  int rc = cggo_dev(H, x, f, h1, h2, mask, mult, *tin, *maxit, maxcg ? *maxcg : 900, binv, niter,
                    rbn0, rbn2);
  if (H->timing) {
    cudaEventRecord(H->evt1, H->stream);
    cudaEventSynchronize(H->evt1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, H->evt0, H->evt1);
    H->ms_total = ms;
  }
  return rc;
}

int nekgpu_cggo(const int64_t* handle, double* x, const double* f, const double* h1,
                const double* h2, const double* mask, const double* mult, const int* imsh,
                const double* tin, const int* maxit, const int* isd, const double* binv,
                const int* maxcg, int* niter, double* rbn0, double* rbn2) {
  GET_HANDLE(handle);
  NEED_MESH();
  if (check_n(H, x) || check_n(H, f) || check_n(H, h1) || check_n(H, h2) || check_n(H, mask) ||
      check_n(H, mult) || check_n(H, binv))
    return NEKGPU_EINVAL;
  const int64_t n = H->mesh.n;
  int rc;
  if ((rc = h2d(H, H->io0, f, n)) || (rc = h2d(H, H->io1, h1, n)) || (rc = h2d(H, H->io2, h2, n)) ||
      (rc = h2d(H, H->io4, mask, n)) || (rc = h2d(H, H->io5, mult, n)) ||
      (rc = h2d(H, H->io6, binv, n)))
    return rc;
  if (H->io3.ensure(n)) return fail(H, NEKGPU_ENOMEM, "staging allocation failed");
  rc = nekgpu_cggo_dev(handle, H->io3.ptr, H->io0.ptr, H->io1.ptr, H->io2.ptr, H->io4.ptr,
                       H->io5.ptr, imsh, tin, maxit, isd, H->io6.ptr, maxcg, niter, rbn0, rbn2);
  if (rc && rc != NEKGPU_ENOTCONV) return rc;
  int rc2 = d2h(H, x, H->io3.ptr, n);
  return rc2 ? rc2 : rc;
}

int nekgpu_hmholtz_dev(const int64_t* handle, double* u, double* rhs, const double* h1,
                       const double* h2, const double* mask, const double* mult,
                       const int* imsh, const double* tli, const int* maxit, const int* isd,
                       const double* binv, const int* maxcg, int* niter, double* rbn0,
                       double* rbn2) {
  GET_HANDLE(handle);
  NEED_MESH();
  (void)imsh;
  (void)isd;
  if (check_n(H, u) || check_n(H, rhs) || check_n(H, mask) || check_n(H, mult) ||
      check_n(H, binv) || !tli || !maxit)
    return fail(H, NEKGPU_EINVAL, "null argument");
  H->ms_axhelm = H->ms_gs = H->ms_update = 0.0;
  H->n_axhelm = 0;
  if (H->timing) cudaEventRecord(H->evt0, H->stream);
  int rc = hmholtz_dev(H, u, rhs, h1, h2, mask, mult, *tli, *maxit, maxcg ? *maxcg : 900, binv,
                       niter, rbn0, rbn2);
  if (H->timing) {
    cudaEventRecord(H->evt1, H->stream);
    cudaEventSynchronize(H->evt1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, H->evt0, H->evt1);
    H->ms_total = ms;
  }
  return rc;
}

int nekgpu_hmholtz(const int64_t* handle, double* u, double* rhs, const double* h1,
                   const double* h2, const double* mask, const double* mult, const int* imsh,
                   const double* tli, const int* maxit, const int* isd, const double* binv,
                   const int* maxcg, int* niter, double* rbn0, double* rbn2) {
  GET_HANDLE(handle);
  NEED_MESH();
  if (check_n(H, u) || check_n(H, rhs) || check_n(H, h1) || check_n(H, h2) || check_n(H, mask) ||
      check_n(H, mult) || check_n(H, binv))
    return NEKGPU_EINVAL;
  const int64_t n = H->mesh.n;
  int rc;
  if ((rc = h2d(H, H->io0, rhs, n)) || (rc = h2d(H, H->io1, h1, n)) ||
      (rc = h2d(H, H->io2, h2, n)) || (rc = h2d(H, H->io4, mask, n)) ||
      (rc = h2d(H, H->io7, mult, n)) || (rc = h2d(H, H->io8, binv, n)))
    return rc;
  if (H->io3.ensure(n)) return fail(H, NEKGPU_ENOMEM, "staging allocation failed");
  rc = nekgpu_hmholtz_dev(handle, H->io3.ptr, H->io0.ptr, H->io1.ptr, H->io2.ptr, H->io4.ptr,
                          H->io7.ptr, imsh, tli, maxit, isd, H->io8.ptr, maxcg, niter, rbn0, rbn2);
  if (rc && rc != NEKGPU_ENOTCONV) return rc;
  int rc2 = d2h(H, u, H->io3.ptr, n);
  if (!rc2) rc2 = d2h(H, rhs, H->io0.ptr, n);
  return rc2 ? rc2 : rc;
}

int nekgpu_hmh_gmres_dev(const int64_t* handle, double* res, const double* h1, const double* h2,
                         const double* wt, const double* mask, const double* tol,
                         const int* maxit, const int* kmax, const int* null_space, int* niter,
                         double* div0, double* rnorm);

int nekgpu_hmh_gmres(const int64_t* handle, double* res, const double* h1, const double* h2,
                     const double* wt, const double* mask, const double* tol, const int* maxit,
                     const int* kmax, const int* null_space, int* niter, double* div0,
                     double* rnorm) {
  GET_HANDLE(handle);
  NEED_MESH();
  if (check_n(H, res) || check_n(H, h1) || check_n(H, h2) || check_n(H, wt) || check_n(H, mask))
    return NEKGPU_EINVAL;
  const int64_t n = H->mesh.n;
  int rc;
  if ((rc = h2d(H, H->io0, res, n)) || (rc = h2d(H, H->io1, h1, n)) ||
      (rc = h2d(H, H->io2, h2, n)) || (rc = h2d(H, H->io4, wt, n)) ||
      (rc = h2d(H, H->io7, mask, n)))
    return rc;
  rc = nekgpu_hmh_gmres_dev(handle, H->io0.ptr, H->io1.ptr, H->io2.ptr, H->io4.ptr, H->io7.ptr,
                            tol, maxit, kmax, null_space, niter, div0, rnorm);
  if (rc && rc != NEKGPU_ENOTCONV) return rc;
  const int rc2 = d2h(H, res, H->io0.ptr, n);
  return rc2 ? rc2 : rc;
}

int nekgpu_hmh_flex_cg_dev(const int64_t* handle, double* res, const double* h1,
                           const double* h2, const double* wt, const double* mask,
                           const double* tol, const int* maxit, const int* null_space,
                           int* niter, double* div0, double* rnorm);

int nekgpu_hmh_flex_cg(const int64_t* handle, double* res, const double* h1, const double* h2,
                       const double* wt, const double* mask, const double* tol, const int* maxit,
                       const int* null_space, int* niter, double* div0, double* rnorm) {
  GET_HANDLE(handle);
  NEED_MESH();
  if (check_n(H, res) || check_n(H, h1) || check_n(H, h2) || check_n(H, wt) || check_n(H, mask))
    return NEKGPU_EINVAL;
  const int64_t n = H->mesh.n;
  int rc;
  if ((rc = h2d(H, H->io0, res, n)) || (rc = h2d(H, H->io1, h1, n)) ||
      (rc = h2d(H, H->io2, h2, n)) || (rc = h2d(H, H->io4, wt, n)) ||
      (rc = h2d(H, H->io7, mask, n)))
    return rc;
  rc = nekgpu_hmh_flex_cg_dev(handle, H->io0.ptr, H->io1.ptr, H->io2.ptr, H->io4.ptr,
                              H->io7.ptr, tol, maxit, null_space, niter, div0, rnorm);
  if (rc && rc != NEKGPU_ENOTCONV) return rc;
  const int rc2 = d2h(H, res, H->io0.ptr, n);
  return rc2 ? rc2 : rc;
}

int nekgpu_cggo_mixed_dev(const int64_t* handle, double* x, const double* f, const double* h1,
                          const double* h2, const double* mask, const double* mult,
                          const int* imsh, const double* tin, const int* maxit, const int* isd,
                          const double* binv, const double* inner_tol, int* niter_outer,
                          int* niter_inner, double* rbn0, double* rbn2) {
  GET_HANDLE(handle);
  NEED_MESH();
  (void)imsh;
  (void)isd;
  if (check_n(H, x) || check_n(H, f) || check_n(H, h1) || check_n(H, h2) || check_n(H, mask) ||
      check_n(H, mult) || check_n(H, binv) || !tin || !maxit)
    return fail(H, NEKGPU_EINVAL, "null argument");
  const double itol = inner_tol ? *inner_tol : (H->mixed_mode == 1 ? 1e-2 : 1e-5);
  if (!(itol > 0.0 && itol < 1.0)) return fail(H, NEKGPU_EINVAL, "inner_tol must be in (0, 1)");
  H->ms_axhelm = H->ms_gs = H->ms_update = 0.0;
  H->n_axhelm = 0;
  if (H->timing) cudaEventRecord(H->evt0, H->stream);
  MixedResult r = mixed_solve(*H, x, f, h1, h2, mask, mult, binv, *tin, *maxit, itol,
                              H->mixed_mode);
  if (H->timing) {
    cudaEventRecord(H->evt1, H->stream);
    cudaEventSynchronize(H->evt1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, H->evt0, H->evt1);
    H->ms_total = ms;
  }
  if (niter_outer) *niter_outer = r.outer;
  if (niter_inner) *niter_inner = r.inner;
  if (rbn0) *rbn0 = r.rbn0;
  if (rbn2) *rbn2 = r.rbn2;
  if (r.status == -5) return NEKGPU_ENOTCONV;
  if (r.status == -7) return NEKGPU_ENAN;
  if (r.status) return fail(H, r.status, H->err.empty() ? "mixed solve failed" : H->err);
  return NEKGPU_OK;
}

int nekgpu_hmholtz_mixed(const int64_t* handle, double* u, double* rhs, const double* h1,
                         const double* h2, const double* mask, const double* mult,
                         const int* imsh, const double* tli, const int* maxit, const int* isd,
                         const double* binv, const double* inner_tol, int* niter_outer,
                         int* niter_inner, double* rbn0, double* rbn2) {
  GET_HANDLE(handle);
  NEED_MESH();
  if (check_n(H, u) || check_n(H, rhs) || check_n(H, h1) || check_n(H, h2) || check_n(H, mask) ||
      check_n(H, mult) || check_n(H, binv) || !tli)
    return NEKGPU_EINVAL;
  const int64_t n = H->mesh.n;
  int rc;
  if ((rc = h2d(H, H->io0, rhs, n)) || (rc = h2d(H, H->io1, h1, n)) ||
      (rc = h2d(H, H->io2, h2, n)) || (rc = h2d(H, H->io4, mask, n)) ||
      (rc = h2d(H, H->io7, mult, n)) || (rc = h2d(H, H->io8, binv, n)))
    return rc;
  if (H->io3.ensure(n)) return fail(H, NEKGPU_ENOMEM, "staging allocation failed");
  // hmholtz (core/hmholtz.f:50-57): dssum + mask the rhs; a relative tolerance
  // (tli < 0) is used as given, an absolute one goes through chktcg1.
  gs_op<double>(H->mesh.gs, H->io0.ptr, 0, H->stream);
  count_launch();
  mul_kernel<<<nblk(n), 256, 0, H->stream>>>(H->io0.ptr, H->io4.ptr, n);
  double tol = *tli;
  if (tol >= 0) {
    Coef<double> c;
    if ((rc = make_coef(H, H->io1.ptr, H->io2.ptr, c))) return rc;
    if ((rc = chktcg1_dev(H, &tol, H->io0.ptr, c, H->io4.ptr, H->io7.ptr, H->io8.ptr))) return rc;
  }
  rc = nekgpu_cggo_mixed_dev(handle, H->io3.ptr, H->io0.ptr, H->io1.ptr, H->io2.ptr, H->io4.ptr,
                             H->io7.ptr, imsh, &tol, maxit, isd, H->io8.ptr, inner_tol,
                             niter_outer, niter_inner, rbn0, rbn2);
  if (rc && rc != NEKGPU_ENOTCONV) return rc;
  int rc2 = d2h(H, u, H->io3.ptr, n);
  if (!rc2) rc2 = d2h(H, rhs, H->io0.ptr, n);
  return rc2 ? rc2 : rc;
}

int nekgpu_axhelm_adjoint_h1_dev(const int64_t* handle, double* gh1, const double* lam,
                                 const double* u) {
  GET_HANDLE(handle);
  NEED_MESH();
  if (check_n(H, gh1) || check_n(H, lam) || check_n(H, u)) return NEKGPU_EINVAL;
  cudaError_t e = axhelm_adjoint_h1(H->mesh, gh1, lam, u, H->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(H->stream);
  if (e != cudaSuccess) return cuda_fail(H, e, "axhelm_adjoint_h1");
  return NEKGPU_OK;
}

int nekgpu_axhelm_adjoint_h1(const int64_t* handle, double* gh1, const double* lam,
                             const double* u) {
  GET_HANDLE(handle);
  NEED_MESH();
  if (check_n(H, gh1) || check_n(H, lam) || check_n(H, u)) return NEKGPU_EINVAL;
  const int64_t n = H->mesh.n;
  int rc;
  if ((rc = h2d(H, H->io0, lam, n)) || (rc = h2d(H, H->io1, u, n))) return rc;
  if (H->io3.ensure(n)) return fail(H, NEKGPU_ENOMEM, "staging allocation failed");
  rc = nekgpu_axhelm_adjoint_h1_dev(handle, H->io3.ptr, H->io0.ptr, H->io1.ptr);
  if (rc) return rc;
  return d2h(H, gh1, H->io3.ptr, n);
}

int nekgpu_cggo_adjoint_dev(const int64_t* handle, double* lam, const double* g,
                            const double* h1, const double* h2, const double* mask,
                            const double* mult, const int* imsh, const double* tin,
                            const int* maxit, const int* isd, const double* binv,
                            const int* maxcg, int* niter, double* rbn0, double* rbn2) {
  // The Helmholtz operator is symmetric, so the adjoint solve is cggo itself.
  return nekgpu_cggo_dev(handle, lam, g, h1, h2, mask, mult, imsh, tin, maxit, isd, binv, maxcg,
                         niter, rbn0, rbn2);
}

// ---- projection onto previous solutions (proj.cu) ----------------------------
int nekgpu_hsolve_dev(const int64_t* handle, const int* space, double* u, double* r,
                      const double* h1, const double* h2, const double* vmk, const double* vml,
                      const int* imsh, const double* tli, const int* maxit, const int* isd,
                      const double* bi, const int* maxcg, int* niter, double* rbn0,
                      double* rbn2, int* m) {
  GET_HANDLE(handle);
  NEED_MESH();
  (void)imsh;
  (void)isd;
  if (!space || !tli || !maxit || check_n(H, u) || check_n(H, r) || check_n(H, h1) ||
      check_n(H, h2) || check_n(H, vmk) || check_n(H, vml) || check_n(H, bi))
    return fail(H, NEKGPU_EINVAL, "null argument");
  H->err.clear();
  ProjSpace* P = nullptr;
  if (proj_space(*H, *space, &P)) return fail(H, NEKGPU_EINVAL, H->err);
  if (proj_alloc(*H, *P)) return fail(H, NEKGPU_ENOMEM, H->err);
  const int64_t n = H->mesh.n;
  count_launch();
  mul_kernel<<<nblk(n), 256, 0, H->stream>>>(r, vmk, n);  // col2(r, vmk)
  gs_op<double>(H->mesh.gs, r, 0, H->stream);               // dssum(r)
  Coef<double> c;
  int rc = make_coef(H, h1, h2, c);
  if (rc) return rc;
  if ((rc = proj_project1(*H, *P, r, c, h1, h2, vmk, vml)))
    return fail(H, rc == -4 ? NEKGPU_ENOMEM : NEKGPU_ECUDA, H->err);
  double tol = *tli;  // hmhzpf: tol = tli, then chktcg1
  if ((rc = chktcg1_dev(H, &tol, r, c, vmk, vml, bi))) return rc;
  const int cap = maxcg ? *maxcg : 900;
  rc = cggo_dev(H, u, r, h1, h2, vmk, vml, tol, *maxit, cap, bi, niter, rbn0, rbn2);
  if (rc && rc != NEKGPU_ENOTCONV) return rc;
  const int rc2 = proj_project2(*H, *P, u, c, vmk, vml);
  if (rc2) return fail(H, rc2 == -4 ? NEKGPU_ENOMEM : NEKGPU_ECUDA, H->err);
  if (m) *m = P->m;
  return rc;
}

int nekgpu_hsolve(const int64_t* handle, const int* space, double* u, double* r,
                  const double* h1, const double* h2, const double* vmk, const double* vml,
                  const int* imsh, const double* tli, const int* maxit, const int* isd,
                  const double* bi, const int* maxcg, int* niter, double* rbn0, double* rbn2,
                  int* m) {
  GET_HANDLE(handle);
  NEED_MESH();
  if (check_n(H, u) || check_n(H, r) || check_n(H, h1) || check_n(H, h2) || check_n(H, vmk) ||
      check_n(H, vml) || check_n(H, bi))
    return NEKGPU_EINVAL;
  const int64_t n = H->mesh.n;
  int rc;
  if ((rc = h2d(H, H->io0, r, n)) || (rc = h2d(H, H->io1, h1, n)) ||
      (rc = h2d(H, H->io2, h2, n)) || (rc = h2d(H, H->io4, vmk, n)) ||
      (rc = h2d(H, H->io7, vml, n)) || (rc = h2d(H, H->io8, bi, n)))
    return rc;
  if (H->io3.ensure(n)) return fail(H, NEKGPU_ENOMEM, "staging allocation failed");
  rc = nekgpu_hsolve_dev(handle, space, H->io3.ptr, H->io0.ptr, H->io1.ptr, H->io2.ptr,
                         H->io4.ptr, H->io7.ptr, imsh, tli, maxit, isd, H->io8.ptr, maxcg, niter,
                         rbn0, rbn2, m);
  if (rc && rc != NEKGPU_ENOTCONV) return rc;
  int rc2 = d2h(H, u, H->io3.ptr, n);
  if (!rc2) rc2 = d2h(H, r, H->io0.ptr, n);
  return rc2 ? rc2 : rc;
}

int nekgpu_proj_setup(const int64_t* handle, const int* space, const int* mmx) {
  GET_HANDLE(handle);
  if (!space || !mmx) return fail(H, NEKGPU_EINVAL, "null argument");
  if (*mmx < 1 || *mmx > NEKGPU_PROJ_MAX)
    return fail(H, NEKGPU_EINVAL, "mmx must be in [1, NEKGPU_PROJ_MAX]");
  ProjSpace* P = nullptr;
  if (proj_space(*H, *space, &P)) return fail(H, NEKGPU_EINVAL, H->err);
  P->xx.release();
  P->bb.release();
  P->h1old.release();
  P->mmx = *mmx;
  P->m = 0;
  return NEKGPU_OK;
}

int nekgpu_proj_count(const int64_t* handle, const int* space, int* m) {
  GET_HANDLE(handle);
  if (!space || !m) return fail(H, NEKGPU_EINVAL, "null argument");
  ProjSpace* P = nullptr;
  if (proj_space(*H, *space, &P)) return fail(H, NEKGPU_EINVAL, H->err);
  *m = P->m;
  return NEKGPU_OK;
}

// ---- operator launch shapes (autotuner) -------------------------------------
int nekgpu_autotune(const int64_t* handle, const int* precision, const int* h1mode,
                    const int* h2mode, int* kind, int* epb, double* ms) {
  GET_HANDLE(handle);
  NEED_MESH();
  if (!precision || !h1mode || !h2mode) return fail(H, NEKGPU_EINVAL, "null argument");
  const int prec = *precision;
  if (prec != 0 && prec != 1) return fail(H, NEKGPU_EINVAL, "precision must be 0 or 1");
  if (*h1mode < 0 || *h1mode > 1 || *h2mode < 0 || *h2mode > 2)
    return fail(H, NEKGPU_EINVAL, "h1mode must be 0..1 and h2mode 0..2");
  const int64_t n = H->mesh.n;
  const bool was = H->autotune;
  H->autotune = true;
  int rc = 0;
  if (prec == 0) {
    PcgWork<double>& wk = H->w64;
    if (wk.h1.ensure(n) || wk.h2.ensure(n)) rc = NEKGPU_ENOMEM;
    if (!rc) {
      Coef<double> c;
      c.h1mode = *h1mode;
      c.h2mode = *h2mode;
      c.h2s = *h2mode == 1 ? 1.0 : 0.0;
      c.h1 = wk.h1.ptr;
      c.h2 = wk.h2.ptr;
      cudaMemsetAsync(wk.h1.ptr, 0, n * sizeof(double), H->stream);
      cudaMemsetAsync(wk.h2.ptr, 0, n * sizeof(double), H->stream);
      rc = tune_operator<double>(*H, H->mesh.f64, wk, c);
    }
  } else {
    PcgWork<float>& wk = H->w32;
    rc = ensure_f32(*H);
    if (!rc && (wk.h1.ensure(n) || wk.h2.ensure(n))) rc = NEKGPU_ENOMEM;
    if (!rc) {
      Coef<float> c;
      c.h1mode = *h1mode;
      c.h2mode = *h2mode;
      c.h2s = *h2mode == 1 ? 1.f : 0.f;
      c.h1 = wk.h1.ptr;
      c.h2 = wk.h2.ptr;
      cudaMemsetAsync(wk.h1.ptr, 0, n * sizeof(float), H->stream);
      cudaMemsetAsync(wk.h2.ptr, 0, n * sizeof(float), H->stream);
      rc = tune_operator<float>(*H, H->mesh.f32, wk, c);
    }
  }
  H->autotune = was;
  if (rc) return fail(H, rc, H->err.empty() ? "autotune failed" : H->err);
  const AxShapeSel sh = ax_shape_in_use(H->mesh, prec);
  if (kind) *kind = sh.kind;
  if (epb) *epb = sh.epb;
  if (ms) *ms = sh.ms;
  return NEKGPU_OK;
}

int nekgpu_gs_shape(const int64_t* handle, const int* precision, int* threads, int* gshift,
                    double* ms) {
  GET_HANDLE(handle);
  NEED_MESH();
  if (!precision || (*precision != 0 && *precision != 1))
    return fail(H, NEKGPU_EINVAL, "precision must be 0 or 1");
  const GsClasses& c = H->mesh.gs.cls_tuned[*precision];
  const bool tuned = c.threads > 0;
  if (threads) *threads = tuned ? c.threads : H->mesh.gs.cls.threads;
  if (gshift) *gshift = tuned ? H->mesh.gs_gshift[*precision] : 0;
  if (ms) *ms = tuned ? H->mesh.gs_ms[*precision] : 0.0;
  return NEKGPU_OK;
}

int nekgpu_set_gs_shape(const int64_t* handle, const int* threads, const int* gshift) {
  GET_HANDLE(handle);
  NEED_MESH();
  if (!threads || !gshift) return fail(H, NEKGPU_EINVAL, "null argument");
  if (*threads == 0) {  // back to the default / tuning
    H->mesh.gs.cls_tuned[1] = GsClasses{};
    H->mesh.gs_gshift[1] = 0;
    H->mesh.gs_ms[1] = 0.f;
    return NEKGPU_OK;
  }
  if ((*threads != 128 && *threads != 256 && *threads != 512) || *gshift < -1 || *gshift > 1)
    return fail(H, NEKGPU_EINVAL, "threads must be 128, 256 or 512 and gshift -1, 0 or 1");
  H->mesh.gs.cls_tuned[1] = gs_shape(H->mesh.gs.cls, *threads, *gshift);
  H->mesh.gs_gshift[1] = *gshift;
  H->mesh.gs_ms[1] = 0.f;
  return NEKGPU_OK;
}

int nekgpu_ax_shape(const int64_t* handle, const int* precision, int* kind, int* epb,
                    double* ms) {
  GET_HANDLE(handle);
  NEED_MESH();
  if (!precision || (*precision != 0 && *precision != 1))
    return fail(H, NEKGPU_EINVAL, "precision must be 0 or 1");
  const AxShapeSel sh = ax_shape_in_use(H->mesh, *precision);
  if (kind) *kind = sh.kind;
  if (epb) *epb = sh.epb;
  if (ms) *ms = H->mesh.ax_sel[*precision].kind >= 0 ? sh.ms : 0.0;
  return NEKGPU_OK;
}

int nekgpu_set_ax_shape(const int64_t* handle, const int* precision, const int* kind,
                        const int* epb) {
  GET_HANDLE(handle);
  NEED_MESH();
  if (!precision || !kind || !epb) return fail(H, NEKGPU_EINVAL, "null argument");
  const int prec = *precision;
  if (prec != 0 && prec != 1) return fail(H, NEKGPU_EINVAL, "precision must be 0 or 1");
  if (*kind == -1) {  // back to the built-in shape / tuning
    H->mesh.ax_sel[prec] = AxShapeSel();
    return NEKGPU_OK;
  }
  for (const AxShapeSel& c : ax_candidates(H->mesh.nx1, prec, H->mesh.use_tma))
    if (c.kind == *kind && c.epb == *epb) {
      H->mesh.ax_sel[prec] = c;
      return NEKGPU_OK;
    }
  return fail(H, NEKGPU_EINVAL, "not a launch shape of this mesh (nekgpu_ax_candidates)");
}

int nekgpu_ax_candidates(const int64_t* handle, const int* precision, int* kinds, int* epbs,
                         int* count) {
  GET_HANDLE(handle);
  NEED_MESH();
  if (!precision || !count || (*precision != 0 && *precision != 1))
    return fail(H, NEKGPU_EINVAL, "bad argument");
  const std::vector<AxShapeSel> v = ax_candidates(H->mesh.nx1, *precision, H->mesh.use_tma);
  const int cap = *count;
  *count = (int)v.size();
  for (int q = 0; q < (int)v.size() && q < cap; ++q) {
    if (kinds) kinds[q] = v[q].kind;
    if (epbs) epbs[q] = v[q].epb;
  }
  return NEKGPU_OK;
}

int nekgpu_launch_count(int64_t* count) {
  if (!count) return NEKGPU_EINVAL;
  *count = (int64_t)launch_counter().load();
  return NEKGPU_OK;
}

int nekgpu_set_timing(const int64_t* handle, const int* on) {
  GET_HANDLE(handle);
  if (!on) return fail(H, NEKGPU_EINVAL, "null argument");
  H->timing = (*on != 0);
  return NEKGPU_OK;
}

int nekgpu_last_kernel_times(const int64_t* handle, double* ms_axhelm, double* ms_gs,
                             double* ms_update, int* iterations) {
  GET_HANDLE(handle);
  if (ms_axhelm) *ms_axhelm = H->ms_axhelm;
  if (ms_gs) *ms_gs = H->ms_gs;
  if (ms_update) *ms_update = H->ms_update;
  if (iterations) *iterations = H->n_axhelm;
  return NEKGPU_OK;
}

int nekgpu_last_timing(const int64_t* handle, double* ms_total, double* ms_axhelm,
                       int* n_axhelm) {
  GET_HANDLE(handle);
  if (ms_total) *ms_total = H->ms_total;
  if (ms_axhelm) *ms_axhelm = H->ms_axhelm;
  if (n_axhelm) *n_axhelm = H->n_axhelm;
  return NEKGPU_OK;
}

}  // extern "C"
