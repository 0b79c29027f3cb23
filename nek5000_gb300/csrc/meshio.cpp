// meshio.cpp -- mesh ingestion on the host: the reference's .re2 mesh and
// .co2 connectivity files, vertex connectivity from element corners (the
// reference's gencon tool), the global numbering of GLL points (set_vert)
// and the GLL coordinates of straight-sided elements (xyzlin).  Host code
// only; the arrays produced are what nekgpu_setup consumes.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <unordered_map>
#include <vector>

#include "nekmesh.h"

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

// ---- raw file access ---------------------------------------------------------
bool slurp(const char* path, std::vector<unsigned char>& buf) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  const long sz = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  if (sz < 0) {
    std::fclose(f);
    return false;
  }
  buf.resize((size_t)sz);
  const size_t got = sz ? std::fread(buf.data(), 1, (size_t)sz, f) : 0;
  std::fclose(f);
  return got == (size_t)sz;
}

// Words of a binary mesh file: 4 or 8 bytes, either byte order.  Integers in
// 8-byte files are stored as reals (the reference converts them by
// truncation, copyi4 in core/math.f:269).
struct Words {
  const unsigned char* p = nullptr;
  size_t size = 0;
  bool swap = false;
  int wd = 8;

  bool has(size_t off, size_t n) const { return off <= size && n <= size - off; }
  uint32_t u32(size_t off) const {
    unsigned char b[4];
    std::memcpy(b, p + off, 4);
    if (swap) std::reverse(b, b + 4);
    uint32_t v;
    std::memcpy(&v, b, 4);
    return v;
  }
  uint64_t u64(size_t off) const {
    unsigned char b[8];
    std::memcpy(b, p + off, 8);
    if (swap) std::reverse(b, b + 8);
    uint64_t v;
    std::memcpy(&v, b, 8);
    return v;
  }
  double real(size_t off) const {
    if (wd == 8) {
      const uint64_t u = u64(off);
      double d;
      std::memcpy(&d, &u, 8);
      return d;
    }
    const uint32_t u = u32(off);
    float f;
    std::memcpy(&f, &u, 4);
    return (double)f;
  }
  int64_t integer(size_t off) const {
    if (wd == 8) return (int64_t)real(off);  // truncation, as copyi4
    return (int64_t)(int32_t)u32(off);
  }
};

// The byte-order test value every binary file carries after its header.
bool byte_order(const unsigned char* p, bool* swap) {
  for (int s = 0; s < 2; ++s) {
    unsigned char b[4];
    std::memcpy(b, p, 4);
    if (s) std::reverse(b, b + 4);
    float f;
    std::memcpy(&f, b, 4);
    if (std::fabs(f - 6.54321f) < 1e-5f) {
      *swap = s != 0;
      return true;
    }
  }
  return false;
}

// Integer field [a, b) of a fixed-format header (blanks allowed).
bool field_int(const std::string& h, size_t a, size_t b, int64_t* v) {
  if (a >= h.size()) return false;
  std::string s = h.substr(a, b - a);
  char* end = nullptr;
  const long long x = std::strtoll(s.c_str(), &end, 10);
  if (end == s.c_str()) return false;
  *v = x;
  return true;
}

// ---- .re2 --------------------------------------------------------------------
struct Curve {
  int64_t e;
  int side;
  double v[5];
  char type;
};
struct Bc {
  int64_t e;
  int face;
  double v[5];
  char type[3];
};
struct Re2 {
  std::string version;
  int wd = 8, ndim = 3;
  int64_t nelgt = 0, nelgv = 0;
  std::vector<int> group;
  std::vector<double> xc, yc, zc;  // 2^ndim per element, file order
  std::vector<Curve> curves;
  std::vector<std::vector<Bc>> bcs;
};

std::mutex g_mu;
std::unordered_map<int64_t, std::unique_ptr<Re2>> g_meshes;
int64_t g_next = 1;

Re2* lookup(const int64_t* h) {
  if (!h) return nullptr;
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_meshes.find(*h);
  return it == g_meshes.end() ? nullptr : it->second.get();
}

int read_re2(const char* path, Re2& m) {
  std::vector<unsigned char> buf;
  if (!path || !slurp(path, buf)) return fail(NEKGPU_EIO, std::string("cannot read ") + (path ? path : "(null)"));
  if (buf.size() < 84) return fail(NEKGPU_EIO, "re2: file shorter than its header");
  const std::string hdr(reinterpret_cast<const char*>(buf.data()), 80);
  m.version = hdr.substr(0, 5);
  if (m.version.size() != 5 || m.version[0] != '#' || m.version[1] != 'v')
    return fail(NEKGPU_EIO, "re2: no #vNNN version in the header");
  int64_t ndim = 0;
  if (m.version == "#v004") {  // free format: version nelgt ndim nelgv nbc
    char v[8];
    long long a = 0, c = 0, nb = 0;
    int d = 0;
    if (std::sscanf(hdr.c_str(), "%5s %lld %d %lld %lld", v, &a, &d, &c, &nb) < 4)
      return fail(NEKGPU_EIO, "re2: unreadable #v004 header");
    m.nelgt = a;
    ndim = d;
    m.nelgv = c;
  } else if (!field_int(hdr, 5, 14, &m.nelgt) || !field_int(hdr, 14, 17, &ndim) ||
             !field_int(hdr, 17, 26, &m.nelgv)) {
    return fail(NEKGPU_EIO, "re2: unreadable header (format a5,i9,i3,i9)");
  }
  m.wd = (m.version == "#v002" || m.version == "#v003" || m.version == "#v004") ? 8 : 4;
  m.ndim = (int)ndim;
  if (m.ndim != 2 && m.ndim != 3) return fail(NEKGPU_EIO, "re2: ndim must be 2 or 3");
  if (m.nelgt <= 0 || m.nelgv <= 0 || m.nelgv > m.nelgt)
    return fail(NEKGPU_EIO, "re2: invalid element counts in the header");
  Words w;
  w.p = buf.data();
  w.size = buf.size();
  w.wd = m.wd;
  if (!byte_order(buf.data() + 80, &w.swap)) return fail(NEKGPU_EIO, "re2: byte-order test value not found");
  const int nv = 1 << m.ndim;
  const size_t rec = (size_t)(1 + m.ndim * nv) * m.wd;  // group, x(nv), y(nv)[, z(nv)]
  size_t off = 84;
  if (!w.has(off, rec * (size_t)m.nelgt)) return fail(NEKGPU_EIO, "re2: file ends inside the element records");
  const size_t ne = (size_t)m.nelgt;
  m.group.resize(ne);
  m.xc.resize(ne * nv);
  m.yc.resize(ne * nv);
  m.zc.assign(m.ndim == 3 ? ne * nv : 0, 0.0);
  for (size_t e = 0; e < ne; ++e, off += rec) {
    m.group[e] = (int)w.integer(off);
    for (int c = 0; c < nv; ++c) {
      m.xc[e * nv + c] = w.real(off + (size_t)(1 + c) * m.wd);
      m.yc[e * nv + c] = w.real(off + (size_t)(1 + nv + c) * m.wd);
      if (m.ndim == 3) m.zc[e * nv + c] = w.real(off + (size_t)(1 + 2 * nv + c) * m.wd);
    }
  }
  // curved sides: a count word, then records eg, side, curve(5), type
  const size_t r8 = (size_t)8 * m.wd;
  if (!w.has(off, m.wd)) return fail(NEKGPU_EIO, "re2: file ends before the curved-side count");
  const int64_t ncurve = w.integer(off);
  off += m.wd;
  if (ncurve < 0 || !w.has(off, r8 * (size_t)ncurve))
    return fail(NEKGPU_EIO, "re2: file ends inside the curved-side records");
  m.curves.resize((size_t)ncurve);
  for (int64_t q = 0; q < ncurve; ++q, off += r8) {
    Curve& c = m.curves[(size_t)q];
    c.e = w.integer(off);
    c.side = (int)w.integer(off + m.wd);
    for (int k = 0; k < 5; ++k) c.v[k] = w.real(off + (size_t)(2 + k) * m.wd);
    c.type = (char)buf[off + 7 * (size_t)m.wd];  // characters are not byte-swapped
    if (c.e < 1 || c.e > m.nelgt) return fail(NEKGPU_EIO, "re2: curved-side record names no element");
  }
  // boundary-condition sections until the end of the file
  while (off < buf.size()) {
    if (!w.has(off, m.wd)) return fail(NEKGPU_EIO, "re2: truncated boundary-condition count");
    const int64_t nbc = w.integer(off);
    off += m.wd;
    if (nbc < 0 || !w.has(off, r8 * (size_t)nbc))
      return fail(NEKGPU_EIO, "re2: file ends inside the boundary-condition records");
    std::vector<Bc> sec((size_t)nbc);
    for (int64_t q = 0; q < nbc; ++q, off += r8) {
      Bc& b = sec[(size_t)q];
      b.e = w.integer(off);
      b.face = (int)w.integer(off + m.wd);
      for (int k = 0; k < 5; ++k) b.v[k] = w.real(off + (size_t)(2 + k) * m.wd);
      std::memcpy(b.type, &buf[off + 7 * (size_t)m.wd], 3);
      if (b.e < 1 || b.e > m.nelgt || b.face < 1 || b.face > 2 * m.ndim)
        return fail(NEKGPU_EIO, "re2: boundary-condition record names no element face");
    }
    m.bcs.push_back(std::move(sec));
  }
  return NEKGPU_OK;
}

// ---- connectivity (the algorithm of the reference's gencon tool) -------------
// Corner order conversions: the file (preprocessor) order lists the bottom
// face counter-clockwise, then the top; tensor order is i + 2 j + 4 k.
constexpr int kPreOfTensor[8] = {0, 1, 3, 2, 4, 5, 7, 6};
// Preprocessor face of each tensor face (r-, r+, s-, s+, t-, t+), and back.
constexpr int kPreFace[6] = {4, 2, 1, 3, 5, 6};
constexpr int kTensorFace[6] = {3, 2, 4, 1, 5, 6};
// Corners of each tensor face in circulant order (counter-clockwise seen
// from outside), used to match periodic face pairs.
constexpr int kFaceCycle[6][4] = {{0, 4, 6, 2}, {1, 3, 7, 5}, {0, 1, 5, 4},
                                  {2, 6, 7, 3}, {0, 2, 3, 1}, {4, 5, 7, 6}};
// Corners of each tensor face (face_chk order).
constexpr int kFaceCorners[6][4] = {{0, 2, 4, 6}, {1, 3, 5, 7}, {0, 1, 4, 5},
                                    {2, 3, 6, 7}, {0, 1, 2, 3}, {4, 5, 6, 7}};
// The three edge neighbours of each tensor corner.
constexpr int kNeighbour[8][3] = {{1, 2, 4}, {0, 3, 5}, {0, 3, 6}, {1, 2, 7},
                                  {0, 5, 6}, {1, 4, 7}, {2, 4, 7}, {3, 5, 6}};

struct Dsu {
  std::vector<int64_t> parent;
  explicit Dsu(int64_t n) : parent((size_t)n) { std::iota(parent.begin(), parent.end(), 0); }
  int64_t find(int64_t a) {
    while (parent[(size_t)a] != a) {
      parent[(size_t)a] = parent[(size_t)parent[(size_t)a]];
      a = parent[(size_t)a];
    }
    return a;
  }
  // the representative of a set is its smallest member
  void join(int64_t a, int64_t b) {
    a = find(a);
    b = find(b);
    if (a == b) return;
    if (b < a) std::swap(a, b);
    parent[(size_t)b] = a;
  }
};

// Rank the values of ids (1-based, ascending order of value).
int64_t rank_ids(std::vector<int64_t>& ids) {
  std::vector<int64_t> u(ids);
  std::sort(u.begin(), u.end());
  u.erase(std::unique(u.begin(), u.end()), u.end());
  for (auto& v : ids) v = (int64_t)(std::lower_bound(u.begin(), u.end(), v) - u.begin()) + 1;
  return (int64_t)u.size();
}

// Lexicographic segmentation of all element corners (unique_vertex2): within
// each segment, sort by one coordinate and cut where neighbours differ by
// more than tol times the smaller of their characteristic lengths; ndim
// passes over the ndim coordinates.  Corners left in one segment are one
// vertex; vertex ids are the segments' ranks in the final order.
std::vector<int64_t> unique_vertices(const std::vector<double>& X, const std::vector<double>& L2,
                                     int64_t n, double tol) {
  const double qq = tol * tol;
  std::vector<int64_t> order((size_t)n);
  std::iota(order.begin(), order.end(), 0);
  std::vector<char> cut((size_t)n, 0);
  if (n) cut[0] = 1;
  for (int pass = 0; pass < 3; ++pass)
    for (int j = 0; j < 3; ++j) {
      int64_t a = 0;
      while (a < n) {
        int64_t b = a + 1;
        while (b < n && !cut[(size_t)b]) ++b;
        std::stable_sort(order.begin() + a, order.begin() + b, [&](int64_t p, int64_t q) {
          return X[(size_t)(3 * p + j)] < X[(size_t)(3 * q + j)];
        });
        a = b;
      }
      for (int64_t i = 1; i < n; ++i) {
        const int64_t p = order[(size_t)i], q = order[(size_t)(i - 1)];
        const double d = X[(size_t)(3 * p + j)] - X[(size_t)(3 * q + j)];
        if (d * d > qq * std::min(L2[(size_t)p], L2[(size_t)q])) cut[(size_t)i] = 1;
      }
    }
  std::vector<int64_t> id((size_t)n);
  int64_t g = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (cut[(size_t)i]) ++g;
    id[(size_t)order[(size_t)i]] = g;
  }
  return id;
}

// face_chk: a face of element e whose corners are shared, three of four, with
// element f gets the fourth joined to the corner of f's matching face that
// e does not share.  Returns whether a join was made.
bool repair_faces(std::vector<int64_t>& cell, int64_t nel) {
  // vertex -> elements
  int64_t nvid = 0;
  for (auto v : cell) nvid = std::max(nvid, v);
  std::vector<int64_t> start((size_t)nvid + 2, 0);
  for (auto v : cell) ++start[(size_t)v + 1];
  for (size_t i = 1; i < start.size(); ++i) start[i] += start[i - 1];
  std::vector<int64_t> elems(cell.size());
  {
    std::vector<int64_t> fill(start.begin(), start.end() - 1);
    for (int64_t e = 0; e < nel; ++e)
      for (int c = 0; c < 8; ++c) elems[(size_t)fill[(size_t)cell[(size_t)(8 * e + c)]]++] = e;
  }
  auto touches = [&](int64_t v, int64_t e) {
    for (int64_t k = start[(size_t)v]; k < start[(size_t)v + 1]; ++k)
      if (elems[(size_t)k] == e) return true;
    return false;
  };
  std::vector<int64_t> share;
  for (int64_t e = 0; e < nel; ++e)
    for (int f = 0; f < 6; ++f) {
      share.clear();
      for (int c = 0; c < 4; ++c) {
        const int64_t v = cell[(size_t)(8 * e + kFaceCorners[f][c])];
        for (int64_t k = start[(size_t)v]; k < start[(size_t)v + 1]; ++k)
          if (elems[(size_t)k] != e) share.push_back(elems[(size_t)k]);
      }
      std::sort(share.begin(), share.end());
      for (size_t a = 0; a < share.size();) {
        size_t b = a;
        while (b < share.size() && share[b] == share[a]) ++b;
        if (b - a == 3) {  // three corners shared with element o: find the fourth
          const int64_t o = share[a];
          int miss = -1;
          for (int c = 0; c < 4; ++c)
            if (!touches(cell[(size_t)(8 * e + kFaceCorners[f][c])], o)) miss = kFaceCorners[f][c];
          // o's face with three corners on e, and its corner not on e
          int other = -1;
          for (int g = 0; g < 6 && other < 0; ++g) {
            int cnt = 0, lone = -1;
            for (int c = 0; c < 4; ++c) {
              if (touches(cell[(size_t)(8 * o + kFaceCorners[g][c])], e)) ++cnt;
              else lone = kFaceCorners[g][c];
            }
            if (cnt == 3) other = lone;
          }
          if (miss < 0 || other < 0) return false;
          const int64_t v1 = cell[(size_t)(8 * e + miss)], v2 = cell[(size_t)(8 * o + other)];
          const int64_t keep = std::min(v1, v2), drop = std::max(v1, v2);
          for (auto& v : cell)
            if (v == drop) v = keep;
          return true;
        }
        a = b;
      }
    }
  return false;
}

}  // namespace

namespace nekgpu {
// the message nekmesh_last_error returns, from the other host-only entry points
int mesh_fail(int code, const std::string& msg) { return fail(code, msg); }
}  // namespace nekgpu

// =============================================================================
// C ABI
extern "C" {

int nekmesh_last_error(char* buf, const int* buflen) {
  if (!buf || !buflen || *buflen <= 0) return NEKGPU_EINVAL;
  std::snprintf(buf, (size_t)*buflen, "%s", g_err.c_str());
  return NEKGPU_OK;
}

int nekmesh_re2_open(const char* path, int64_t* mesh) {
  if (!mesh) return fail(NEKGPU_EINVAL, "null mesh handle");
  auto m = std::make_unique<Re2>();
  const int rc = read_re2(path, *m);
  if (rc) return rc;
  std::lock_guard<std::mutex> lk(g_mu);
  *mesh = g_next++;
  g_meshes[*mesh] = std::move(m);
  return NEKGPU_OK;
}

int nekmesh_re2_header(const int64_t* mesh, int* nelgt, int* ndim, int* nelgv, int* wdsize,
                       int64_t* ncurve, int* nbcfield) {
  Re2* m = lookup(mesh);
  if (!m) return fail(NEKGPU_EHANDLE, "unknown mesh handle");
  if (nelgt) *nelgt = (int)m->nelgt;
  if (ndim) *ndim = m->ndim;
  if (nelgv) *nelgv = (int)m->nelgv;
  if (wdsize) *wdsize = m->wd;
  if (ncurve) *ncurve = (int64_t)m->curves.size();
  if (nbcfield) *nbcfield = (int)m->bcs.size();
  return NEKGPU_OK;
}

int nekmesh_re2_xyz(const int64_t* mesh, double* xc, double* yc, double* zc, int* group) {
  Re2* m = lookup(mesh);
  if (!m) return fail(NEKGPU_EHANDLE, "unknown mesh handle");
  if (xc) std::copy(m->xc.begin(), m->xc.end(), xc);
  if (yc) std::copy(m->yc.begin(), m->yc.end(), yc);
  if (zc && m->ndim == 3) std::copy(m->zc.begin(), m->zc.end(), zc);
  if (group) std::copy(m->group.begin(), m->group.end(), group);
  return NEKGPU_OK;
}

int nekmesh_re2_curves(const int64_t* mesh, int* elem, int* side, double* curve, char* ccurve) {
  Re2* m = lookup(mesh);
  if (!m) return fail(NEKGPU_EHANDLE, "unknown mesh handle");
  for (size_t q = 0; q < m->curves.size(); ++q) {
    const Curve& c = m->curves[q];
    if (elem) elem[q] = (int)c.e;
    if (side) side[q] = c.side;
    if (curve) std::copy(c.v, c.v + 5, curve + 5 * q);
    if (ccurve) ccurve[q] = c.type;
  }
  return NEKGPU_OK;
}

int nekmesh_re2_bc(const int64_t* mesh, const int* field, char* cbc, double* bc) {
  Re2* m = lookup(mesh);
  if (!m) return fail(NEKGPU_EHANDLE, "unknown mesh handle");
  if (!field || *field < 0 || *field >= (int)m->bcs.size())
    return fail(NEKGPU_EINVAL, "no such boundary-condition section");
  const int nf = 2 * m->ndim;
  const size_t nfe = (size_t)m->nelgt * nf;
  if (cbc)
    for (size_t q = 0; q < nfe; ++q) std::memcpy(cbc + 3 * q, "E  ", 3);
  if (bc) std::fill(bc, bc + 5 * nfe, 0.0);
  for (const Bc& b : m->bcs[(size_t)*field]) {
    const size_t q = (size_t)(b.e - 1) * nf + (size_t)(b.face - 1);
    if (cbc) std::memcpy(cbc + 3 * q, b.type, 3);
    if (bc) std::copy(b.v, b.v + 5, bc + 5 * q);
  }
  return NEKGPU_OK;
}

int nekmesh_re2_close(int64_t* mesh) {
  if (!mesh) return fail(NEKGPU_EINVAL, "null mesh handle");
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_meshes.erase(*mesh)) return fail(NEKGPU_EHANDLE, "unknown mesh handle");
  *mesh = 0;
  return NEKGPU_OK;
}

int nekmesh_co2_read(const char* path, int* nelgt, int* nelgv, int* nv, int64_t* vertex) {
  std::vector<unsigned char> buf;
  if (!path || !slurp(path, buf)) return fail(NEKGPU_EIO, std::string("cannot read ") + (path ? path : "(null)"));
  if (buf.size() < 136) return fail(NEKGPU_EIO, "co2: file shorter than its header");
  const std::string hdr(reinterpret_cast<const char*>(buf.data()), 132);
  const std::string version = hdr.substr(0, 5);
  int64_t a = 0, b = 0, c = 0;
  if (version == "#v002") {
    char v[8];
    long long x = 0, y = 0, z = 0;
    if (std::sscanf(hdr.c_str(), "%5s %lld %lld %lld", v, &x, &y, &z) != 4)
      return fail(NEKGPU_EIO, "co2: unreadable #v002 header");
    a = x;
    b = y;
    c = z;
  } else if (!field_int(hdr, 5, 17, &a) || !field_int(hdr, 17, 29, &b) || !field_int(hdr, 29, 41, &c)) {
    return fail(NEKGPU_EIO, "co2: unreadable header (format a5,3i12)");
  }
  if (a <= 0 || b <= 0 || b > a || (c != 4 && c != 8)) return fail(NEKGPU_EIO, "co2: invalid sizes in the header");
  Words w;
  w.p = buf.data();
  w.size = buf.size();
  w.wd = 4;
  if (!byte_order(buf.data() + 132, &w.swap)) return fail(NEKGPU_EIO, "co2: byte-order test value not found");
  if (nelgt) *nelgt = (int)a;
  if (nelgv) *nelgv = (int)b;
  if (nv) *nv = (int)c;
  if (!vertex) return NEKGPU_OK;
  const size_t rec = (size_t)(c + 1) * 4;
  if (!w.has(136, rec * (size_t)a)) return fail(NEKGPU_EIO, "co2: file ends inside the records");
  std::vector<char> seen((size_t)a, 0);
  for (int64_t r = 0; r < a; ++r) {
    const size_t off = 136 + rec * (size_t)r;
    const int64_t eid = (int64_t)(int32_t)w.u32(off);
    if (eid < 1 || eid > a || seen[(size_t)(eid - 1)])
      return fail(NEKGPU_EIO, "co2: element ids are not a permutation of 1..nelgt");
    seen[(size_t)(eid - 1)] = 1;
    for (int64_t k = 0; k < c; ++k)
      vertex[(size_t)((eid - 1) * c + k)] = (int64_t)(int32_t)w.u32(off + 4 * (size_t)(k + 1));
  }
  return NEKGPU_OK;
}

int nekmesh_ma2_read(const char* path, int* nel, int* nv, int64_t* vertex, int* part) {
  std::vector<unsigned char> buf;
  if (!path || !slurp(path, buf)) return fail(NEKGPU_EIO, std::string("cannot read ") + (path ? path : "(null)"));
  if (buf.size() < 136) return fail(NEKGPU_EIO, "ma2: file shorter than its header");
  const std::string hdr(reinterpret_cast<const char*>(buf.data()), 132);
  int64_t ne = 0;
  if (hdr.compare(0, 2, "#v") != 0 || !field_int(hdr, 5, 17, &ne) || ne <= 0)
    return fail(NEKGPU_EIO, "ma2: unreadable header (format a5,7i12)");
  Words w;
  w.p = buf.data();
  w.size = buf.size();
  w.wd = 4;
  if (!byte_order(buf.data() + 132, &w.swap)) return fail(NEKGPU_EIO, "ma2: byte-order test value not found");
  const size_t body = buf.size() - 136;
  if (body % ((size_t)ne * 4) != 0) return fail(NEKGPU_EIO, "ma2: records do not fill the file");
  const int64_t per = (int64_t)(body / ((size_t)ne * 4));  // partition + vertices
  if (per != 5 && per != 9) return fail(NEKGPU_EIO, "ma2: records of neither 4 nor 8 vertices");
  if (nel) *nel = (int)ne;
  if (nv) *nv = (int)(per - 1);
  for (int64_t e = 0; e < ne; ++e) {
    const size_t off = 136 + (size_t)(e * per) * 4;
    if (part) part[e] = (int)(int32_t)w.u32(off);
    if (vertex)
      for (int64_t k = 0; k < per - 1; ++k)
        vertex[(size_t)(e * (per - 1) + k)] = (int64_t)(int32_t)w.u32(off + 4 * (size_t)(k + 1));
  }
  return NEKGPU_OK;
}

int nekmesh_co2_write(const char* path, const int* nelgt, const int* nelgv, const int* nv,
                      const int64_t* vertex) {
  if (!path || !nelgt || !nelgv || !nv || !vertex || *nelgt <= 0 || *nelgv <= 0 ||
      *nelgv > *nelgt || (*nv != 4 && *nv != 8))
    return fail(NEKGPU_EINVAL, "co2 write: bad arguments");
  FILE* f = std::fopen(path, "wb");
  if (!f) return fail(NEKGPU_EIO, std::string("cannot write ") + path);
  char hdr[133];
  std::memset(hdr, ' ', 132);
  char tmp[64];
  const int len = std::snprintf(tmp, sizeof tmp, "#v001%12d%12d%12d", *nelgt, *nelgv, *nv);
  std::memcpy(hdr, tmp, (size_t)len);
  const float test = 6.54321f;
  bool ok = std::fwrite(hdr, 1, 132, f) == 132 && std::fwrite(&test, 4, 1, f) == 1;
  std::vector<int32_t> rec((size_t)*nv + 1);
  for (int e = 0; ok && e < *nelgt; ++e) {
    rec[0] = e + 1;
    for (int k = 0; k < *nv; ++k) {
      const int64_t v = vertex[(size_t)e * *nv + k];
      if (v < 1 || v > INT32_MAX) ok = false;
      rec[(size_t)k + 1] = (int32_t)v;
    }
    ok = ok && std::fwrite(rec.data(), 4, rec.size(), f) == rec.size();
  }
  ok = (std::fclose(f) == 0) && ok;
  return ok ? NEKGPU_OK : fail(NEKGPU_EIO, std::string("co2 write failed: ") + path);
}

int nekmesh_connect(const int* nel_, const int* ndim_, const double* xc, const double* yc,
                    const double* zc, const char* cbc, const double* bc, const double* tol_,
                    int64_t* vertex, int64_t* nvert) {
  if (!nel_ || !ndim_ || !xc || !yc || !zc || !vertex || *nel_ <= 0)
    return fail(NEKGPU_EINVAL, "connect: bad arguments");
  if (*ndim_ != 3) return fail(NEKGPU_EINVAL, "connect: only ndim = 3 is served");
  const int64_t nel = *nel_, n = 8 * nel;
  const double tol = tol_ ? *tol_ : 0.2;
  if (!(tol > 0.0)) return fail(NEKGPU_EINVAL, "connect: tolerance must be positive");
  // corners in tensor order; squared shortest edge at each corner (set_d2)
  std::vector<double> X((size_t)(3 * n)), L2((size_t)n);
  for (int64_t e = 0; e < nel; ++e)
    for (int c = 0; c < 8; ++c) {
      const size_t src = (size_t)(8 * e + kPreOfTensor[c]), dst = (size_t)(8 * e + c);
      X[3 * dst] = xc[src];
      X[3 * dst + 1] = yc[src];
      X[3 * dst + 2] = zc[src];
    }
  for (int64_t e = 0; e < nel; ++e)
    for (int c = 0; c < 8; ++c) {
      double m = 1e300;
      const size_t p = (size_t)(8 * e + c);
      for (int k = 0; k < 3; ++k) {
        const size_t q = (size_t)(8 * e + kNeighbour[c][k]);
        double d2 = 0.0;
        for (int j = 0; j < 3; ++j) d2 += (X[3 * q + j] - X[3 * p + j]) * (X[3 * q + j] - X[3 * p + j]);
        m = std::min(m, d2);
      }
      L2[p] = m;
    }
  std::vector<int64_t> cell = unique_vertices(X, L2, n, tol);
  rank_ids(cell);
  // repair faces that share three of four corners (at most five rounds)
  for (int round = 0; round < 5; ++round)
    if (!repair_faces(cell, nel)) break;
  rank_ids(cell);
  // periodic face pairs
  if (cbc && bc) {
    Dsu dsu(n + 1);
    bool any = false;
    for (int64_t e = 0; e < nel; ++e)
      for (int tf = 0; tf < 6; ++tf) {
        const size_t q = (size_t)(6 * e + kPreFace[tf] - 1);
        if (std::memcmp(cbc + 3 * q, "P  ", 3) != 0) continue;
        any = true;
        const int64_t je = (int64_t)std::fabs(bc[5 * q]) - 1;
        const int jpf = (int)bc[5 * q + 1];
        if (je < 0 || je >= nel || jpf < 1 || jpf > 6)
          return fail(NEKGPU_EINVAL, "connect: periodic face names no element face");
        const int jf = kTensorFace[jpf - 1] - 1;
        const size_t qj = (size_t)(6 * je + jpf - 1);
        if (std::memcmp(cbc + 3 * qj, "P  ", 3) != 0 || (int64_t)std::fabs(bc[5 * qj]) - 1 != e ||
            kTensorFace[(int)bc[5 * qj + 1] - 1] - 1 != tf)
          return fail(NEKGPU_EINVAL, "connect: periodic faces do not point at each other");
        // both faces' corners about their means; the cyclic shift (walking the
        // partner face backwards) that brings them closest
        double a[4][3], b[4][3], mean_a[3] = {0, 0, 0}, mean_b[3] = {0, 0, 0}, x0m = 0.0;
        for (int i = 0; i < 4; ++i)
          for (int k = 0; k < 3; ++k) {
            a[i][k] = X[(size_t)(3 * (8 * e + kFaceCycle[tf][i]) + k)];
            b[i][k] = X[(size_t)(3 * (8 * je + kFaceCycle[jf][i]) + k)];
            mean_a[k] += a[i][k];
            mean_b[k] += b[i][k];
            x0m = std::max(x0m, std::max(std::fabs(a[i][k]), std::fabs(b[i][k])));
          }
        for (int i = 0; i < 4; ++i)
          for (int k = 0; k < 3; ++k) {
            a[i][k] -= mean_a[k] / 4;
            b[i][k] -= mean_b[k] / 4;
          }
        int best = 0;
        double dmin = 1e300;
        for (int s = 0; s < 4; ++s) {
          double d2 = 0.0;
          for (int i = 0; i < 4; ++i) {
            const int j = 3 - (i + s) % 4;
            for (int k = 0; k < 3; ++k) d2 += (a[i][k] - b[j][k]) * (a[i][k] - b[j][k]);
          }
          if (d2 < dmin) {
            dmin = d2;
            best = s;
          }
        }
        if (std::sqrt(dmin) > 1e-3 * x0m)
          return fail(NEKGPU_EINVAL, "connect: periodic face pair " + std::to_string(e + 1) + "/" +
                                         std::to_string(tf + 1) + " does not match its partner");
        for (int i = 0; i < 4; ++i) {
          const int j = 3 - (i + best) % 4;
          dsu.join(cell[(size_t)(8 * e + kFaceCycle[tf][i])], cell[(size_t)(8 * je + kFaceCycle[jf][j])]);
        }
      }
    if (any) {
      for (auto& v : cell) v = dsu.find(v);
      rank_ids(cell);
    }
  }
  // no element may meet itself (self_chk)
  for (int64_t e = 0; e < nel; ++e)
    for (int i = 0; i < 8; ++i)
      for (int j = i + 1; j < 8; ++j)
        if (cell[(size_t)(8 * e + i)] == cell[(size_t)(8 * e + j)])
          return fail(NEKGPU_EINVAL, "connect: element " + std::to_string(e + 1) +
                                         " has two corners on one vertex (tighten the tolerance)");
  int64_t nv = 0;
  for (int64_t i = 0; i < n; ++i) {
    vertex[i] = cell[(size_t)i];
    nv = std::max(nv, cell[(size_t)i]);
  }
  if (nvert) *nvert = nv;
  return NEKGPU_OK;
}

int nekmesh_setvert3d(const int* nx_, const int* nel_, const int64_t* vertex, int64_t* glo_num,
                      int64_t* ngv_out) {
  if (!nx_ || !nel_ || !vertex || !glo_num || *nx_ < 2 || *nel_ <= 0)
    return fail(NEKGPU_EINVAL, "setvert3d: bad arguments");
  const int64_t nx = *nx_, nel = *nel_, nxyz = nx * nx * nx, nxx = nx * nx;
  auto G = [&](int64_t e, int64_t i, int64_t j, int64_t k) -> int64_t& {  // 0-based i, j, k
    return glo_num[(size_t)(nxyz * e + i + nx * (j + nx * k))];
  };
  std::fill(glo_num, glo_num + nxyz * nel, (int64_t)0);
  int64_t ngv = 0;
  for (int64_t q = 0; q < 8 * nel; ++q) ngv = std::max(ngv, vertex[q]);
  for (int64_t e = 0; e < nel; ++e)
    for (int c = 0; c < 8; ++c)
      G(e, (c & 1) * (nx - 1), ((c >> 1) & 1) * (nx - 1), (c >> 2) * (nx - 1)) = vertex[8 * e + c];
  if (nx == 2) {
    if (ngv_out) *ngv_out = ngv;
    return NEKGPU_OK;
  }
  // ---- edges: ranked by their (smaller, larger) end ids.  Edge slot s of an
  // element: r-edges s = j + 2k, s-edges 4 + i + 2k, t-edges 8 + i + 2j.
  struct Key {
    int64_t a, b, c;
    int64_t pos;
  };
  auto rank_keys = [](std::vector<Key>& t, std::vector<int64_t>& rank) {
    std::sort(t.begin(), t.end(), [](const Key& x, const Key& y) {
      if (x.a != y.a) return x.a < y.a;
      if (x.b != y.b) return x.b < y.b;
      if (x.c != y.c) return x.c < y.c;
      return x.pos < y.pos;
    });
    int64_t r = 0;
    for (size_t i = 0; i < t.size(); ++i) {
      if (i == 0 || t[i].a != t[i - 1].a || t[i].b != t[i - 1].b || t[i].c != t[i - 1].c) ++r;
      rank[(size_t)t[i].pos] = r;
    }
    return r;
  };
  std::vector<Key> keys((size_t)(12 * nel));
  std::vector<int64_t> enm((size_t)(12 * nel));
  for (int64_t e = 0; e < nel; ++e) {
    const int64_t* v = vertex + 8 * e;
    for (int s = 0; s < 12; ++s) {
      int c0, c1;
      const int b0 = s & 1, b1 = (s >> 1) & 1;
      if (s < 4) {  // r-edge (j, k) = (b0, b1)
        c0 = 2 * b0 + 4 * b1;
        c1 = c0 + 1;
      } else if (s < 8) {  // s-edge (i, k)
        c0 = b0 + 4 * b1;
        c1 = c0 + 2;
      } else {  // t-edge (i, j)
        c0 = b0 + 2 * b1;
        c1 = c0 + 4;
      }
      keys[(size_t)(12 * e + s)] = {std::min(v[c0], v[c1]), std::max(v[c0], v[c1]), 0, 12 * e + s};
    }
  }
  const int64_t nedge = rank_keys(keys, enm);
  const int64_t ne = nx - 2;
  for (int64_t e = 0; e < nel; ++e)
    for (int s = 0; s < 12; ++s) {
      const int64_t igv = ngv + ne * (enm[(size_t)(12 * e + s)] - 1);
      const int b0 = s & 1, b1 = (s >> 1) & 1;
      // the edge's first corner, its step through the element, its last corner
      int64_t i0 = 0, j0 = 0, k0 = 0, di = 0, dj = 0, dk = 0;
      if (s < 4) {
        j0 = b0 * (nx - 1);
        k0 = b1 * (nx - 1);
        di = 1;
      } else if (s < 8) {
        i0 = b0 * (nx - 1);
        k0 = b1 * (nx - 1);
        dj = 1;
      } else {
        i0 = b0 * (nx - 1);
        j0 = b1 * (nx - 1);
        dk = 1;
      }
      const bool forward =
          G(e, i0, j0, k0) < G(e, i0 + di * (nx - 1), j0 + dj * (nx - 1), k0 + dk * (nx - 1));
      for (int64_t t = 1; t <= nx - 2; ++t)
        G(e, i0 + di * t, j0 + dj * t, k0 + dk * t) = forward ? igv + t : igv + 1 + ne - t;
    }
  ngv += nedge * ne;
  // ---- faces: ranked by their three smallest corner ids
  static const int fc[6][4] = {{0, 2, 4, 6}, {1, 3, 5, 7}, {0, 1, 4, 5},
                               {2, 3, 6, 7}, {0, 1, 2, 3}, {4, 5, 6, 7}};
  keys.assign((size_t)(6 * nel), Key{});
  std::vector<int64_t> fnm((size_t)(6 * nel));
  for (int64_t e = 0; e < nel; ++e)
    for (int f = 0; f < 6; ++f) {
      int64_t c[4];
      for (int q = 0; q < 4; ++q) c[q] = vertex[8 * e + fc[f][q]];
      std::sort(c, c + 4);
      keys[(size_t)(6 * e + f)] = {c[0], c[1], c[2], 6 * e + f};
    }
  const int64_t nface = rank_keys(keys, fnm);
  // A face's points as (i index, j index) over the 1-based linear point
  // numbering of the element: face f runs i from i0 to i1 by is and j from j0
  // to j1 by js, point = i + nx (j - 1) (the reference's skpdat, dsset).
  const int64_t sk[6][6] = {{1, nx * (nx - 1) + 1, nx, 1, nx * (nx - 1) + 1, nx},
                            {nx, nx * (nx - 1) + nx, nx, 1, nx * (nx - 1) + 1, nx},
                            {1, nx, 1, 1, nx * (nx - 1) + 1, nx},
                            {1 + nx * (nx - 1), nx * nx, 1, 1, nx * (nx - 1) + 1, nx},
                            {1, nx, 1, 1, nx, 1},
                            {1 + nxx * (nx - 1), nx + nxx * (nx - 1), 1, 1, nx, 1}};
  const int64_t nif = (nx - 2) * (nx - 2);
  for (int64_t e = 0; e < nel; ++e) {
    int64_t* ge = glo_num + nxyz * e - 1;  // 1-based point index
    for (int f = 0; f < 6; ++f) {
      int64_t i0 = sk[f][0], i1 = sk[f][1], is = sk[f][2], j0 = sk[f][3], j1 = sk[f][4], js = sk[f][5];
      const int64_t g[4] = {ge[i0 + nx * (j0 - 1)], ge[i1 + nx * (j0 - 1)], ge[i0 + nx * (j1 - 1)],
                            ge[i1 + nx * (j1 - 1)]};
      const int lo = (int)(std::min_element(g, g + 4) - g);
      // count from the smallest corner towards its smaller neighbour
      bool ij = false;
      int idir = 1, jdir = 1;
      switch (lo) {
        case 0: ij = g[1] < g[2]; break;
        case 1: idir = -1; ij = g[0] < g[3]; break;
        case 2: jdir = -1; ij = g[3] < g[0]; break;
        default: idir = jdir = -1; ij = g[2] < g[1]; break;
      }
      if (idir < 0) {
        std::swap(i0, i1);
        is = -is;
      }
      if (jdir < 0) {
        std::swap(j0, j1);
        js = -js;
      }
      const int64_t ig0 = ngv + nif * (fnm[(size_t)(6 * e + f)] - 1);
      const int64_t ni = (i1 - i0) / is + 1, nj = (j1 - j0) / js + 1;
      int64_t k = 0, l = 0;
      for (int64_t outer = 0; outer < (ij ? nj : ni); ++outer)
        for (int64_t inner = 0; inner < (ij ? ni : nj); ++inner) {
          const int64_t i = i0 + (ij ? inner : outer) * is, j = j0 + (ij ? outer : inner) * js;
          ++k;
          if (k > nx && k < nxx - nx && k % nx != 1 && k % nx != 0) ge[i + nx * (j - 1)] = ++l + ig0;
        }
    }
  }
  ngv += nface * nif;
  if (ngv_out) *ngv_out = ngv;
  return NEKGPU_OK;
}

}  // extern "C"

namespace {

// Interpolation weights at xx from the nodes x[0..n] (order 0 of Fornberg's
// recursion, as fd_weights_full, core/fast3d.f:1294, evaluates them).
void fd_weights0(double xx, const double* x, int n, double* c) {
  double c1 = 1.0, c4 = x[0] - xx;
  for (int j = 0; j <= n; ++j) c[j] = 0.0;
  c[0] = 1.0;
  for (int i = 1; i <= n; ++i) {
    double c2 = 1.0;
    const double c5 = c4;
    c4 = x[i] - xx;
    for (int j = 0; j < i; ++j) {
      const double c3 = x[i] - x[j];
      c2 = c2 * c3;
      c[i] = -(((c1 * c5) * c[i - 1]) / c2);
      c[j] = (c4 * c[j]) / c3;
    }
    c1 = c2;
  }
}

// v (nv^3) = (C x B x A) u (nu^3) with A[i][a] = wt[i*nu + a] for all three
// directions, as tensr3 (core/fasts.f:125): r, then s, then t, each an
// nu-term sum in order.
void tensor3(double* v, int nv, const double* u, int nu, const double* wt) {
  std::vector<double> t1((size_t)nv * nu * nu), t2((size_t)nv * nv * nu);
  for (int bc = 0; bc < nu * nu; ++bc)
    for (int i = 0; i < nv; ++i) {
      double s = wt[i * nu] * u[nu * bc];
      for (int a = 1; a < nu; ++a) s = s + wt[i * nu + a] * u[a + nu * bc];
      t1[(size_t)(i + nv * bc)] = s;
    }
  for (int c = 0; c < nu; ++c)
    for (int j = 0; j < nv; ++j)
      for (int i = 0; i < nv; ++i) {
        double s = t1[(size_t)(i + nv * (nu * c))] * wt[j * nu];
        for (int b = 1; b < nu; ++b) s = s + t1[(size_t)(i + nv * (b + nu * c))] * wt[j * nu + b];
        t2[(size_t)(i + nv * (j + nv * c))] = s;
      }
  for (int k = 0; k < nv; ++k)
    for (int j = 0; j < nv; ++j)
      for (int i = 0; i < nv; ++i) {
        double s = t2[(size_t)(i + nv * j)] * wt[k * nu];
        for (int c = 1; c < nu; ++c) s = s + t2[(size_t)(i + nv * (j + nv * c))] * wt[k * nu + c];
        v[i + nv * (j + nv * k)] = s;
      }
}

// Gordon-Hall extension of a 3x3x3 array from its vertices and edges
// (gh_face_extend_3d, core/navier5.f:2502, gh_type 2) at nodes -1, 0, 1.
void gordon_hall_edges3(double* x) {
  constexpr int n = 3;
  const double zg[3] = {-1.0, 0.0, 1.0};
  auto at = [](int i, int j, int k) { return i + n * (j + n * k); };
  auto lin = [&](int end, int i) {  // 0.5 ((n-end)(1-z) + (end-1)(1+z)) / (n-1), end 1 or n
    return 0.5 * ((double)(n - end) * (1.0 - zg[i]) + (double)(end - 1) * (1.0 + zg[i])) / (double)(n - 1);
  };
  double v[27] = {0}, e[27] = {0};
  for (int kk = 1; kk <= n; kk += n - 1)
    for (int jj = 1; jj <= n; jj += n - 1)
      for (int ii = 1; ii <= n; ii += n - 1)
        for (int k = 0; k < n; ++k)
          for (int j = 0; j < n; ++j)
            for (int i = 0; i < n; ++i)
              v[at(i, j, k)] = v[at(i, j, k)] +
                               lin(ii, i) * lin(jj, j) * lin(kk, k) * x[at(ii - 1, jj - 1, kk - 1)];
  for (int kk = 1; kk <= n; kk += n - 1)  // x-edges
    for (int jj = 1; jj <= n; jj += n - 1)
      for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j)
          for (int i = 0; i < n; ++i)
            e[at(i, j, k)] = e[at(i, j, k)] + lin(jj, j) * lin(kk, k) *
                                                  (x[at(i, jj - 1, kk - 1)] - v[at(i, jj - 1, kk - 1)]);
  for (int kk = 1; kk <= n; kk += n - 1)  // y-edges
    for (int ii = 1; ii <= n; ii += n - 1)
      for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j)
          for (int i = 0; i < n; ++i)
            e[at(i, j, k)] = e[at(i, j, k)] + lin(ii, i) * lin(kk, k) *
                                                  (x[at(ii - 1, j, kk - 1)] - v[at(ii - 1, j, kk - 1)]);
  for (int jj = 1; jj <= n; jj += n - 1)  // z-edges
    for (int ii = 1; ii <= n; ii += n - 1)
      for (int k = 0; k < n; ++k)
        for (int j = 0; j < n; ++j)
          for (int i = 0; i < n; ++i)
            e[at(i, j, k)] = e[at(i, j, k)] + lin(ii, i) * lin(jj, j) *
                                                  (x[at(ii - 1, jj - 1, k)] - v[at(ii - 1, jj - 1, k)]);
  for (int q = 0; q < 27; ++q) x[q] = e[q] + v[q];
}

// Midside node of each preprocessor edge (1..12) in the 3x3x3 array.
constexpr int kEdgeMid[12] = {1, 5, 7, 3, 19, 23, 25, 21, 9, 11, 17, 15};

// sphsrf (core/genxyz.f:677-842): face ifce (1..6, preprocessor order) of an
// element made a patch of the sphere of the given centre and radius: the
// face's four edges become great-circle arcs (edg3d :844), the interior
// points the normalised crossings of the arcs through opposite edge points,
// then the face's deflection is spread linearly from the opposite face.
// xc, yc, zc: the element's corners (file order); x, y, z its GLL
// coordinates.  Returns false when a corner is not on the sphere or the
// radius is not positive (crn3d :929-1021).
bool sphere_face(int nx, const double* zg, const double* xc, const double* yc, const double* zc,
                 int ifce, const double* cv, double* x, double* y, double* z) {
  const double ctr[3] = {cv[0], cv[1], cv[2]}, radius = cv[3];
  if (!(radius > 0.0)) return false;
  const int iface = kTensorFace[ifce - 1];  // eface1
  // corners of the face (crn3d: indvtx, tensor numbering, to file order)
  static const int indvtx[6][4] = {{1, 5, 3, 7}, {2, 4, 6, 8}, {1, 2, 5, 6},
                                   {3, 7, 4, 8}, {1, 3, 2, 4}, {5, 6, 7, 8}};
  double xcv[4][3];
  for (int i = 0; i < 4; ++i) {
    const int k = kPreOfTensor[indvtx[iface - 1][i] - 1];
    xcv[i][0] = xc[k] - ctr[0];
    xcv[i][1] = yc[k] - ctr[1];
    xcv[i][2] = zc[k] - ctr[2];
    const double radt = std::sqrt(xcv[i][0] * xcv[i][0] + xcv[i][1] * xcv[i][1] +
                                  xcv[i][2] * xcv[i][2]);
    if (std::fabs(radt - radius) / radius > 1e-4) return false;
  }
  auto dot = [](const double* a, const double* b) {
    double s = 0.0;
    for (int k = 0; k < 3; ++k) s = s + a[k] * b[k];
    return s;
  };
  auto cross = [](double* v1, const double* v2, const double* v3) {
    v1[0] = v2[1] * v3[2] - v2[2] * v3[1];
    v1[1] = v2[2] * v3[0] - v2[0] * v3[2];
    v1[2] = v2[0] * v3[1] - v2[1] * v3[0];
  };
  auto norm3 = [&](double* v) {
    const double l = std::sqrt(dot(v, v));
    if (l > 0) {
      v[0] = v[0] / l;
      v[1] = v[1] / l;
      v[2] = v[2] / l;
    }
  };
  std::vector<double> srf((size_t)3 * nx * nx);  // srf(3, nx, nx), (i, j)
  auto S = [&](int i, int j) { return &srf[(size_t)3 * (i + nx * j)]; };
  // edg3d: the great-circle arc from x1 to x2 at the GLL nodes
  auto edge = [&](const double* x1, const double* x2, int i1, int i2, int j1, int j2) {
    double u1[3] = {x1[0], x1[1], x1[2]}, u2[3] = {x2[0], x2[1], x2[2]}, vn[3], b[3];
    norm3(u1);
    norm3(u2);
    cross(vn, x1, x2);
    cross(b, vn, x1);
    norm3(vn);
    norm3(b);
    const double theta = std::acos(dot(u1, u2));
    int ij = 0;
    for (int j = j1; j <= j2; ++j)
      for (int i = i1; i <= i2; ++i, ++ij) {
        const double tp = 0.5 * theta * (zg[ij] + 1.0);
        const double ct = std::cos(tp), st = std::sin(tp);
        for (int v = 0; v < 3; ++v) S(i, j)[v] = ct * u1[v] + st * b[v];
      }
  };
  // xcv(3,2,2): corner (a, b) is xcv[a + 2 b]
  edge(xcv[0], xcv[2], 0, 0, 0, nx - 1);
  edge(xcv[1], xcv[3], nx - 1, nx - 1, 0, nx - 1);
  edge(xcv[0], xcv[1], 0, nx - 1, 0, 0);
  edge(xcv[2], xcv[3], 0, nx - 1, nx - 1, nx - 1);
  // sign of the curvature from a face corner and the corner opposite it
  static const int cface[6][2] = {{1, 4}, {2, 1}, {3, 2}, {4, 3}, {1, 5}, {5, 1}};
  const int iv = cface[ifce - 1][0] - 1, io = cface[ifce - 1][1] - 1;
  const double vout[3] = {xc[iv] - xc[io], yc[iv] - yc[io], zc[iv] - zc[io]};
  const double vsph[3] = {xc[iv] - ctr[0], yc[iv] - ctr[1], zc[iv] - ctr[2]};
  const bool concave = !(dot(vsph, vout) > 0);
  for (int j = 1; j < nx - 1; ++j) {
    double vn1[3], vn2[3];
    cross(vn1, S(0, j), S(nx - 1, j));
    for (int i = 1; i < nx - 1; ++i) {
      cross(vn2, S(i, 0), S(i, nx - 1));
      if (concave) cross(S(i, j), vn2, vn1);
      else cross(S(i, j), vn1, vn2);
    }
  }
  for (int q = 0; q < nx * nx; ++q) norm3(&srf[(size_t)3 * q]);
  for (double& v : srf) v = v * radius;
  for (int q = 0; q < nx * nx; ++q)
    for (int v = 0; v < 3; ++v) srf[(size_t)3 * q + v] = srf[(size_t)3 * q + v] + ctr[v];
  if (iface == 1 || iface == 4 || iface == 5)  // transpose
    for (int j = 0; j < nx; ++j)
      for (int i = j + 1; i < nx; ++i)
        for (int v = 0; v < 3; ++v) std::swap(S(i, j)[v], S(j, i)[v]);
  // the face's deflection, spread linearly from the opposite face
  const int64_t NX = nx, NXX = (int64_t)nx * nx;
  const int64_t sk[6][6] = {{1, NX * (NX - 1) + 1, NX, 1, NX * (NX - 1) + 1, NX},
                            {NX, NX * (NX - 1) + NX, NX, 1, NX * (NX - 1) + 1, NX},
                            {1, NX, 1, 1, NX * (NX - 1) + 1, NX},
                            {1 + NX * (NX - 1), NXX, 1, 1, NX * (NX - 1) + 1, NX},
                            {1, NX, 1, 1, NX, 1},
                            {1 + NXX * (NX - 1), NX + NXX * (NX - 1), 1, 1, NX, 1}};
  const int64_t* d = sk[iface - 1];
  const int64_t iopp[3] = {NX - 1, NX * (NX - 1), NXX * (NX - 1)};
  const int idir = 2 * (iface % 2) - 1, ifc2 = (iface + 1) / 2;
  double* c3[3] = {x, y, z};
  int q = 0;
  for (int64_t j2 = d[3]; d[5] > 0 ? j2 <= d[4] : j2 >= d[4]; j2 += d[5])
    for (int64_t j1 = d[0]; d[2] > 0 ? j1 <= d[1] : j1 >= d[1]; j1 += d[2], ++q) {
      const int64_t jopp = j1 + iopp[ifc2 - 1] * idir;
      const int64_t face_pt = j1 - 1 + NX * (j2 - 1);
      double dx[3];
      for (int v = 0; v < 3; ++v) dx[v] = srf[(size_t)3 * q + v] - c3[v][face_pt];
      const int64_t joff = (j1 - jopp) / (NX - 1);
      for (int ix = 2; ix <= nx; ++ix) {
        const int64_t jj = jopp + joff * (ix - 1);
        const double zeta = 0.5 * (zg[ix - 1] + 1.0);
        const int64_t pt = jj - 1 + NX * (j2 - 1);
        for (int v = 0; v < 3; ++v) c3[v][pt] = c3[v][pt] + dx[v] * zeta;
      }
    }
  return true;
}

// arcsrf (core/genxyz.f:2-101): edge isid (1..8, in a face of constant t)
// of an element bent into a circular arc of the given radius in the x-y
// plane (positive: centre on the element's side), the bend blended linearly
// across the element.  xc, yc: the element's 8 corners (file order); x, y its
// GLL coordinates (nx^3).  Returns false when the radius is shorter than half
// the chord.
bool arc_edge(int nx, const double* zg, const double* xc, const double* yc, int isid,
              double radius, double* x, double* y) {
  const int c1 = isid - 1, c2 = isid == 4 ? 0 : isid == 8 ? 4 : isid;
  const double p1x = xc[c1], p1y = yc[c1], p2x = xc[c2], p2y = yc[c2];
  const double gap = std::sqrt((p1x - p2x) * (p1x - p2x) + (p1y - p2y) * (p1y - p2y));
  if (std::fabs(2.0 * radius) <= gap * 1.00001) return false;
  const double xs = p2y - p1y, ys = p1x - p2x;
  const double xys = std::sqrt(xs * xs + ys * ys);
  const double dtheta = std::fabs(std::asin(0.5 * gap / radius));
  const double p12x = (p1x + p2x) / 2.0, p12y = (p1y + p2y) / 2.0;
  const double xcen = p12x - xs / xys * radius * std::cos(dtheta);
  const double ycen = p12y - ys / xys * radius * std::cos(dtheta);
  const double theta0 = std::atan2(p12y - ycen, p12x - xcen);
  // the bend along the edge, in the edge's r (or s) order
  const int side = (isid - 1) % 4 + 1;  // mod1(isid, 4)
  std::vector<double> bx((size_t)nx), by((size_t)nx), h0((size_t)nx), h1((size_t)nx);
  for (int i = 0; i < nx; ++i) {
    h0[(size_t)i] = (1.0 - zg[i]) * 0.5;
    h1[(size_t)i] = (1.0 + zg[i]) * 0.5;
  }
  for (int ix = 0; ix < nx; ++ix) {
    const int it = side > 2 ? nx - 1 - ix : ix;
    const double r = radius < 0.0 ? -zg[ix] : zg[ix];
    bx[(size_t)it] = xcen + std::fabs(radius) * std::cos(theta0 + r * dtheta) -
                     (h0[(size_t)ix] * p1x + h1[(size_t)ix] * p2x);
    by[(size_t)it] = ycen + std::fabs(radius) * std::sin(theta0 + r * dtheta) -
                     (h0[(size_t)ix] * p1y + h1[(size_t)ix] * p2y);
  }
  // tensor face of the edge (eface1: 3, 2, 4, 1): r- / r+ faces carry a bend
  // along s, s- / s+ faces a bend along r; blended in t by the edge's level
  const int tf = kTensorFace[side - 1];  // 1..4
  const std::vector<double>& hz = (isid - 1) / 4 == 0 ? h0 : h1;
  for (int k = 0; k < nx; ++k)
    for (int j = 0; j < nx; ++j)
      for (int i = 0; i < nx; ++i) {
        const size_t q = (size_t)(i + nx * (j + nx * k));
        if (tf <= 2) {  // addtnsr(x, H(:,1,tf), bend, H(:,3,izt))
          const double hh = bx[(size_t)j] * hz[(size_t)k], hy = by[(size_t)j] * hz[(size_t)k];
          const double hr = tf == 1 ? h0[(size_t)i] : h1[(size_t)i];
          x[q] = x[q] + hh * hr;
          y[q] = y[q] + hy * hr;
        } else {  // addtnsr(x, bend, H(:,2,tf-2), H(:,3,izt))
          const double hh = (tf == 3 ? h0[(size_t)j] : h1[(size_t)j]) * hz[(size_t)k];
          x[q] = x[q] + hh * bx[(size_t)i];
          y[q] = y[q] + hh * by[(size_t)i];
        }
      }
  return true;
}

}  // namespace

extern "C" {

int nekmesh_genxyz(const int* nx_, const int* nel_, const double* zg, const double* xc,
                   const double* yc, const double* zc, const int64_t* ncurve, const int* elem,
                   const int* side, const double* curve, const char* ccurve, double* x, double* y,
                   double* z) {
  if (!nx_ || !nel_ || !zg || !xc || !yc || !zc || !x || !y || !z || *nx_ < 2 || *nel_ <= 0 ||
      (ncurve && *ncurve > 0 && (!elem || !side || !curve || !ccurve)))
    return fail(NEKGPU_EINVAL, "genxyz: bad arguments");
  const int nx = *nx_;
  const int64_t nel = *nel_, nxyz = (int64_t)nx * nx * nx, nc = ncurve ? *ncurve : 0;
  // midside nodes per element (edges 1..12); any other curve type is refused
  std::vector<int64_t> first((size_t)nel, -1);
  std::vector<std::array<int, 12>> mid;
  std::vector<int64_t> arcs;  // records of circular-arc edges
  for (int64_t q = 0; q < nc; ++q) {
    const int64_t e = elem[q] - 1;
    if (e < 0 || e >= nel) return fail(NEKGPU_EINVAL, "genxyz: curve record names no element");
    if (ccurve[q] == ' ' || ccurve[q] == '\0') continue;
    if (ccurve[q] == 'C') {
      if (side[q] < 1 || side[q] > 12) return fail(NEKGPU_EINVAL, "genxyz: arc on no edge");
      if (side[q] <= 8) arcs.push_back(q);  // the reference bends edges 1..8 only
      continue;
    }
    if (ccurve[q] == 's') {
      if (side[q] < 1 || side[q] > 6) return fail(NEKGPU_EINVAL, "genxyz: sphere on no face");
      arcs.push_back(q);  // applied with the arcs, faces first
      continue;
    }
    if (ccurve[q] != 'm')
      return fail(NEKGPU_EINVAL, std::string("genxyz: curved side type '") + ccurve[q] +
                                     "' not served (midside nodes 'm', arcs 'C', spheres 's' are)");
    if (side[q] < 1 || side[q] > 12) return fail(NEKGPU_EINVAL, "genxyz: midside node on no edge");
    if (first[(size_t)e] < 0) {
      first[(size_t)e] = (int64_t)mid.size();
      std::array<int, 12> none;
      none.fill(-1);
      mid.push_back(none);
    }
    mid[(size_t)first[(size_t)e]][side[q] - 1] = (int)q;
  }
  // straight-sided elements (and every element when nx = 2, as linquad)
  int rc = nekmesh_xyzlin(nx_, nel_, zg, xc, yc, zc, x, y, z);
  if (rc) return rc;
  if (nx == 2 && arcs.empty()) return NEKGPU_OK;
  // quadratic elements (xyzquad, core/genxyz.f:1334): the trilinear 3x3x3
  // map, the file's midside nodes on their edges, edges extended inward by
  // Gordon-Hall, then the quadratic interpolant at the GLL nodes
  const double zq[3] = {-1.0, 0.0, 1.0};
  std::vector<double> wq((size_t)nx * 3);
  for (int i = 0; i < nx; ++i) fd_weights0(zg[i], zq, 2, &wq[(size_t)i * 3]);
  const double* src[3] = {xc, yc, zc};
  double* dst[3] = {x, y, z};
  const double wl[6] = {1.0, 0.0, 0.5, 0.5, 0.0, 1.0};  // (1-z)/2, (1+z)/2 at -1, 0, 1
  for (int64_t e = 0; e < nel && nx > 2; ++e) {
    if (first[(size_t)e] < 0) continue;
    const auto& m = mid[(size_t)first[(size_t)e]];
    for (int d = 0; d < 3; ++d) {
      double u[8], q3[27];
      for (int c = 0; c < 8; ++c) u[c] = src[d][8 * e + kPreOfTensor[c]];
      tensor3(q3, 3, u, 2, wl);
      for (int k = 0; k < 12; ++k)
        if (m[k] >= 0) q3[kEdgeMid[k]] = curve[5 * (size_t)m[k] + d];
      gordon_hall_edges3(q3);
      tensor3(dst[d] + nxyz * e, nx, q3, 3, wq.data());
    }
  }
  // spherical faces, then circular-arc edges, after the linear / quadratic
  // map, element by element, faces and edges in order (genxyz's order)
  auto rank = [&](int64_t q) { return (ccurve[q] == 's' ? 0 : 100) + side[q]; };
  std::stable_sort(arcs.begin(), arcs.end(), [&](int64_t a, int64_t b) {
    return elem[a] != elem[b] ? elem[a] < elem[b] : rank(a) < rank(b);
  });
  for (const int64_t q : arcs) {
    const int64_t e = elem[q] - 1;
    if (ccurve[q] == 's') {
      if (!sphere_face(nx, zg, xc + 8 * e, yc + 8 * e, zc + 8 * e, side[q], curve + 5 * (size_t)q,
                       x + nxyz * e, y + nxyz * e, z + nxyz * e))
        return fail(NEKGPU_EINVAL, "genxyz: element " + std::to_string(e + 1) + " face " +
                                       std::to_string(side[q]) +
                                       ": corner not on its sphere, or radius not positive");
      continue;
    }
    if (!arc_edge(nx, zg, xc + 8 * e, yc + 8 * e, side[q], curve[5 * (size_t)q], x + nxyz * e,
                  y + nxyz * e))
      return fail(NEKGPU_EINVAL, "genxyz: arc radius shorter than half its chord (element " +
                                     std::to_string(e + 1) + ", edge " + std::to_string(side[q]) + ")");
  }
  return NEKGPU_OK;
}

int nekmesh_check_p_bc(const int* nx_, const int* nel_, const char* cbc, int64_t* glo_num) {
  if (!nx_ || !nel_ || !cbc || !glo_num || *nx_ < 2 || *nel_ <= 0)
    return fail(NEKGPU_EINVAL, "check_p_bc: bad arguments");
  const int64_t nx = *nx_, nel = *nel_, nxyz = nx * nx * nx;
  for (int64_t e = 0; e < nel; ++e)
    for (int dir = 0; dir < 3; ++dir) {  // tensor faces 2 dir and 2 dir + 1
      const char* a = cbc + 3 * (6 * e + kPreFace[2 * dir] - 1);
      const char* b = cbc + 3 * (6 * e + kPreFace[2 * dir + 1] - 1);
      if (std::memcmp(a, "p  ", 3) != 0 || std::memcmp(b, "p  ", 3) != 0) continue;
      int64_t* g = glo_num + nxyz * e;
      const int64_t st = dir == 0 ? 1 : dir == 1 ? nx : nx * nx;  // step across the element
      for (int64_t v = 0; v < nx; ++v)
        for (int64_t u = 0; u < nx; ++u) {
          // the point (u, v) of the face pair: the other two indices
          int64_t i0;
          if (dir == 0) i0 = nx * (u + nx * v);
          else if (dir == 1) i0 = u + nx * nx * v;
          else i0 = u + nx * v;
          const int64_t lo = i0, hi = i0 + (nx - 1) * st;
          const int64_t m = std::min(g[lo], g[hi]);
          g[lo] = m;
          g[hi] = m;
        }
    }
  return NEKGPU_OK;
}

int nekmesh_xyzlin(const int* nx_, const int* nel_, const double* zg, const double* xc,
                   const double* yc, const double* zc, double* x, double* y, double* z) {
  if (!nx_ || !nel_ || !zg || !xc || !yc || !zc || !x || !y || !z || *nx_ < 2 || *nel_ <= 0)
    return fail(NEKGPU_EINVAL, "xyzlin: bad arguments");
  const int nx = *nx_;
  const int64_t nel = *nel_, nxyz = (int64_t)nx * nx * nx;
  // linear interpolation weights at the nodes: (1 - z)/2 and (1 + z)/2
  std::vector<double> h0((size_t)nx), h1((size_t)nx);
  for (int i = 0; i < nx; ++i) {
    h0[(size_t)i] = (1.0 - zg[i]) / 2.0;
    h1[(size_t)i] = (1.0 + zg[i]) / 2.0;
  }
  const double* src[3] = {xc, yc, zc};
  double* dst[3] = {x, y, z};
  std::vector<double> t1((size_t)nx * 4), t2((size_t)nx * nx * 2);
  for (int64_t e = 0; e < nel; ++e)
    for (int d = 0; d < 3; ++d) {
      double u[8];  // tensor order
      for (int c = 0; c < 8; ++c) u[c] = src[d][8 * e + kPreOfTensor[c]];
      // r, then s, then t (each a two-term sum)
      for (int bc = 0; bc < 4; ++bc)
        for (int i = 0; i < nx; ++i)
          t1[(size_t)(i + nx * bc)] = h0[(size_t)i] * u[2 * bc] + h1[(size_t)i] * u[2 * bc + 1];
      for (int c = 0; c < 2; ++c)
        for (int j = 0; j < nx; ++j)
          for (int i = 0; i < nx; ++i)
            t2[(size_t)(i + nx * (j + nx * c))] =
                t1[(size_t)(i + nx * (2 * c))] * h0[(size_t)j] + t1[(size_t)(i + nx * (2 * c + 1))] * h1[(size_t)j];
      double* out = dst[d] + nxyz * e;
      for (int k = 0; k < nx; ++k)
        for (int j = 0; j < nx; ++j)
          for (int i = 0; i < nx; ++i)
            out[i + nx * (j + nx * k)] = t2[(size_t)(i + nx * j)] * h0[(size_t)k] +
                                         t2[(size_t)(i + nx * (j + nx))] * h1[(size_t)k];
    }
  return NEKGPU_OK;
}

}  // extern "C"
