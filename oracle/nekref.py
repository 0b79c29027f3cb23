"""ctypes front end of the CPU oracle (oracle/nekref.c).

TEST INFRASTRUCTURE ONLY.  The parity tests, ``__graft_entry__.smoke()`` and
the CPU-baseline leg of ``bench.py`` import this module as the checker / the
timed CPU restatement of the reference.  The product package
(``nek5000_gb300``) never imports it.

Every routine mirrors one reference routine; see nekref.c for the file:line
citations.  Arrays are numpy float64 / int64 in the reference's element-major
layout (lx1, ly1, lz1, nel) flattened with x fastest.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libnekref.so")
_lock = threading.Lock()
_lib = None

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_ip = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_vp = C.c_void_p


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP, -ffp-contract=off)."""
    srcs = [os.path.join(_HERE, f) for f in ("nekref.c", "h1mg.c", "gradops.c", "nekref.h",
                                              "Makefile")]
    if force or not os.path.exists(_LIB_PATH) or \
            os.path.getmtime(_LIB_PATH) < max(os.path.getmtime(f) for f in srcs):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_LIB_PATH)
            L.ref_zwgll.argtypes = [_dp, _dp, C.c_int]
            L.ref_dgll.argtypes = [_dp, _dp, _dp, C.c_int]
            L.ref_box_mesh.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                       C.c_double, _dp, _dp, _dp, _dp, _ip]
            L.ref_geom.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp]
            L.ref_setvert3d.argtypes = [_ip, C.POINTER(C.c_int64), C.c_int, C.c_int, _ip]
            L.ref_gs_setup.argtypes = [_ip, C.c_int64]
            L.ref_gs_setup.restype = _vp
            L.ref_gs_free.argtypes = [_vp]
            L.ref_gs_op.argtypes = [_vp, _dp, C.c_int]
            L.ref_gs_nseg.argtypes = [_vp]
            L.ref_gs_nseg.restype = C.c_int64
            L.ref_gs_nidx.argtypes = [_vp]
            L.ref_gs_nidx.restype = C.c_int64
            L.ref_gs_maps.argtypes = [_vp, _ip, _ip, _ip]
            L.ref_ops_create.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _dp, _ip, C.c_int]
            _i32 = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
            L.ref_h1mg_create.argtypes = [_vp, _dp, _dp, _dp, _i32, _ip, C.c_int]
            L.ref_h1mg_create.restype = _vp
            L.ref_h1mg_free.argtypes = [_vp]
            L.ref_h1mg_solve.argtypes = [_vp, _dp, _dp]
            L.ref_h1mg_nlev.argtypes = [_vp]
            L.ref_h1mg_nx.argtypes = [_vp, C.c_int]
            L.ref_h1mg_ncoarse.argtypes = [_vp]
            L.ref_h1mg_ncoarse.restype = C.c_int64
            L.ref_h1mg_level.argtypes = [_vp, C.c_int, _vp, _vp, _vp]
            L.ref_h1mg_schwarz.argtypes = [_vp, C.c_int, _dp, _dp]
            L.ref_h1mg_coarse.argtypes = [_vp, _dp, _dp]
            L.ref_h1mg_levels.argtypes = [C.c_int, _i32]
            L.ref_h1mg_lengths.argtypes = [_vp, _dp]
            L.ref_geom_rst.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
            L.ref_wgradm1.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp]
            L.ref_cdtp.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _dp, _dp, C.c_int]
            L.ref_dudxyz.argtypes = [C.c_int, C.c_int, _dp, _dp, _dp, _dp, C.c_int]
            L.ref_op_curl.argtypes = [_vp, _dp, _dp, _dp, _dp, _dp, _dp, C.c_int, _dp, _dp, _dp,
                                      _dp]
            L.ref_conv1.argtypes = [C.c_int, C.c_int] + [_dp] * 7
            L.ref_advab.argtypes = [C.c_int, C.c_int] + [_dp] * 9
            L.ref_makeabf.argtypes = [C.c_int64, _dp, _dp, _dp, _dp, _dp]
            L.ref_makebdf.argtypes = [C.c_int64, _dp, _dp, _dp, _dp, _dp, _dp, C.c_int,
                                      C.c_double]
            L.ref_sumab.argtypes = [C.c_int64, _dp, _dp, _dp, _dp, C.c_int]
            L.ref_convect_new.argtypes = [C.c_int, C.c_int, C.c_int] + [_dp] * 7
            L.ref_convect_cons.argtypes = [C.c_int, C.c_int, C.c_int] + [_dp] * 7
            L.ref_conv2.argtypes = [C.c_int, C.c_int] + [_dp] * 7
            L.ref_convopo.argtypes = [C.c_int, C.c_int] + [_dp] * 8 + [_vp]
            L.ref_cresvsp.argtypes = [_vp] + [_dp] * 15
            L.ref_cresvsp_weak.argtypes = [_vp] + [_dp] * 17 + [C.c_int]
            L.ref_axsf.argtypes = [_vp] + [_dp] * 11
            L.ref_hmhzsf.argtypes = [_vp] + [_dp] * 16 + [C.c_double, C.c_double,
                                                           C.POINTER(C.c_double),
                                                           C.POINTER(C.c_double)]
            L.ref_hmhzsf.restype = C.c_int
            L.ref_crespsp.argtypes = [_vp] + [_dp] * 13 + [C.c_double, C.c_int, _dp, _dp, _dp, _dp,
                                                           _dp, _vp, _dp]
            L.ref_fdm1d.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                    _dp, _dp]
            L.ref_gmres_h1mg.argtypes = [_vp, _vp, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_int,
                                         C.c_int, C.c_int, C.POINTER(C.c_double),
                                         C.POINTER(C.c_double)]
            L.ref_flex_cg_h1mg.argtypes = [_vp, _vp, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_int,
                                           C.c_int, C.POINTER(C.c_double),
                                           C.POINTER(C.c_double)]
            L.ref_ops_create.restype = _vp
            L.ref_ops_free.argtypes = [_vp]
            L.ref_ops_gs.argtypes = [_vp]
            L.ref_ops_gs.restype = _vp
            L.ref_axhelm.argtypes = [_vp, _dp, _dp, _dp, _dp]
            L.ref_dssum.argtypes = [_vp, _dp]
            L.ref_dsop.argtypes = [_vp, _dp, C.c_int]
            L.ref_setprec.argtypes = [_vp, _dp, _dp, _dp]
            L.ref_setprec_local.argtypes = [_vp, _dp, _dp, _dp]
            L.ref_glsc3.argtypes = [_vp, _dp, _dp, _dp]
            L.ref_glsc3.restype = C.c_double
            L.ref_chktcg1.argtypes = [_vp, C.POINTER(C.c_double), _dp, _dp, _dp, _dp, _dp, _dp]
            L.ref_cggo.argtypes = [_vp, _dp, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_int, C.c_int,
                                   C.c_int, _dp, C.POINTER(C.c_double), C.POINTER(C.c_double)]
            L.ref_cggo.restype = C.c_int
            L.ref_hmholtz.argtypes = [_vp, _dp, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_int,
                                      C.c_int, C.c_int, _dp, C.POINTER(C.c_double),
                                      C.POINTER(C.c_double)]
            L.ref_hmholtz.restype = C.c_int
            L.ref_proj_create.argtypes = [_vp, C.c_int]
            L.ref_proj_create.restype = _vp
            L.ref_proj_free.argtypes = [_vp]
            L.ref_proj_m.argtypes = [_vp]
            L.ref_proj_m.restype = C.c_int
            L.ref_proj_x.argtypes = [_vp, C.c_int]
            L.ref_proj_x.restype = C.POINTER(C.c_double)
            L.ref_proj_b.argtypes = [_vp, C.c_int]
            L.ref_proj_b.restype = C.POINTER(C.c_double)
            L.ref_hsolve.argtypes = [_vp, _vp, _dp, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_int,
                                     C.c_int, C.c_int, _dp, C.POINTER(C.c_double),
                                     C.POINTER(C.c_double)]
            L.ref_hsolve.restype = C.c_int
            L.ref_gmres.argtypes = [_vp, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_int, C.c_int,
                                    C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
            L.ref_gmres.restype = C.c_int
            L.ref_flex_cg.argtypes = [_vp, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_int, C.c_int,
                                      C.POINTER(C.c_double), C.POINTER(C.c_double)]
            L.ref_flex_cg.restype = C.c_int
            L.ref_local_grad3.argtypes = [_dp, _dp, _dp, _dp, C.c_int, _dp, _dp]
            L.ref_local_grad3_t.argtypes = [_dp, _dp, _dp, _dp, C.c_int, _dp, _dp, _dp]
            L.ref_mxm.argtypes = [_dp, C.c_int, _dp, C.c_int, _dp, C.c_int]
            L.ref_max_threads.restype = C.c_int
            _lib = L
    return _lib


def _c(a, dt=np.float64):
    return np.ascontiguousarray(a, dtype=dt)


# ---- spectral library -------------------------------------------------------
def zwgll(np_: int):
    z = np.zeros(np_)
    w = np.zeros(np_)
    lib().ref_zwgll(z, w, np_)
    return z, w


def dgll(z):
    nz = len(z)
    d = np.zeros(nz * nz)
    dt = np.zeros(nz * nz)
    lib().ref_dgll(d, dt, _c(z), nz)
    # Fortran D(i,j) = d[i + j*nz]  ->  numpy D[i, j]
    return d.reshape(nz, nz).T.copy(), dt.reshape(nz, nz).T.copy()


def mxm(a, b):
    """C = A B with the reference's mxf<n> left-to-right sums (2-D numpy in)."""
    n1, n2 = a.shape
    n3 = b.shape[1]
    c = np.zeros(n1 * n3)
    lib().ref_mxm(_c(a.T.ravel()), n1, _c(b.T.ravel()), n2, c, n3)
    return c.reshape(n3, n1).T


# ---- mesh / geometry / numbering -------------------------------------------
def box_mesh(nx1, kx, ky, kz, periodic=(False, False, False), amp=0.05, v=(0.0, 0.0, 1.0)):
    nel = kx * ky * kz
    n = nx1 ** 3 * nel
    x = np.zeros(n)
    y = np.zeros(n)
    z = np.zeros(n)
    vert = np.zeros(8 * nel, dtype=np.int64)
    if periodic[0]:
        raise ValueError("periodic x is not supported by the box mesher")
    lib().ref_box_mesh(nx1, kx, ky, kz, int(periodic[1]), int(periodic[2]), float(amp),
                       _c(v), x, y, z, vert)
    return x, y, z, vert


def geom(nx1, nel, x, y, z):
    n = nx1 ** 3 * nel
    g = np.zeros(6 * n)
    bm1 = np.zeros(n)
    jac = np.zeros(n)
    lib().ref_geom(nx1, nel, _c(x), _c(y), _c(z), g, bm1, jac)
    return g.reshape(6, n), bm1, jac


def setvert3d(nx, nel, vertex):
    glo = np.zeros(nx ** 3 * nel, dtype=np.int64)
    ngv = C.c_int64(0)
    lib().ref_setvert3d(glo, C.byref(ngv), nx, nel, _c(vertex, np.int64))
    return glo, int(ngv.value)


class GS:
    """gs_setup / gs_op semantics; maps exported for bit-exact comparison."""

    def __init__(self, glo_num):
        self._glo = _c(glo_num, np.int64)
        self.h = lib().ref_gs_setup(self._glo, len(self._glo))

    def op(self, u, op="+"):
        lib().ref_gs_op(self.h, u, {"+": 0, "*": 1, "M": 2, "m": 3}[op])

    def maps(self):
        L = lib()
        ns, ni = L.ref_gs_nseg(self.h), L.ref_gs_nidx(self.h)
        start = np.zeros(ns + 1, dtype=np.int64)
        idx = np.zeros(max(ni, 1), dtype=np.int64)
        ids = np.zeros(max(ns, 1), dtype=np.int64)
        L.ref_gs_maps(self.h, start, idx, ids)
        return start, idx[:ni], ids[:ns]

    def __del__(self):
        try:
            lib().ref_gs_free(self.h)
        except Exception:
            pass


class Ops:
    """Operator state for axhelm / dssum / setprec / cggo (borrowed arrays kept alive)."""

    def __init__(self, nx1, nel, D, g, bm1, glo_num, nthreads=1):
        self.nx1, self.nel = nx1, nel
        self.n = nx1 ** 3 * nel
        self._d = _c(D.T.ravel())      # Fortran order D(i,j) at [i + j*nx]
        self._dt = _c(D.ravel())       # D^T in Fortran order
        self._g = _c(g.reshape(-1))
        self._bm1 = _c(bm1)
        self._glo = _c(glo_num, np.int64)
        self.nthreads = nthreads
        self.h = lib().ref_ops_create(nx1, nel, self._d, self._dt, self._g, self._bm1, self._glo,
                                      int(nthreads))

    def __del__(self):
        try:
            lib().ref_ops_free(self.h)
        except Exception:
            pass

    def axhelm(self, u, h1, h2):
        au = np.zeros(self.n)
        lib().ref_axhelm(self.h, au, _c(u), _c(h1), _c(h2))
        return au

    def dssum(self, u):
        u = np.array(u, dtype=np.float64, copy=True)
        lib().ref_dssum(self.h, u)
        return u

    def dsop(self, u, op):
        u = np.array(u, dtype=np.float64, copy=True)
        lib().ref_dsop(self.h, u, {"+": 0, "*": 1, "M": 2, "m": 3}[op])
        return u

    def setprec(self, h1, h2):
        d = np.zeros(self.n)
        lib().ref_setprec(self.h, d, _c(h1), _c(h2))
        return d

    def setprec_local(self, h1, h2):
        """setprec's element-local diagonal (before dssum and reciprocal)"""
        d = np.zeros(self.n)
        lib().ref_setprec_local(self.h, d, _c(h1), _c(h2))
        return d

    def glsc3(self, a, b, m):
        return lib().ref_glsc3(self.h, _c(a), _c(b), _c(m))

    def chktcg1(self, tol, res, h1, h2, mask, mult, binv):
        t = C.c_double(tol)
        lib().ref_chktcg1(self.h, C.byref(t), _c(res), _c(h1), _c(h2), _c(mask), _c(mult), _c(binv))
        return t.value

    def cggo(self, f, h1, h2, mask, mult, binv, tin, maxit=10 ** 9, maxcg=900, istep=0):
        x = np.zeros(self.n)
        r0, r2 = C.c_double(0), C.c_double(0)
        it = lib().ref_cggo(self.h, x, _c(f), _c(h1), _c(h2), _c(mask), _c(mult), float(tin),
                            int(min(maxit, 2 ** 31 - 1)), int(min(maxcg, 2 ** 31 - 1)), int(istep),
                            _c(binv), C.byref(r0), C.byref(r2))
        return x, it, r0.value, r2.value

    def gmres(self, rhs, h1, h2, wt, mask, tol, maxit=10 ** 6, m=30, null_space=False, mg=None):
        """hmh_gmres with the Jacobi stand-in preconditioner, or h1mg_solve
        when mg (an H1mg) is given.  Returns (x, iterations, div0, rnorm)."""
        x = np.array(rhs, dtype=np.float64, copy=True)
        d0, rn = C.c_double(0), C.c_double(0)
        if mg is None:
            it = lib().ref_gmres(self.h, x, _c(h1), _c(h2), _c(wt), _c(mask), float(tol),
                                 int(maxit), int(m), int(bool(null_space)), C.byref(d0),
                                 C.byref(rn))
        else:
            it = lib().ref_gmres_h1mg(self.h, mg.h, x, _c(h1), _c(h2), _c(wt), _c(mask),
                                      float(tol), int(maxit), int(m), int(bool(null_space)),
                                      C.byref(d0), C.byref(rn))
        return x, it, d0.value, rn.value

    def flex_cg(self, rhs, h1, h2, wt, mask, tol, maxit=10 ** 6, null_space=False, mg=None):
        """hmh_flex_cg with the Jacobi stand-in preconditioner, or h1mg_solve
        when mg (an H1mg) is given.  Returns (x, iterations, div0, rnorm)."""
        x = np.array(rhs, dtype=np.float64, copy=True)
        d0, rn = C.c_double(0), C.c_double(0)
        if mg is None:
            it = lib().ref_flex_cg(self.h, x, _c(h1), _c(h2), _c(wt), _c(mask), float(tol),
                                   int(maxit), int(bool(null_space)), C.byref(d0), C.byref(rn))
        else:
            it = lib().ref_flex_cg_h1mg(self.h, mg.h, x, _c(h1), _c(h2), _c(wt), _c(mask),
                                        float(tol), int(maxit), int(bool(null_space)),
                                        C.byref(d0), C.byref(rn))
        return x, it, d0.value, rn.value

    def hmholtz(self, rhs, h1, h2, mask, mult, binv, tli, maxit=10 ** 9, maxcg=900, istep=0):
        """Returns (u, rhs_after_dssum_mask, niter, rbn0, rbn2)."""
        u = np.zeros(self.n)
        rhs = np.array(rhs, dtype=np.float64, copy=True)
        r0, r2 = C.c_double(0), C.c_double(0)
        it = lib().ref_hmholtz(self.h, u, rhs, _c(h1), _c(h2), _c(mask), _c(mult), float(tli),
                               int(min(maxit, 2 ** 31 - 1)), int(min(maxcg, 2 ** 31 - 1)),
                               int(istep), _c(binv), C.byref(r0), C.byref(r2))
        return u, rhs, it, r0.value, r2.value


def face_types(nx1, nel, glo_num, mask):
    """Face types per element (r-, r+, s-, s+, t-, t+) as get_fast_bc gives
    them for the pressure (core/fast3d.f:802-870), read from the numbering
    and the mask: 0 where the face's point (1, 1) is shared with another
    element (interior or periodic face), else 1 where it is masked
    (Dirichlet), else 2 (Neumann)."""
    g = np.asarray(glo_num).reshape(nel, nx1, nx1, nx1)  # [e, k, j, i]
    m = np.asarray(mask).reshape(nel, nx1, nx1, nx1)
    _, inv, cnt = np.unique(g.reshape(-1), return_inverse=True, return_counts=True)
    shared = (cnt[inv] > 1).reshape(g.shape)
    n2 = nx1 - 1
    pts = [(slice(None), 1, 1, 0), (slice(None), 1, 1, n2), (slice(None), 1, 0, 1),
           (slice(None), 1, n2, 1), (slice(None), 0, 1, 1), (slice(None), n2, 1, 1)]
    fbc = np.empty((nel, 6), dtype=np.int32)
    for f, p in enumerate(pts):
        fbc[:, f] = np.where(shared[p], 0, np.where(m[p] == 0.0, 1, 2))
    return fbc


class H1mg:
    """The pressure preconditioner h1mg_solve (h1mg.c) on an Ops mesh:
    x, y, z the fine GLL coordinates, fbc the face types (face_types),
    vertex the 8 vertex ids per element (tensor corner order)."""

    def __init__(self, ops, x, y, z, fbc, vertex, null_space=False):
        self.ops = ops
        self._keep = [_c(x), _c(y), _c(z)]
        self.h = lib().ref_h1mg_create(ops.h, self._keep[0], self._keep[1], self._keep[2],
                                       np.ascontiguousarray(fbc, dtype=np.int32).reshape(-1),
                                       _c(vertex, np.int64).reshape(-1), int(bool(null_space)))
        if not self.h:
            raise ValueError("h1mg setup failed (lx1 < 3 or a singular coarse matrix)")

    def __del__(self):
        try:
            lib().ref_h1mg_free(self.h)
        except Exception:
            pass

    @property
    def levels(self):
        return [lib().ref_h1mg_nx(self.h, l) for l in range(lib().ref_h1mg_nlev(self.h))]

    @property
    def ncoarse(self):
        return lib().ref_h1mg_ncoarse(self.h)

    def level(self, l):
        """(mask, rwt, swt) of level l (0 = coarsest; swt zero there)."""
        n = self.levels[l] ** 3 * self.ops.nel
        out = [np.zeros(n) for _ in range(3)]
        lib().ref_h1mg_level(self.h, l, *[o.ctypes.data_as(C.c_void_p) for o in out])
        return tuple(out)

    def lengths(self):
        """per element (3, 3): left, middle, right widths in r, s, t"""
        out = np.zeros(9 * self.ops.nel)
        lib().ref_h1mg_lengths(self.h, out)
        return out.reshape(self.ops.nel, 3, 3)

    def solve(self, rhs):
        """z = M rhs; returns (z, rhs masked as the reference leaves it)."""
        r = np.array(rhs, dtype=np.float64, copy=True)
        z = np.zeros_like(r)
        lib().ref_h1mg_solve(self.h, z, r)
        return z, r

    def schwarz(self, l, r):
        r = np.array(r, dtype=np.float64, copy=True)
        e = np.zeros_like(r)
        lib().ref_h1mg_schwarz(self.h, l, e, r)
        return e

    def coarse(self, r):
        r = np.ascontiguousarray(r, dtype=np.float64)
        e = np.zeros_like(r)
        lib().ref_h1mg_coarse(self.h, e, r)
        return e


def fdm1d(n, lbc, rbc, ll, lm, lr):
    """(S, lam) of one 1-D fast-diagonalisation operator; S[i, j] is
    component i of eigenvector j."""
    nl = n + 3
    s, lam = np.zeros(nl * nl), np.zeros(nl)
    lib().ref_fdm1d(int(n), int(lbc), int(rbc), float(ll), float(lm), float(lr), s, lam)
    return s.reshape(nl, nl).T.copy(), lam


def geom_rst(nx1, nel, x, y, z):
    """(rst (9, n): rx ry rz sx sy sz tx ty tz, jac (n)) of glmapm1."""
    n = nx1 ** 3 * nel
    g, bm1, jac, rst = np.zeros(6 * n), np.zeros(n), np.zeros(n), np.zeros(9 * n)
    lib().ref_geom_rst(int(nx1), int(nel), _c(x), _c(y), _c(z), g, bm1, jac, rst)
    return rst.reshape(9, n), jac


def wgradm1(nx1, nel, u, rst):
    n = nx1 ** 3 * nel
    out = [np.zeros(n) for _ in range(3)]
    lib().ref_wgradm1(int(nx1), int(nel), *out, _c(u), _c(rst))
    return out


def cdtp(nx1, nel, x, rst, jac, bm1, isd):
    out = np.zeros(nx1 ** 3 * nel)
    lib().ref_cdtp(int(nx1), int(nel), out, _c(x), _c(rst), _c(jac), _c(bm1), int(isd))
    return out


def dudxyz(nx1, nel, u, rst, jac, isd):
    out = np.zeros(nx1 ** 3 * nel)
    lib().ref_dudxyz(int(nx1), int(nel), out, _c(u), _c(rst), _c(jac), int(isd))
    return out


def op_curl(ops, u1, u2, u3, rst, jac, bm1, binv, ifavg=True):
    out = [np.zeros(ops.n) for _ in range(3)]
    lib().ref_op_curl(ops.h, *out, _c(u1), _c(u2), _c(u3), int(bool(ifavg)), _c(rst), _c(jac),
                      _c(bm1), _c(binv))
    return out


def conv1(nx1, nel, u, v, rst, jac):
    out = np.zeros(nx1 ** 3 * nel)
    lib().ref_conv1(int(nx1), int(nel), out, _c(u), *[_c(a) for a in v], _c(rst), _c(jac))
    return out


def advab(nx1, nel, bf, v, bm1, rst, jac):
    out = [np.array(a, dtype=np.float64, copy=True) for a in bf]
    lib().ref_advab(int(nx1), int(nel), *out, *[_c(a) for a in v], _c(bm1), _c(rst), _c(jac))
    return out


def makeabf(bf, abx1, abx2, vtrans, ab):
    """returns (bf, abx1, abx2) after makeabf (one component)"""
    bf, a1, a2 = (np.array(a, dtype=np.float64, copy=True) for a in (bf, abx1, abx2))
    lib().ref_makeabf(bf.size, bf, a1, a2, _c(vtrans), _c(ab))
    return bf, a1, a2


def makebdf(bf, v, vlag, bm1, vtrans, bd, nbd, dt):
    bf = np.array(bf, dtype=np.float64, copy=True)
    lag = _c(np.concatenate([np.asarray(a, dtype=np.float64) for a in vlag])) if vlag else \
        np.zeros(1)
    lib().ref_makebdf(bf.size, bf, _c(v), lag, _c(bm1), _c(vtrans), _c(bd), int(nbd), float(dt))
    return bf


def sumab(vv, vvlag, ab, nab):
    v = np.zeros(len(vv))
    lib().ref_sumab(v.size, v, _c(vv), _c(np.concatenate(vvlag)), _c(ab), int(nab))
    return v


def convect_new(nx1, nel, lxd, u, v, rst, bm1):
    """convop with dealiasing on lxd Gauss points: convect_new(u) / bm1"""
    out = np.zeros(nx1 ** 3 * nel)
    lib().ref_convect_new(int(nx1), int(nel), int(lxd), out, _c(u), *[_c(a) for a in v],
                          _c(rst), _c(bm1))
    return out


def convect_cons(nx1, nel, lxd, u, v, rst, bm1):
    """convop with the conservative form on lxd Gauss points: div(v u) / bm1"""
    out = np.zeros(nx1 ** 3 * nel)
    lib().ref_convect_cons(int(nx1), int(nel), int(lxd), out, _c(u), *[_c(a) for a in v],
                           _c(rst), _c(bm1))
    return out


def conv2(nx1, nel, fi, v, rst, bm1):
    out = np.zeros(nx1 ** 3 * nel)
    lib().ref_conv2(int(nx1), int(nel), out, _c(fi), *[_c(a) for a in v], _c(rst), _c(bm1))
    return out


def convopo(nx1, nel, fi, v, rst, jac, bm1, ofc):
    """the skew-symmetric convective form; ofc (nel, 6) outflow-face flags"""
    out = np.zeros(nx1 ** 3 * nel)
    of = np.ascontiguousarray(ofc, dtype=np.int32).reshape(-1)
    lib().ref_convopo(int(nx1), int(nel), out, _c(fi), *[_c(a) for a in v], _c(rst), _c(jac),
                      _c(bm1), of.ctypes.data_as(C.c_void_p))
    return out


def cresvsp(ops, v, h1, h2, vdiff, qtl, pr, bf, rst):
    """velocity residual of the splitting step; v, bf: 3 components"""
    out = [np.zeros(ops.n) for _ in range(3)]
    lib().ref_cresvsp(ops.h, *out, *[_c(a) for a in v], _c(h1), _c(h2), _c(vdiff), _c(qtl),
                      _c(pr), *[_c(a) for a in bf], _c(rst))
    return out


def cresvsp_weak(ops, v, h1, h2, vdiff, qtl, pr, bf, rst, jac, bm1, stress=True):
    """velocity residual of the stress formulation's branch of the splitting
    step (weak pressure gradient); v, bf: 3 components"""
    out = [np.zeros(ops.n) for _ in range(3)]
    lib().ref_cresvsp_weak(ops.h, *out, *[_c(a) for a in v], _c(h1), _c(h2), _c(vdiff),
                           _c(qtl), _c(pr), *[_c(a) for a in bf], _c(rst), _c(jac), _c(bm1),
                           1 if stress else 0)
    return out


def axsf(ops, u, h1, h2, rst, jac, bm1):
    """the stress formulation's coupled operator (axsf_e_3d); u: 3 components"""
    out = [np.zeros(ops.n) for _ in range(3)]
    lib().ref_axsf(ops.h, *out, *[_c(a) for a in u], _c(h1), _c(h2), _c(rst), _c(jac), _c(bm1))
    return out


def hmhzsf(ops, r, h1, h2, masks, mult, binv, rst, jac, bm1, vol, tol):
    """the stress formulation's coupled solve (hmhzsf without projection);
    returns (u, r after, iterations (-1: 200 reached), rbn0, rbn2)"""
    u = [np.zeros(ops.n) for _ in range(3)]
    rr = [np.array(a, dtype=np.float64, copy=True) for a in r]
    r0, r2 = C.c_double(0), C.c_double(0)
    it = lib().ref_hmhzsf(ops.h, *u, *rr, _c(h1), _c(h2), *[_c(m) for m in masks], _c(mult),
                          _c(binv), _c(rst), _c(jac), _c(bm1), float(vol), float(tol),
                          C.byref(r0), C.byref(r2))
    return u, rr, it, r0.value, r2.value


def crespsp(ops, ve, pr, qtl, vdiff, vtrans, bf, bm1, binv, dtbd, null_space, rst, jac,
            v=None, fbc=None):
    """pressure right-hand side of the splitting step; fbc (nel, 6) face
    types (0 none, 1 velocity scaled by dtbd, 2 'shl', 3 'SYM') with v the
    current velocity"""
    out = np.zeros(ops.n)
    z, w = zwgll(ops.nx1)
    vv = v if v is not None else [np.zeros(ops.n)] * 3
    fb = None if fbc is None else np.ascontiguousarray(fbc, dtype=np.int32).reshape(-1)
    lib().ref_crespsp(ops.h, out, *[_c(a) for a in ve], _c(pr), _c(qtl), _c(vdiff), _c(vtrans),
                      *[_c(a) for a in bf], _c(bm1), _c(binv), float(dtbd),
                      int(bool(null_space)), _c(rst), _c(jac), *[_c(a) for a in vv],
                      None if fb is None else fb.ctypes.data_as(C.c_void_p), _c(w))
    return out


def h1mg_levels(lx1):
    o = np.zeros(4, dtype=np.int32)
    lmax = lib().ref_h1mg_levels(int(lx1), o)
    return [int(v) for v in o[:lmax]]


class Projection:
    """One projection space of previous solutions (navier4.f:562-1188) on an
    Ops mesh; hsolve() is the reference's hsolve with projection on."""

    def __init__(self, ops, mmx=8):
        self.ops = ops
        self.h = lib().ref_proj_create(ops.h, int(mmx))

    def __del__(self):
        try:
            lib().ref_proj_free(self.h)
        except Exception:
            pass

    @property
    def m(self):
        return lib().ref_proj_m(self.h)

    def basis(self):
        """(X, B) as (m, n) arrays (copies)."""
        n, m = self.ops.n, self.m
        X = np.array([np.ctypeslib.as_array(lib().ref_proj_x(self.h, k), (n,)) for k in range(m)])
        B = np.array([np.ctypeslib.as_array(lib().ref_proj_b(self.h, k), (n,)) for k in range(m)])
        return X.reshape(m, n), B.reshape(m, n)

    def hsolve(self, r, h1, h2, vmk, vml, binv, tli, maxit=10 ** 9, maxcg=900, istep=0):
        """Returns (u, r_after, niter, rbn0, rbn2)."""
        o = self.ops
        u = np.zeros(o.n)
        r = np.array(r, dtype=np.float64, copy=True)
        r0, r2 = C.c_double(0), C.c_double(0)
        it = lib().ref_hsolve(o.h, self.h, u, r, _c(h1), _c(h2), _c(vmk), _c(vml), float(tli),
                              int(min(maxit, 2 ** 31 - 1)), int(min(maxcg, 2 ** 31 - 1)),
                              int(istep), _c(binv), C.byref(r0), C.byref(r2))
        return u, r, it, r0.value, r2.value


def local_grad3(u, D):
    N = D.shape[0] - 1
    m3 = (N + 1) ** 3
    ur, us, ut = np.zeros(m3), np.zeros(m3), np.zeros(m3)
    lib().ref_local_grad3(ur, us, ut, _c(u), N, _c(D.T.ravel()), _c(D.ravel()))
    return ur, us, ut


def local_grad3_t(ur, us, ut, D):
    N = D.shape[0] - 1
    m3 = (N + 1) ** 3
    u, w = np.zeros(m3), np.zeros(m3)
    lib().ref_local_grad3_t(u, _c(ur), _c(us), _c(ut), N, _c(D.T.ravel()), _c(D.ravel()), w)
    return u


def max_threads():
    return lib().ref_max_threads()


# ---- problem assembly (what Nek's setup produces for a box case) ------------
def box_problem(nx1, kx, ky, kz, periodic=(False, False, False), dirichlet=None, amp=0.05,
                v=(0.0, 0.0, 1.0), nthreads=1):
    """Mesh + geometry + numbering + masks + multiplicity + inverse mass.

    dirichlet: 6 flags for the domain faces (x-, x+, y-, y+, z-, z+); default:
    every non-periodic face.  The mask follows bcmask (bdry.f:317): zero on
    Dirichlet faces (facev) then dsop 'MUL'.  vmult = 1/dssum(1)
    (connect1.f:126-135), binvm1 = 1/dssum(bm1) (coef.f:1500-1545).
    """
    nel = kx * ky * kz
    nxyz = nx1 ** 3
    n = nxyz * nel
    x, y, z, vert = box_mesh(nx1, kx, ky, kz, periodic, amp, v)
    g, bm1, jac = geom(nx1, nel, x, y, z)
    glo, ngv = setvert3d(nx1, nel, vert)
    z1, w1 = zwgll(nx1)
    D, DT = dgll(z1)
    ops = Ops(nx1, nel, D, g, bm1, glo, nthreads)
    if dirichlet is None:
        dirichlet = (not periodic[0],) * 2 + (not periodic[1],) * 2 + (not periodic[2],) * 2
    mask = np.ones((nel, nx1, nx1, nx1))  # [e, iz, iy, ix]
    e = np.arange(nel)
    ex, ey, ez = e % kx, (e // kx) % ky, e // (kx * ky)
    if dirichlet[0]:
        mask[ex == 0, :, :, 0] = 0.0
    if dirichlet[1]:
        mask[ex == kx - 1, :, :, -1] = 0.0
    if dirichlet[2]:
        mask[ey == 0, :, 0, :] = 0.0
    if dirichlet[3]:
        mask[ey == ky - 1, :, -1, :] = 0.0
    if dirichlet[4]:
        mask[ez == 0, 0, :, :] = 0.0
    if dirichlet[5]:
        mask[ez == kz - 1, -1, :, :] = 0.0
    mask = ops.dsop(mask.reshape(-1), "*")
    mult = 1.0 / ops.dssum(np.ones(n))
    binv = 1.0 / ops.dssum(bm1)
    return dict(nx1=nx1, nel=nel, n=n, kx=kx, ky=ky, kz=kz, x=x, y=y, z=z, vertex=vert, g=g,
                bm1=bm1, jac=jac, glo_num=glo, ngv=ngv, zgll=z1, wgll=w1, D=D, mask=mask,
                mult=mult, binv=binv, ops=ops)
