"""Python front end mirroring the reference's Helmholtz interface.

Method names, argument order and meaning follow the Fortran routines they
replace (core/hmholtz.f: hmholtz :2, axhelm :72, setprec :380, cggo :611;
core/dssum.f: dssum :33, dsop :100).  Every call goes through the C ABI of
libnekgpu.so.  Arrays may be

  * numpy float64 host arrays -> the host entry points (copies inside the call)
  * torch float64 CUDA tensors -> the *_dev entry points (no copies)

Output arrays are written in place, as the Fortran routines do; the solver
calls also return (niter, rbn0, rbn2).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi

_cdouble = C.c_double
_cint = C.c_int


def _is_dev(a) -> bool:
    return hasattr(a, "is_cuda") and a.is_cuda


def _ptr(a):
    if a is None:
        return None
    if _is_dev(a):
        if str(a.dtype) != "torch.float64" or not a.is_contiguous():
            raise TypeError("device arrays must be contiguous torch.float64 CUDA tensors")
        return C.c_void_p(a.data_ptr())
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError("host arrays must be C-contiguous numpy float64 arrays")
    return a.ctypes.data_as(C.c_void_p)


class NekGpu:
    """One library handle: one device, one stream, one mesh."""

    def __init__(self, device: int = 0):
        self._L = _capi.load()
        self._h = C.c_int64(0)
        self._check(self._L.nekgpu_init(C.byref(_cint(device)), C.byref(self._h)), orphan=True)
        self.n = 0
        self.lx1 = 0
        self.nel = 0

    # ---- plumbing ---------------------------------------------------------
    def last_error(self) -> str:
        buf = C.create_string_buffer(1024)
        self._L.nekgpu_last_error(C.byref(self._h), buf, C.byref(_cint(1024)))
        return buf.value.decode(errors="replace")

    def _check(self, rc: int, orphan: bool = False, allow=()):
        if rc != 0 and rc not in allow:
            raise _capi.NekGpuError(rc, self.last_error())
        return rc

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._L.nekgpu_finalize(C.byref(self._h))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_option(self, key: int, value: int):
        self._check(self._L.nekgpu_set_option(C.byref(self._h), C.byref(_cint(key)),
                                              C.byref(_cint(int(value)))))

    def set_exact(self, on: bool = True):
        """Round every FP64 product and sum separately, in the reference's order."""
        self.set_option(_capi.OPT_EXACT, int(on))

    def set_timing(self, on: bool = True):
        self.set_option(_capi.OPT_TIMING, int(on))

    def last_timing(self):
        t, a, k = _cdouble(0), _cdouble(0), _cint(0)
        self._check(self._L.nekgpu_last_timing(C.byref(self._h), C.byref(t), C.byref(a),
                                               C.byref(k)))
        return t.value, a.value, k.value

    def last_kernel_times(self):
        """(ms operator, ms boundary groups, ms update, iterations) of the last
        solve with kernel timing on, summed over its iterations."""
        a, g, u, k = _cdouble(0), _cdouble(0), _cdouble(0), _cint(0)
        self._check(self._L.nekgpu_last_kernel_times(C.byref(self._h), C.byref(a), C.byref(g),
                                                     C.byref(u), C.byref(k)))
        return a.value, g.value, u.value, k.value

    def launch_count(self) -> int:
        c = C.c_int64(0)
        self._L.nekgpu_launch_count(C.byref(c))
        return c.value

    # ---- operator launch shapes ---------------------------------------------
    def autotune(self, precision: int = 0, h1mode: int = 0, h2mode: int = 1):
        """Time the operator's launch shapes now; returns (kind, epb, ms)."""
        k, e, ms = _cint(0), _cint(0), _cdouble(0)
        self._check(self._L.nekgpu_autotune(C.byref(self._h), C.byref(_cint(precision)),
                                            C.byref(_cint(h1mode)), C.byref(_cint(h2mode)),
                                            C.byref(k), C.byref(e), C.byref(ms)))
        return k.value, e.value, ms.value

    def ax_shape(self, precision: int = 0):
        """Launch shape in use: (kind, elements per block, tuned ms or 0)."""
        k, e, ms = _cint(0), _cint(0), _cdouble(0)
        self._check(self._L.nekgpu_ax_shape(C.byref(self._h), C.byref(_cint(precision)),
                                            C.byref(k), C.byref(e), C.byref(ms)))
        return k.value, e.value, ms.value

    def gs_shape(self, precision: int = 1):
        """Boundary-group kernel shape: (threads, gshift, tuned ms or 0)."""
        t, g, ms = _cint(0), _cint(0), _cdouble(0)
        self._check(self._L.nekgpu_gs_shape(C.byref(self._h), C.byref(_cint(precision)),
                                            C.byref(t), C.byref(g), C.byref(ms)))
        return t.value, g.value, ms.value

    def set_gs_shape(self, threads: int, gshift: int = 0):
        """Pin the FP32 boundary-group kernel shape (threads 0: default / tuning)."""
        self._check(self._L.nekgpu_set_gs_shape(C.byref(self._h), C.byref(_cint(threads)),
                                                C.byref(_cint(gshift))))

    def set_ax_shape(self, precision: int, kind: int, epb: int = 0):
        self._check(self._L.nekgpu_set_ax_shape(C.byref(self._h), C.byref(_cint(precision)),
                                                C.byref(_cint(kind)), C.byref(_cint(epb))))

    def ax_candidates(self, precision: int = 0):
        """Candidate launch shapes [(kind, epb), ...] of this mesh."""
        cnt = _cint(64)
        kinds = (C.c_int * 64)()
        epbs = (C.c_int * 64)()
        self._check(self._L.nekgpu_ax_candidates(C.byref(self._h), C.byref(_cint(precision)),
                                                 kinds, epbs, C.byref(cnt)))
        return [(kinds[q], epbs[q]) for q in range(min(cnt.value, 64))]

    # ---- mesh -------------------------------------------------------------
    def setup(self, lx1: int, nel: int, D, g, bm1, glo_num):
        """D: (lx1,lx1) numpy with D[i,j] = dl_j/dr(z_i) (the reference's dxm1);
        g: (6, n) geometric factors G1..G6; bm1: (n,); glo_num: (n,) int64."""
        n = lx1 ** 3 * nel
        D = np.asarray(D, dtype=np.float64)
        dxm1 = np.ascontiguousarray(D.T)  # Fortran order: dxm1(i,j) at [i + j*lx1]
        g = np.ascontiguousarray(np.asarray(g, dtype=np.float64).reshape(6, n))
        bm1 = np.ascontiguousarray(bm1, dtype=np.float64)
        glo = np.ascontiguousarray(glo_num, dtype=np.int64)
        if bm1.size != n or glo.size != n:
            raise ValueError("bm1 / glo_num must have lx1^3*nel entries")
        gp = [g[q].ctypes.data_as(C.c_void_p) for q in range(6)]
        self._check(self._L.nekgpu_setup(C.byref(self._h), C.byref(_cint(lx1)),
                                         C.byref(_cint(nel)), dxm1.ctypes.data_as(C.c_void_p),
                                         *gp, bm1.ctypes.data_as(C.c_void_p),
                                         glo.ctypes.data_as(C.c_void_p)))
        self.n, self.lx1, self.nel = n, lx1, nel

    def hmh_gmres(self, res, h1, h2, wt, mask, tol, maxit=10 ** 6, kmax=30, null_space=False):
        """The pressure solve's GMRES (res: rhs in, solution out; all device
        arrays or all host arrays).  Returns (iterations, div0, rnorm, status)."""
        dev = [_is_dev(t) for t in (res, h1, h2, wt, mask)]
        if any(dev) and not all(dev):
            raise TypeError("hmh_gmres takes all device or all host arrays")
        fn = self._L.nekgpu_hmh_gmres_dev if dev[0] else self._L.nekgpu_hmh_gmres
        it, d0, rn = _cint(0), _cdouble(0), _cdouble(0)
        rc = fn(
            C.byref(self._h), _ptr(res), _ptr(h1), _ptr(h2), _ptr(wt), _ptr(mask),
            C.byref(_cdouble(tol)), C.byref(_cint(int(maxit))), C.byref(_cint(kmax)),
            C.byref(_cint(int(bool(null_space)))), C.byref(it), C.byref(d0), C.byref(rn))
        self._check(rc, allow=(_capi.ENOTCONV,))
        return it.value, d0.value, rn.value, rc

    def hmh_flex_cg(self, res, h1, h2, wt, mask, tol, maxit=10 ** 6, null_space=False):
        """The pressure solve's flexible CG (res: rhs in, solution out; all
        device or all host arrays).  Returns (iterations, div0, rnorm, status)."""
        dev = [_is_dev(t) for t in (res, h1, h2, wt, mask)]
        if any(dev) and not all(dev):
            raise TypeError("hmh_flex_cg takes all device or all host arrays")
        fn = self._L.nekgpu_hmh_flex_cg_dev if dev[0] else self._L.nekgpu_hmh_flex_cg
        it, d0, rn = _cint(0), _cdouble(0), _cdouble(0)
        rc = fn(C.byref(self._h), _ptr(res), _ptr(h1), _ptr(h2), _ptr(wt), _ptr(mask),
                C.byref(_cdouble(tol)), C.byref(_cint(int(maxit))),
                C.byref(_cint(int(bool(null_space)))), C.byref(it), C.byref(d0), C.byref(rn))
        self._check(rc, allow=(_capi.ENOTCONV,))
        return it.value, d0.value, rn.value, rc

    # ---- gradient-type operators of the splitting step (device arrays) --------
    def wgradm1(self, ux, uy, uz, u):
        self._check(self._L.nekgpu_wgradm1_dev(C.byref(self._h), _ptr(ux), _ptr(uy), _ptr(uz),
                                               _ptr(u)))

    def dudxyz(self, du, u, isd: int):
        self._check(self._L.nekgpu_dudxyz_dev(C.byref(self._h), _ptr(du), _ptr(u),
                                              C.byref(_cint(isd))))

    def cdtp(self, dtx, x, isd: int):
        self._check(self._L.nekgpu_cdtp_dev(C.byref(self._h), _ptr(dtx), _ptr(x),
                                            C.byref(_cint(isd))))

    def op_curl(self, w1, w2, w3, u1, u2, u3, ifavg=True, binv=None):
        self._check(self._L.nekgpu_op_curl_dev(C.byref(self._h), _ptr(w1), _ptr(w2), _ptr(w3),
                                               _ptr(u1), _ptr(u2), _ptr(u3),
                                               C.byref(_cint(int(bool(ifavg)))), _ptr(binv)))

    def dealias_setup(self, lxd: int):
        self._check(self._L.nekgpu_dealias_setup(C.byref(self._h), C.byref(_cint(lxd))))

    def convop(self, conv, u, v):
        """convop: dealiased once dealias_setup has run, conv1 otherwise"""
        self._check(self._L.nekgpu_convop_dev(C.byref(self._h), _ptr(conv), _ptr(u),
                                              *[_ptr(a) for a in v]))

    def conv2(self, dtfi, fi, v):
        self._check(self._L.nekgpu_conv2_dev(C.byref(self._h), _ptr(dtfi), _ptr(fi),
                                             *[_ptr(a) for a in v]))

    def convopo(self, conv, fi, v, ofc=None):
        """skew-symmetric convective form; ofc: host (nel, 6) outflow-face flags"""
        of = None if ofc is None else np.ascontiguousarray(ofc, dtype=np.int32).reshape(-1)
        self._check(self._L.nekgpu_convopo_dev(C.byref(self._h), _ptr(conv), _ptr(fi),
                                               *[_ptr(a) for a in v],
                                               None if of is None else C.c_void_p(of.ctypes.data)))

    def convect_cons(self, conv, u, v):
        """the conservative dealiased form div(v u) / bm1 (needs dealias_setup)"""
        self._check(self._L.nekgpu_convect_cons_dev(C.byref(self._h), _ptr(conv), _ptr(u),
                                                    *[_ptr(a) for a in v]))

    def conv1(self, du, u, v):
        """du = (v . grad) u without dealiasing (device arrays; v: 3 components)"""
        self._check(self._L.nekgpu_conv1_dev(C.byref(self._h), _ptr(du), _ptr(u),
                                             *[_ptr(a) for a in v]))

    def advab(self, bf, v):
        """bf_c -= bm1 (v . grad) v_c (device arrays, 3 components each)"""
        self._check(self._L.nekgpu_advab_dev(C.byref(self._h), *[_ptr(a) for a in bf],
                                             *[_ptr(a) for a in v]))

    def makeabf(self, bf, abx1, abx2, vtrans, ab):
        a = np.ascontiguousarray(ab, dtype=np.float64)
        self._check(self._L.nekgpu_makeabf_dev(C.byref(self._h), _ptr(bf), _ptr(abx1), _ptr(abx2),
                                               _ptr(vtrans), C.c_void_p(a.ctypes.data)))

    def makebdf(self, bf, v, vlag, vtrans, bd, nbd: int, dt: float):
        """vlag: one device array holding the nbd - 1 lagged fields back to back"""
        b = np.ascontiguousarray(bd, dtype=np.float64)
        self._check(self._L.nekgpu_makebdf_dev(C.byref(self._h), _ptr(bf), _ptr(v), _ptr(vlag),
                                               _ptr(vtrans), C.c_void_p(b.ctypes.data),
                                               C.byref(_cint(nbd)), C.byref(_cdouble(dt))))

    def sumab(self, v, vv, vvlag, ab, nab: int):
        a = np.ascontiguousarray(ab, dtype=np.float64)
        self._check(self._L.nekgpu_sumab_dev(C.byref(self._h), _ptr(v), _ptr(vv), _ptr(vvlag),
                                             C.c_void_p(a.ctypes.data), C.byref(_cint(nab))))

    def cresvsp(self, r, v, h1, h2, vdiff, qtl, pr, bf):
        """velocity residual of the splitting step (r, v, bf: 3 device arrays each)"""
        self._check(self._L.nekgpu_cresvsp_dev(C.byref(self._h), *[_ptr(a) for a in r],
                                               *[_ptr(a) for a in v], _ptr(h1), _ptr(h2),
                                               _ptr(vdiff), _ptr(qtl), _ptr(pr),
                                               *[_ptr(a) for a in bf]))

    def cresvsp_weak(self, r, v, h1, h2, vdiff, qtl, pr, bf, stress=True):
        """velocity residual with the weak pressure gradient (the stress
        formulation's branch of the splitting step; 3 device arrays each)"""
        self._check(self._L.nekgpu_cresvsp_weak_dev(C.byref(self._h), *[_ptr(a) for a in r],
                                                    *[_ptr(a) for a in v], _ptr(h1), _ptr(h2),
                                                    _ptr(vdiff), _ptr(qtl), _ptr(pr),
                                                    *[_ptr(a) for a in bf],
                                                    C.byref(_cint(1 if stress else 0))))

    def axhmsf(self, au, u, h1, h2):
        """the stress formulation's coupled operator (au, u: 3 device arrays)"""
        self._check(self._L.nekgpu_axhmsf_dev(C.byref(self._h), *[_ptr(a) for a in au],
                                              *[_ptr(a) for a in u], _ptr(h1), _ptr(h2)))

    def hmhzsf(self, u, r, h1, h2, masks, mult, binv, tol):
        """the stress formulation's coupled solve (u, r, masks: 3 device
        arrays each; r is masked and dssum'ed in place).  Returns
        (iterations, rbn0, rbn2, status)."""
        it, r0, r2 = _cint(0), _cdouble(0), _cdouble(0)
        rc = self._L.nekgpu_hmhzsf_dev(C.byref(self._h), *[_ptr(a) for a in u],
                                       *[_ptr(a) for a in r], _ptr(h1), _ptr(h2),
                                       *[_ptr(a) for a in masks], _ptr(mult), _ptr(binv),
                                       C.byref(_cdouble(tol)), C.byref(it), C.byref(r0),
                                       C.byref(r2))
        self._check(rc, allow=(_capi.ENOTCONV,))
        return it.value, r0.value, r2.value, rc

    def crespsp(self, respr, ve, pr, qtl, vdiff, vtrans, bf, binv, dtbd, null_space=False,
                v=None, fbc=None):
        """pressure right-hand side of the splitting step; fbc: host (nel, 6)
        face types (0 none, 1 velocity times dtbd, 2 'shl', 3 'SYM'), v the
        current velocity (3 device arrays) for types 1 and 2"""
        fb = None if fbc is None else np.ascontiguousarray(fbc, dtype=np.int32).reshape(-1)
        vv = v if v is not None else [None] * 3
        self._check(self._L.nekgpu_crespsp_dev(C.byref(self._h), _ptr(respr),
                                               *[_ptr(a) for a in ve], _ptr(pr), _ptr(qtl),
                                               _ptr(vdiff), _ptr(vtrans),
                                               *[_ptr(a) for a in bf], _ptr(binv),
                                               C.byref(_cdouble(dtbd)),
                                               C.byref(_cint(int(bool(null_space)))),
                                               *[_ptr(a) for a in vv],
                                               None if fb is None else C.c_void_p(fb.ctypes.data)))

    def h1mg_setup(self, x, y, z, glo_num, mask=None, fbc=None, null_space=False):
        """The pressure preconditioner h1mg_solve (nekgpu_h1mg_setup): host
        numpy coordinates, the numbering given to setup, and the pressure
        mask or the face types (6 per element).  The pressure solves of this
        handle use it until h1mg_free."""
        f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
        xs, ys, zs = f64(x), f64(y), f64(z)
        glo = np.ascontiguousarray(glo_num, dtype=np.int64).reshape(-1)
        m = None if mask is None else f64(mask)
        fb = None if fbc is None else np.ascontiguousarray(fbc, dtype=np.int32).reshape(-1)
        if m is None and fb is None:
            raise TypeError("h1mg_setup needs the mask or the face types")
        rc = self._L.nekgpu_h1mg_setup(C.byref(self._h), _ptr(xs), _ptr(ys), _ptr(zs), _ptr(m),
                                       C.c_void_p(glo.ctypes.data),
                                       None if fb is None else C.c_void_p(fb.ctypes.data),
                                       C.byref(_cint(int(bool(null_space)))))
        self._check(rc)

    def h1mg_free(self):
        self._check(self._L.nekgpu_h1mg_free(C.byref(self._h)))

    def h1mg_apply(self, z, rhs):
        """z = M rhs on device tensors; rhs is masked in place."""
        if not (_is_dev(z) and _is_dev(rhs)):
            raise TypeError("h1mg_apply takes device arrays")
        self._check(self._L.nekgpu_h1mg_apply_dev(C.byref(self._h), _ptr(z), _ptr(rhs)))

    def setup_xyz(self, lx1: int, nel: int, D, w, x, y, z, glo_num):
        """setup with G1..G6 and bm1 computed on the GPU from the GLL
        coordinates x, y, z ((n,) numpy each) and the GLL weights w (lx1)."""
        n = lx1 ** 3 * nel
        dxm1 = np.ascontiguousarray(np.asarray(D, dtype=np.float64).T)
        w = np.ascontiguousarray(w, dtype=np.float64)
        xyz = [np.ascontiguousarray(a, dtype=np.float64).reshape(-1) for a in (x, y, z)]
        glo = np.ascontiguousarray(glo_num, dtype=np.int64)
        if any(a.size != n for a in xyz) or glo.size != n or w.size != lx1:
            raise ValueError("x, y, z, glo_num must have lx1^3*nel entries, w lx1")
        self._check(self._L.nekgpu_setup_xyz(C.byref(self._h), C.byref(_cint(lx1)),
                                             C.byref(_cint(nel)), _ptr(dxm1), _ptr(w),
                                             *(_ptr(a) for a in xyz),
                                             glo.ctypes.data_as(C.c_void_p)))
        self.n, self.lx1, self.nel = n, lx1, nel

    def geom_update(self, w, x, y, z):
        """New coordinates (torch float64 CUDA tensors) of the same mesh."""
        w = np.ascontiguousarray(w, dtype=np.float64)
        for t in (x, y, z):
            if not _is_dev(t):
                raise TypeError("geom_update takes device arrays")
        self._check(self._L.nekgpu_geom_update_dev(C.byref(self._h), _ptr(w), _ptr(x), _ptr(y),
                                                   _ptr(z)))

    def geometry(self):
        """(g (6, n), bm1 (n,)) in use, as numpy."""
        g = np.zeros((6, self.n))
        bm1 = np.zeros(self.n)
        self._check(self._L.nekgpu_geometry(C.byref(self._h), *(_ptr(g[q]) for q in range(6)),
                                            _ptr(bm1)))
        return g, bm1

    def gs_maps(self):
        ns, ni = C.c_int64(0), C.c_int64(0)
        self._check(self._L.nekgpu_gs_maps(C.byref(self._h), C.byref(ns), C.byref(ni), None, None))
        start = np.zeros(ns.value + 1, dtype=np.int64)
        idx = np.zeros(max(ni.value, 1), dtype=np.int64)
        self._check(self._L.nekgpu_gs_maps(C.byref(self._h), C.byref(ns), C.byref(ni),
                                           start.ctypes.data_as(C.c_void_p),
                                           idx.ctypes.data_as(C.c_void_p)))
        return start, idx[: ni.value]

    # ---- operator ---------------------------------------------------------
    def axhelm(self, au, u, helm1, helm2, imesh: int = 1, isd: int = 1):
        fn = self._L.nekgpu_axhelm_dev if _is_dev(u) else self._L.nekgpu_axhelm
        self._check(fn(C.byref(self._h), _ptr(au), _ptr(u), _ptr(helm1), _ptr(helm2),
                       C.byref(_cint(imesh)), C.byref(_cint(isd))))
        return au

    def dssum(self, u):
        fn = self._L.nekgpu_dssum_dev if _is_dev(u) else self._L.nekgpu_dssum
        self._check(fn(C.byref(self._h), _ptr(u)))
        return u

    def dsop(self, u, op: str):
        if not _is_dev(u):
            raise TypeError("dsop takes a device array")
        self._check(self._L.nekgpu_dsop_dev(C.byref(self._h), _ptr(u), op.encode()[:1]))
        return u

    def setprec(self, dpcm1, helm1, helm2, imsh: int = 1, isd: int = 1):
        fn = self._L.nekgpu_setprec_dev if _is_dev(dpcm1) else self._L.nekgpu_setprec
        self._check(fn(C.byref(self._h), _ptr(dpcm1), _ptr(helm1), _ptr(helm2),
                       C.byref(_cint(imsh)), C.byref(_cint(isd))))
        return dpcm1

    # ---- solvers ----------------------------------------------------------
    def _solve(self, fn, a, b, h1, h2, mask, mult, imsh, tol, maxit, isd, binv, maxcg):
        niter, r0, r2 = _cint(0), _cdouble(0), _cdouble(0)
        mc = C.byref(_cint(int(maxcg))) if maxcg is not None else None
        rc = fn(C.byref(self._h), _ptr(a), _ptr(b), _ptr(h1), _ptr(h2), _ptr(mask), _ptr(mult),
                C.byref(_cint(imsh)), C.byref(_cdouble(tol)), C.byref(_cint(int(maxit))),
                C.byref(_cint(isd)), _ptr(binv), mc, C.byref(niter), C.byref(r0), C.byref(r2))
        self._check(rc, allow=(_capi.ENOTCONV,))
        return niter.value, r0.value, r2.value, rc

    def cggo(self, x, f, h1, h2, mask, mult, imsh, tin, maxit, isd, binv, maxcg=900):
        """x: out.  Returns (niter, rbn0, rbn2, status)."""
        fn = self._L.nekgpu_cggo_dev if _is_dev(x) else self._L.nekgpu_cggo
        return self._solve(fn, x, f, h1, h2, mask, mult, imsh, tin, maxit, isd, binv, maxcg)

    def hsolve(self, name, u, r, h1, h2, vmk, vml, imsh, tol, maxit, isd, bi, space=0,
               maxcg=900):
        """hsolve with projection onto previous solutions of projection space
        `space` (navier4.f:562).  u: out; r: in/out (masked, dssum'ed and
        projected in place).  Returns (niter, rbn0, rbn2, m, status)."""
        del name
        fn = self._L.nekgpu_hsolve_dev if _is_dev(u) else self._L.nekgpu_hsolve
        niter, r0, r2, m = _cint(0), _cdouble(0), _cdouble(0), _cint(0)
        mc = C.byref(_cint(int(maxcg))) if maxcg is not None else None
        rc = fn(C.byref(self._h), C.byref(_cint(space)), _ptr(u), _ptr(r), _ptr(h1), _ptr(h2),
                _ptr(vmk), _ptr(vml), C.byref(_cint(imsh)), C.byref(_cdouble(tol)),
                C.byref(_cint(int(maxit))), C.byref(_cint(isd)), _ptr(bi), mc, C.byref(niter),
                C.byref(r0), C.byref(r2), C.byref(m))
        self._check(rc, allow=(_capi.ENOTCONV,))
        return niter.value, r0.value, r2.value, m.value, rc

    def proj_setup(self, space: int, mmx: int = 8):
        """Empty projection space `space` and give it room for mmx vectors."""
        self._check(self._L.nekgpu_proj_setup(C.byref(self._h), C.byref(_cint(space)),
                                              C.byref(_cint(mmx))))

    def proj_count(self, space: int) -> int:
        m = _cint(0)
        self._check(self._L.nekgpu_proj_count(C.byref(self._h), C.byref(_cint(space)), C.byref(m)))
        return m.value

    def hmholtz(self, name, u, rhs, h1, h2, mask, mult, imsh, tli, maxit, isd, binv, maxcg=900):
        """name is accepted for signature parity (the reference uses it only for
        the pressure branch and log lines).  rhs is dssum'd and masked in place."""
        del name
        fn = self._L.nekgpu_hmholtz_dev if _is_dev(u) else self._L.nekgpu_hmholtz
        return self._solve(fn, u, rhs, h1, h2, mask, mult, imsh, tli, maxit, isd, binv, maxcg)

    def axhelm_adjoint_h1(self, gh1, lam, u):
        """gh1 = d(lam^T A(h1) u)/dh1 per local point (dJ/dh1 = -gh1 for the adjoint lam)."""
        fn = self._L.nekgpu_axhelm_adjoint_h1_dev if _is_dev(u) else self._L.nekgpu_axhelm_adjoint_h1
        self._check(fn(C.byref(self._h), _ptr(gh1), _ptr(lam), _ptr(u)))
        return gh1

    def cggo_adjoint(self, lam, g, h1, h2, mask, mult, imsh, tin, maxit, isd, binv, maxcg=900):
        """Adjoint solve A lam = g (device arrays; the operator is symmetric)."""
        return self._solve(self._L.nekgpu_cggo_adjoint_dev, lam, g, h1, h2, mask, mult, imsh, tin,
                           maxit, isd, binv, maxcg)

    def _solve_mixed(self, fn, a, b, h1, h2, mask, mult, imsh, tol, maxit, isd, binv, inner_tol):
        no, ni, r0, r2 = _cint(0), _cint(0), _cdouble(0), _cdouble(0)
        rc = fn(C.byref(self._h), _ptr(a), _ptr(b), _ptr(h1), _ptr(h2), _ptr(mask), _ptr(mult),
                C.byref(_cint(imsh)), C.byref(_cdouble(tol)), C.byref(_cint(int(maxit))),
                C.byref(_cint(isd)), _ptr(binv),
                None if inner_tol is None else C.byref(_cdouble(inner_tol)), C.byref(no),
                C.byref(ni), C.byref(r0), C.byref(r2))
        self._check(rc, allow=(_capi.ENOTCONV,))
        return no.value, ni.value, r0.value, r2.value, rc

    def cggo_mixed(self, x, f, h1, h2, mask, mult, imsh, tin, maxit, isd, binv, inner_tol=None):
        """FP32-inner / FP64-defect-correction form of cggo (device arrays).
        inner_tol None takes the library's default for the mixed mode.  Returns (outer steps, inner iterations, rbn0, rbn2, status)."""
        if not _is_dev(x):
            raise TypeError("cggo_mixed takes device arrays")
        return self._solve_mixed(self._L.nekgpu_cggo_mixed_dev, x, f, h1, h2, mask, mult, imsh,
                                 tin, maxit, isd, binv, inner_tol)

    def cggo_mixed_multi(self, xs, fs, h1, h2, masks, mult, imsh, tin, maxit, isd, binv,
                         inner_tol=None):
        """Several fields sharing h1, h2, mult, binv (device arrays; one x, f
        and mask per field) in one fused mixed solve.  Returns a dict of
        per-field lists: nouter, ninner, rbn0, rbn2, status."""
        nf = len(xs)
        if not (len(fs) == len(masks) == nf) or not 1 <= nf <= _capi.MULTI_MAX:
            raise ValueError("one x, f and mask per field, at most MULTI_MAX fields")
        for t in list(xs) + list(fs) + list(masks):
            if not _is_dev(t):
                raise TypeError("cggo_mixed_multi takes device arrays")
        arr = lambda ts: (C.c_void_p * nf)(*[t.data_ptr() for t in ts])
        no, ni = (C.c_int * nf)(), (C.c_int * nf)()
        r0, r2, st = (C.c_double * nf)(), (C.c_double * nf)(), (C.c_int * nf)()
        rc = self._L.nekgpu_cggo_mixed_multi_dev(
            C.byref(self._h), C.byref(_cint(nf)), arr(xs), arr(fs), _ptr(h1), _ptr(h2),
            arr(masks), _ptr(mult), C.byref(_cint(imsh)), C.byref(_cdouble(tin)),
            C.byref(_cint(int(maxit))), C.byref(_cint(isd)), _ptr(binv),
            None if inner_tol is None else C.byref(_cdouble(inner_tol)), no, ni, r0, r2, st)
        self._check(rc)
        return dict(nouter=list(no), ninner=list(ni), rbn0=list(r0), rbn2=list(r2),
                    status=list(st))

    def hmholtz_mixed(self, name, u, rhs, h1, h2, mask, mult, imsh, tli, maxit, isd, binv,
                      inner_tol=None):
        """hmholtz with the mixed-precision solve (host arrays)."""
        del name
        return self._solve_mixed(self._L.nekgpu_hmholtz_mixed, u, rhs, h1, h2, mask, mult, imsh,
                                 tli, maxit, isd, binv, inner_tol)


class NekGpuBatch:
    """Many independent problems solved together (nekgpu_batch_*).

    add() takes one problem's mesh like NekGpu.setup(); solve() takes lists of
    torch float64 CUDA tensors, one per problem in the order added."""

    def __init__(self, device: int = 0):
        self._L = _capi.load()
        self._b = C.c_int64(0)
        rc = self._L.nekgpu_batch_create(C.byref(_cint(device)), C.byref(self._b))
        if rc:
            raise _capi.NekGpuError(rc, self.last_error())
        self.sizes = []
        self._keep = []

    def last_error(self) -> str:
        buf = C.create_string_buffer(1024)
        self._L.nekgpu_batch_last_error(C.byref(self._b), buf, C.byref(_cint(1024)))
        return buf.value.decode(errors="replace")

    def add(self, lx1, nel, D, g, bm1, glo_num) -> int:
        n = lx1 ** 3 * nel
        dxm1 = np.ascontiguousarray(np.asarray(D, dtype=np.float64).T)
        g = np.ascontiguousarray(np.asarray(g, dtype=np.float64).reshape(6, n))
        bm1 = np.ascontiguousarray(bm1, dtype=np.float64)
        glo = np.ascontiguousarray(glo_num, dtype=np.int64)
        idx = _cint(0)
        gp = [g[q].ctypes.data_as(C.c_void_p) for q in range(6)]
        rc = self._L.nekgpu_batch_add(C.byref(self._b), C.byref(_cint(lx1)), C.byref(_cint(nel)),
                                      dxm1.ctypes.data_as(C.c_void_p), *gp,
                                      bm1.ctypes.data_as(C.c_void_p),
                                      glo.ctypes.data_as(C.c_void_p), C.byref(idx))
        if rc:
            raise _capi.NekGpuError(rc, self.last_error())
        self.sizes.append(n)
        return idx.value

    def solve(self, x, f, h1, h2, mask, mult, binv, tin=-1e-10, maxit=10 ** 6, mixed=False,
              inner_tol=None):
        """mixed: False/0 FP64; True/1 FP32 inner PCG with residual replacement;
        2 restarted FP32 inner PCG.  inner_tol None takes the library default.
        Returns a dict of per-problem lists: niter, nouter, rbn0, rbn2, status."""
        np_ = len(self.sizes)
        arr = lambda ts: (C.c_void_p * np_)(*[t.data_ptr() for t in ts])
        for ts in (x, f, h1, h2, mask, mult, binv):
            if len(ts) != np_:
                raise ValueError("one array per problem is required")
            for t in ts:
                _ptr(t)  # type / device checks
        niter = (C.c_int * np_)()
        nouter = (C.c_int * np_)()
        r0 = (C.c_double * np_)()
        r2 = (C.c_double * np_)()
        st = (C.c_int * np_)()
        rc = self._L.nekgpu_batch_solve_dev(
            C.byref(self._b), C.byref(_cint(np_)), arr(x), arr(f), arr(h1), arr(h2), arr(mask),
            arr(mult), arr(binv), C.byref(_cdouble(tin)), C.byref(_cint(int(maxit))),
            C.byref(_cint(int(mixed))),
            None if inner_tol is None else C.byref(_cdouble(inner_tol)), niter, nouter, r0, r2, st)
        if rc:
            raise _capi.NekGpuError(rc, self.last_error())
        return dict(niter=list(niter), nouter=list(nouter), rbn0=list(r0), rbn2=list(r2),
                    status=list(st))

    def shape(self, precision: int = 0):
        """Operator block size in use for the batch: (threads, tuned ms)."""
        t, ms = _cint(0), _cdouble(0)
        rc = self._L.nekgpu_batch_shape(C.byref(self._b), C.byref(_cint(precision)), C.byref(t),
                                        C.byref(ms))
        if rc:
            raise _capi.NekGpuError(rc, self.last_error())
        return t.value, ms.value

    def operator_forms(self):
        """FP32 operator body per order: {lx1: 1 TMA-staged, 0 plain} for the
        orders timed so far."""
        forms = (C.c_int * (_capi.MAX_LX1 + 1))()
        rc = self._L.nekgpu_batch_operator_forms(C.byref(self._b), forms)
        if rc:
            raise _capi.NekGpuError(rc, self.last_error())
        return {nx: v for nx, v in enumerate(forms) if v >= 0}

    def set_shape(self, precision: int, threads: int):
        """Pin the operator block size (128 or 256; 0 returns to tuning)."""
        rc = self._L.nekgpu_batch_set_shape(C.byref(self._b), C.byref(_cint(precision)),
                                            C.byref(_cint(threads)))
        if rc:
            raise _capi.NekGpuError(rc, self.last_error())

    def set_persistent(self, on: bool = True):
        """One persistent cooperative launch per batch segment (default), or
        three graph-replayed launches per iteration."""
        rc = self._L.nekgpu_batch_set_persistent(C.byref(self._b), C.byref(_cint(int(bool(on)))))
        if rc:
            raise _capi.NekGpuError(rc, self.last_error())

    def close(self):
        if getattr(self, "_b", None) is not None and self._b.value:
            self._L.nekgpu_batch_destroy(C.byref(self._b))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
