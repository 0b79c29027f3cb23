"""Mesh ingestion: the reference's .re2 / .co2 files to the arrays the solve
path takes (python side of include/nekmesh.h; the work is done by the
library's host code).

    M = load_mesh("case.re2", N=7)             # connectivity from coordinates
    M = load_mesh("case.re2", N=7, co2="case.co2")   # or ma2="case.ma2"
    h = NekGpu(0); h.setup(M["lx1"], M["nel"], M["D"], M["g"], M["bm1"], M["glo_num"])

load_mesh returns the same keys as mesh.box_mesh (lx1, nel, n, D, g, bm1,
glo_num, mask, mult, binv, vol, x, y, z, zgll, wgll) plus the file's
boundary conditions.  Elements are mapped from their corners (core/genxyz.f
xyzlin) or, with 'm' midside nodes, quadratically (xyzquad); 's' faces are
made sphere patches (sphsrf) and 'C' edges circular arcs (arcsrf); 'e'
surfaces are refused.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi
from .mesh import deriv_matrix, geometry, gll

DIRICHLET_VELOCITY = ("W  ", "V  ", "v  ")  # wall and prescribed velocity


def _lib():
    return _capi.load()


def _check(rc):
    if rc != 0:
        buf = C.create_string_buffer(512)
        _lib().nekmesh_last_error(buf, C.byref(C.c_int(512)))
        raise _capi.NekGpuError(rc, buf.value.decode(errors="replace"))


def _p(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


def read_re2(path: str) -> dict:
    """Everything a .re2 file holds (core/reader_re2.f): header fields, element
    groups, corners (nel, 2^ndim) in file order, curved sides and every
    boundary-condition section as the reference's dense (cbc, bc) arrays."""
    L = _lib()
    h = C.c_int64(0)
    _check(L.nekmesh_re2_open(str(path).encode(), C.byref(h)))
    try:
        nelgt, ndim, nelgv, wd, nbf = (C.c_int() for _ in range(5))
        ncurve = C.c_int64()
        _check(L.nekmesh_re2_header(C.byref(h), C.byref(nelgt), C.byref(ndim), C.byref(nelgv),
                                    C.byref(wd), C.byref(ncurve), C.byref(nbf)))
        ne, nd, nv = nelgt.value, ndim.value, 1 << ndim.value
        xc, yc = np.zeros((ne, nv)), np.zeros((ne, nv))
        zc = np.zeros((ne, nv)) if nd == 3 else None
        group = np.zeros(ne, dtype=np.int32)
        _check(L.nekmesh_re2_xyz(C.byref(h), _p(xc), _p(yc), _p(zc), _p(group)))
        nc = ncurve.value
        elem, side = np.zeros(nc, dtype=np.int32), np.zeros(nc, dtype=np.int32)
        curve, ctype = np.zeros((nc, 5)), C.create_string_buffer(max(nc, 1))
        _check(L.nekmesh_re2_curves(C.byref(h), _p(elem), _p(side), _p(curve), ctype))
        bcs = []
        nf = 2 * nd
        for f in range(nbf.value):
            cbc = C.create_string_buffer(3 * nf * ne)
            bc = np.zeros((ne, nf, 5))
            _check(L.nekmesh_re2_bc(C.byref(h), C.byref(C.c_int(f)), cbc, _p(bc)))
            raw = cbc.raw.decode("latin-1")
            types = np.array([raw[3 * q:3 * q + 3] for q in range(nf * ne)]).reshape(ne, nf)
            bcs.append((types, bc))
        return dict(nelgt=ne, ndim=nd, nelgv=nelgv.value, wdsize=wd.value, group=group, xc=xc,
                    yc=yc, zc=zc,
                    curves=dict(elem=elem, side=side, curve=curve,
                                ccurve=ctype.raw[:nc].decode("latin-1")),
                    bcs=bcs)
    finally:
        L.nekmesh_re2_close(C.byref(h))


def read_co2(path: str) -> dict:
    """A .co2 connectivity file (core/map2.f read_con): vertex ids (nel, nv)
    in tensor corner order, placed by element id."""
    L = _lib()
    ne, nev, nv = C.c_int(), C.c_int(), C.c_int()
    _check(L.nekmesh_co2_read(str(path).encode(), C.byref(ne), C.byref(nev), C.byref(nv), None))
    vertex = np.zeros((ne.value, nv.value), dtype=np.int64)
    _check(L.nekmesh_co2_read(str(path).encode(), C.byref(ne), C.byref(nev), C.byref(nv),
                              _p(vertex)))
    return dict(nelgt=ne.value, nelgv=nev.value, nv=nv.value, vertex=vertex)


def read_ma2(path: str) -> dict:
    """A .ma2 map file (core/map2.f read_map): vertex ids (nel, nv) and the
    0-based partition of every element."""
    L = _lib()
    ne, nv = C.c_int(), C.c_int()
    _check(L.nekmesh_ma2_read(str(path).encode(), C.byref(ne), C.byref(nv), None, None))
    vertex = np.zeros((ne.value, nv.value), dtype=np.int64)
    part = np.zeros(ne.value, dtype=np.int32)
    _check(L.nekmesh_ma2_read(str(path).encode(), C.byref(ne), C.byref(nv), _p(vertex),
                              _p(part)))
    return dict(nel=ne.value, nv=nv.value, vertex=vertex, part=part)


def write_co2(path: str, vertex, nelgv: int | None = None) -> None:
    vertex = np.ascontiguousarray(vertex, dtype=np.int64)
    ne, nv = vertex.shape
    _check(_lib().nekmesh_co2_write(str(path).encode(), C.byref(C.c_int(ne)),
                                    C.byref(C.c_int(nelgv or ne)), C.byref(C.c_int(nv)),
                                    _p(vertex)))


def connect(xc, yc, zc, cbc=None, bc=None, tol: float = 0.2):
    """Vertex ids (nel, 8), tensor corner order, from the corners (file
    order) and the periodic faces of the first boundary section (the
    reference's gencon algorithm).  Returns (vertex, number of vertices)."""
    xc, yc, zc = (np.ascontiguousarray(a, dtype=np.float64) for a in (xc, yc, zc))
    ne = xc.shape[0]
    vertex = np.zeros((ne, 8), dtype=np.int64)
    nvert = C.c_int64()
    cbuf = None
    if cbc is not None:
        cbuf = C.create_string_buffer("".join(np.asarray(cbc).reshape(-1)).encode("latin-1"))
        bc = np.ascontiguousarray(bc, dtype=np.float64)
    _check(_lib().nekmesh_connect(C.byref(C.c_int(ne)), C.byref(C.c_int(3)), _p(xc), _p(yc),
                                  _p(zc), cbuf, _p(bc) if cbc is not None else None,
                                  C.byref(C.c_double(tol)), _p(vertex), C.byref(nvert)))
    return vertex, nvert.value


def setvert3d(nx: int, vertex):
    """glo_num of every GLL point (core/navier8.f setvert3d); returns
    (glo_num, number of ids)."""
    vertex = np.ascontiguousarray(vertex, dtype=np.int64)
    ne = vertex.shape[0]
    glo = np.zeros(ne * nx ** 3, dtype=np.int64)
    ngv = C.c_int64()
    _check(_lib().nekmesh_setvert3d(C.byref(C.c_int(nx)), C.byref(C.c_int(ne)), _p(vertex),
                                    _p(glo), C.byref(ngv)))
    return glo, ngv.value


def h1mg_levels(lx1: int):
    """Polynomial orders of the pressure preconditioner's levels, coarsest
    first (h1mg_setup_mg_nx, core/hsmg.f:2272)."""
    o = np.zeros(4, dtype=np.int32)
    lmax = _lib().nekmesh_h1mg_levels(C.byref(C.c_int(int(lx1))), _p(o))
    if lmax < 0:
        _check(lmax)
    return [int(v) for v in o[:lmax]]


def face_types(nx: int, glo, mask):
    """Pressure face types (6 per element: 0 shared, 1 Dirichlet, 2 Neumann)
    read from a numbering and mask (nekmesh_face_types)."""
    glo = np.ascontiguousarray(glo, dtype=np.int64).reshape(-1)
    mask = np.ascontiguousarray(mask, dtype=np.float64).reshape(-1)
    nel = glo.size // nx ** 3
    fbc = np.zeros(6 * nel, dtype=np.int32)
    _check(_lib().nekmesh_face_types(C.byref(C.c_int(nx)), C.byref(C.c_int(nel)), _p(glo),
                                     _p(mask), _p(fbc)))
    return fbc.reshape(nel, 6)


def h1mg_level(nx1: int, glo, x, y, z, level: int, mask=None, fbc=None):
    """The preconditioner's setup of one level (nekmesh_h1mg_level): returns
    (nx, mask, rwt, swt, lengths[nel, 3, 3])."""
    glo = np.ascontiguousarray(glo, dtype=np.int64).reshape(-1)
    nel = glo.size // nx1 ** 3
    f64 = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
    xs, ys, zs, m = f64(x), f64(y), f64(z), f64(mask)
    fb = None if fbc is None else np.ascontiguousarray(fbc, dtype=np.int32).reshape(-1)
    nx = C.c_int(0)
    npt = nx1 ** 3 * nel  # large enough for every level
    out = [np.zeros(npt) for _ in range(3)]
    lengths = np.zeros(9 * nel)
    _check(_lib().nekmesh_h1mg_level(C.byref(C.c_int(nx1)), C.byref(C.c_int(nel)), _p(glo),
                                     _p(xs), _p(ys), _p(zs), _p(m), _p(fb),
                                     C.byref(C.c_int(int(level))), C.byref(nx), *[_p(o) for o in out],
                                     _p(lengths)))
    k = nx.value ** 3 * nel
    return nx.value, out[0][:k], out[1][:k], out[2][:k], lengths.reshape(nel, 3, 3)


def fdm1d(n: int, lbc: int, rbc: int, ll: float, lm: float, lr: float):
    """One 1-D fast-diagonalisation operator (nekmesh_fdm1d): (S, lam)."""
    nl = n + 3
    s = np.zeros(nl * nl)
    lam = np.zeros(nl)
    _check(_lib().nekmesh_fdm1d(C.byref(C.c_int(n)), C.byref(C.c_int(lbc)), C.byref(C.c_int(rbc)),
                                C.byref(C.c_double(ll)), C.byref(C.c_double(lm)),
                                C.byref(C.c_double(lr)), _p(s), _p(lam)))
    return s.reshape(nl, nl).T.copy(), lam  # S[i, j]: component i of vector j


def xxt_factor(A, xyz):
    """X with A^-1 = X X^T for a symmetric positive definite scipy/numpy
    matrix A whose unknowns sit at xyz (n, 3) (nekmesh_xxt_factor); returns
    (perm, X) with X dense, rows and columns in the nested-dissection order
    perm (perm[k] = the unknown numbered k)."""
    import scipy.sparse as sp
    A = sp.csr_matrix(A)
    n = A.shape[0]
    ptr = np.ascontiguousarray(A.indptr, dtype=np.int64)
    idx = np.ascontiguousarray(A.indices, dtype=np.int32)
    val = np.ascontiguousarray(A.data, dtype=np.float64)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
    nnz = C.c_int64(0)
    args = [C.byref(C.c_int64(n)), _p(ptr), _p(idx), _p(val), _p(xyz), C.byref(nnz)]
    _check(_lib().nekmesh_xxt_factor(*args, None, None, None, None))
    perm = np.zeros(n, dtype=np.int32)
    cptr = np.zeros(n + 1, dtype=np.int64)
    cidx = np.zeros(nnz.value, dtype=np.int32)
    cval = np.zeros(nnz.value)
    _check(_lib().nekmesh_xxt_factor(*args, _p(perm), _p(cptr), _p(cidx), _p(cval)))
    X = np.zeros((n, n))
    for j in range(n):
        X[cidx[cptr[j]:cptr[j + 1]], j] = cval[cptr[j]:cptr[j + 1]]
    return perm, X


def check_p_bc(nx: int, cbc, glo):
    """Single-element periodicity ('p  ' on two opposite faces of an element:
    core/navier8.f check_p_bc), applied to glo in place."""
    cbuf = C.create_string_buffer("".join(np.asarray(cbc).reshape(-1)).encode("latin-1"))
    _check(_lib().nekmesh_check_p_bc(C.byref(C.c_int(nx)), C.byref(C.c_int(len(cbc))), cbuf,
                                     _p(glo)))
    return glo


def xyzlin(nx: int, zgll, xc, yc, zc):
    """GLL coordinates (nel*nx^3 each) of straight-sided elements."""
    xc, yc, zc = (np.ascontiguousarray(a, dtype=np.float64) for a in (xc, yc, zc))
    zgll = np.ascontiguousarray(zgll, dtype=np.float64)
    ne = xc.shape[0]
    out = [np.zeros(ne * nx ** 3) for _ in range(3)]
    _check(_lib().nekmesh_xyzlin(C.byref(C.c_int(nx)), C.byref(C.c_int(ne)), _p(zgll), _p(xc),
                                 _p(yc), _p(zc), *(_p(o) for o in out)))
    return out


def genxyz(nx: int, zgll, xc, yc, zc, curves=None):
    """GLL coordinates (nel*nx^3 each): straight-sided elements by the
    trilinear map, elements with 'm' midside nodes by the reference's
    quadratic map (xyzquad), 's' faces made sphere patches (sphsrf), 'C'
    edges bent into arcs (arcsrf); curves as read_re2 returns them."""
    xc, yc, zc = (np.ascontiguousarray(a, dtype=np.float64) for a in (xc, yc, zc))
    zgll = np.ascontiguousarray(zgll, dtype=np.float64)
    ne = xc.shape[0]
    out = [np.zeros(ne * nx ** 3) for _ in range(3)]
    nc = 0 if curves is None else len(curves["elem"])
    if nc:
        elem = np.ascontiguousarray(curves["elem"], dtype=np.int32)
        side = np.ascontiguousarray(curves["side"], dtype=np.int32)
        cv = np.ascontiguousarray(curves["curve"], dtype=np.float64)
        ctype = curves["ccurve"].encode("latin-1")
    else:
        elem = side = cv = None
        ctype = None
    _check(_lib().nekmesh_genxyz(C.byref(C.c_int(nx)), C.byref(C.c_int(ne)), _p(zgll), _p(xc),
                                 _p(yc), _p(zc), C.byref(C.c_int64(nc)), _p(elem), _p(side),
                                 _p(cv), ctype, *(_p(o) for o in out)))
    return out


# Points of each preprocessor face (1-based face number) of an element, as
# (ix, iy, iz) selections on the (iz, iy, ix) element array.
def _face_points(face: int, nx: int):
    s = slice(None)
    return {1: (s, 0, s), 2: (s, s, nx - 1), 3: (s, nx - 1, s), 4: (s, s, 0),
            5: (0, s, s), 6: (nx - 1, s, s)}[face]


def _dsop(glo, u, op):
    """Host direct-stiffness sum ('+') or product ('*') over shared points."""
    out = u.copy()
    shared = glo > 0
    ids = glo[shared]
    uniq, inv = np.unique(ids, return_inverse=True)
    if op == "+":
        acc = np.bincount(inv, weights=u[shared], minlength=len(uniq))
    else:
        acc = np.ones(len(uniq))
        np.multiply.at(acc, inv, u[shared])
    out[shared] = acc[inv]
    return out


def load_mesh(re2: str, N: int, co2: str | None = None, field: int = 0,
              dirichlet=DIRICHLET_VELOCITY, tol: float = 0.2, ma2: str | None = None) -> dict:
    """The operator data of a .re2 mesh at polynomial order N (lx1 = N+1):
    GLL coordinates (genxyz), geometric factors and mass, global numbering
    (the .co2 file when given, else connectivity from the corners), the mask
    of boundary-condition section `field` (zero on faces whose type is in
    `dirichlet`, then multiplied across shared points as dsop '*'),
    multiplicity and inverse mass."""
    R = read_re2(re2)
    if R["ndim"] != 3:
        raise ValueError("only 3-D meshes are served")
    nx = N + 1
    ne = R["nelgt"]
    zg, wg = gll(nx)
    D = deriv_matrix(zg)
    x, y, z = genxyz(nx, zg, R["xc"], R["yc"], R["zc"], R["curves"])
    shape = (ne, nx, nx, nx)
    g, bm1, jac = geometry(x.reshape(shape), y.reshape(shape), z.reshape(shape), D, wg)
    cbc, bc = R["bcs"][field] if R["bcs"] else (None, None)
    if co2 is not None:
        C2 = read_co2(co2)
        if C2["nelgt"] != ne or C2["nv"] != 8:
            raise ValueError("the .co2 file does not match the mesh")
        vertex = C2["vertex"]
    elif ma2 is not None:
        M2 = read_ma2(ma2)
        if M2["nel"] != ne or M2["nv"] != 8:
            raise ValueError("the .ma2 file does not match the mesh")
        vertex = M2["vertex"]
    else:
        vertex, _ = connect(R["xc"], R["yc"], R["zc"], cbc, bc, tol)
    glo, ngv = setvert3d(nx, vertex)
    if cbc is not None:
        check_p_bc(nx, cbc, glo)
    n = ne * nx ** 3
    mask = np.ones(shape)
    if cbc is not None:
        for e, f in zip(*np.nonzero(np.isin(cbc, list(dirichlet)))):
            mask[(e,) + _face_points(int(f) + 1, nx)] = 0.0
    mask = _dsop(glo, mask.reshape(-1), "*")
    mult = 1.0 / _dsop(glo, np.ones(n), "+")
    binv = 1.0 / _dsop(glo, bm1, "+")
    return dict(lx1=nx, nel=ne, n=n, D=D, zgll=zg, wgll=wg, g=g, bm1=bm1, jac=jac,
                glo_num=glo, ngv=ngv, vertex=vertex, mask=mask, mult=mult, binv=binv,
                vol=float(bm1.sum()), x=x, y=y, z=z, cbc=cbc, bc=bc, group=R["group"])
