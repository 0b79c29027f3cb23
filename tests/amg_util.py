"""Test matrices for the algebraic multigrid coarse solve: the trilinear
(Q1) finite-element Laplacian of a box of m^3 elements -- the kind of matrix
the pressure preconditioner's coarse problem is -- and the plan arrays the
library's host inspection entry points return."""
import ctypes as C

import numpy as np


def q1_element_stiffness(h=1.0, aniso=(1.0, 1.0, 1.0)):
    """8 x 8 stiffness of a trilinear hex of edge h (vertex v = i + 2 j + 4 k)."""
    g = np.array([-1.0, 1.0]) / np.sqrt(3.0)
    K = np.zeros((8, 8))
    for a in g:
        for b in g:
            for c in g:
                r, s, t = (a + 1) / 2, (b + 1) / 2, (c + 1) / 2
                grads = []
                for v in range(8):
                    i, j, k = v & 1, (v >> 1) & 1, (v >> 2) & 1
                    fr = (r if i else 1 - r)
                    fs = (s if j else 1 - s)
                    ft = (t if k else 1 - t)
                    dr = (1 if i else -1) * fs * ft
                    ds = fr * (1 if j else -1) * ft
                    dt = fr * fs * (1 if k else -1)
                    grads.append(np.array([dr, ds, dt]) / h)
                w = (h / 2) ** 3
                for p in range(8):
                    for q in range(8):
                        K[p, q] += w * np.dot(np.array(aniso) * grads[p], grads[q])
    return K


def q1_laplacian(m, dirichlet=True, seed=None):
    """CSR (ptr, idx, val) and COO of the assembled Q1 Laplacian on an m^3
    box of unit-size elements; Dirichlet: boundary vertices removed.  With a
    seed the element coefficients vary (0.5 .. 2)."""
    n1 = m + 1
    K = q1_element_stiffness()
    rng = np.random.default_rng(seed) if seed is not None else None
    vid = -np.ones((n1, n1, n1), dtype=np.int64)
    cnt = 0
    for k in range(n1):
        for j in range(n1):
            for i in range(n1):
                if dirichlet and (i in (0, m) or j in (0, m) or k in (0, m)):
                    continue
                vid[i, j, k] = cnt
                cnt += 1
    rows, cols, vals = [], [], []
    for ez in range(m):
        for ey in range(m):
            for ex in range(m):
                sc = rng.uniform(0.5, 2.0) if rng is not None else 1.0
                ids = [vid[ex + (v & 1), ey + ((v >> 1) & 1), ez + ((v >> 2) & 1)]
                       for v in range(8)]
                for p in range(8):
                    for q in range(8):
                        if ids[p] >= 0 and ids[q] >= 0:
                            rows.append(ids[p])
                            cols.append(ids[q])
                            vals.append(sc * K[p, q])
    rows, cols, vals = np.array(rows), np.array(cols), np.array(vals)
    import scipy.sparse as sp
    A = sp.csr_matrix((vals, (rows, cols)), shape=(cnt, cnt))
    A.sort_indices()
    return cnt, A, (rows.astype(np.int32), cols.astype(np.int32), vals)


def amg_plan(L, n, A):
    """Build the library's hierarchy of A (host) and return (levels, off,
    perm, plan id) with the levels as scipy CSR matrices for oracle.amg."""
    import scipy.sparse as sp
    ptr = np.ascontiguousarray(A.indptr, dtype=np.int64)
    idx = np.ascontiguousarray(A.indices, dtype=np.int32)
    val = np.ascontiguousarray(A.data, dtype=np.float64)
    h = C.c_int64(0)
    rc = L.nekmesh_amg_setup(C.byref(C.c_int64(n)), ptr.ctypes.data_as(C.c_void_p),
                             idx.ctypes.data_as(C.c_void_p), val.ctypes.data_as(C.c_void_p),
                             C.byref(h))
    assert rc == 0
    nl = C.c_int(0)
    assert L.nekmesh_amg_layout(C.byref(h), C.byref(nl), None, None) == 0
    off = np.zeros(nl.value + 1, dtype=np.int64)
    perm = np.zeros(n, dtype=np.int64)
    assert L.nekmesh_amg_layout(C.byref(h), C.byref(nl), off.ctypes.data_as(C.c_void_p),
                                perm.ctypes.data_as(C.c_void_p)) == 0
    levels = []
    P = lambda a: a.ctypes.data_as(C.c_void_p)
    for lv in range(nl.value):
        sz = np.zeros(6, dtype=np.int64)
        m, rho = C.c_int(0), C.c_double(0)
        assert L.nekmesh_amg_level(C.byref(h), C.byref(C.c_int(lv)), P(sz), C.byref(m),
                                   C.byref(rho), *([None] * 13)) == 0
        nf, nc = int(sz[0]), int(sz[1])
        dff = np.zeros(max(nf, 1))
        arrs = []
        for rows_, nnz in ((nf, sz[2]), (nc, sz[3]), (nf, sz[4]), (nf, sz[5])):
            arrs += [np.zeros(rows_ + 1, dtype=np.int64), np.zeros(max(nnz, 1), dtype=np.int32),
                     np.zeros(max(nnz, 1))]
        assert L.nekmesh_amg_level(C.byref(h), C.byref(C.c_int(lv)), P(sz), C.byref(m),
                                   C.byref(rho), P(dff), *[P(a) for a in arrs]) == 0
        mk = lambda p_, i_, v_, r_, c_: sp.csr_matrix(
            (v_[:p_[-1]], i_[:p_[-1]], p_), shape=(r_, c_))
        lvd = dict(nf=nf, nc=nc, m=m.value, rho=rho.value, dff=dff[:nf])
        if nc > 0:
            lvd.update(W=mk(*arrs[0:3], nf, nc), WT=mk(*arrs[3:6], nc, nf),
                       AFP=mk(*arrs[6:9], nf, nc), AFF=mk(*arrs[9:12], nf, nf))
        levels.append(lvd)
    return levels, off, perm, h
