"""The algebraic multigrid coarse solve on the host (no GPU): the hierarchy
the library builds (amg_plan.cpp) for the trilinear finite-element Laplacian
of a box -- the kind of matrix the pressure preconditioner's coarse problem
is -- applied by the oracle's restatement of the reference's V-cycle
(oracle/amg.py: amg_exec, core/crs_amg.c:129-186) and by the library's host
apply must agree, and the cycle must be a usable solver: as a stationary
iteration it contracts the error (by 0.7 or better per cycle), and as a GMRES
preconditioner it reaches 1e-10 in at most 30 iterations, fewer than GMRES
alone."""
import ctypes as C

import numpy as np
import pytest

from amg_util import amg_plan, q1_laplacian


@pytest.fixture(scope="module")
def lib():
    from nek5000_gb300 import _capi, build
    build.build()
    return _capi.load()


@pytest.mark.parametrize("m,seed", [(10, None), (12, 7)])
def test_host_cycle_equals_oracle_and_converges(lib, m, seed):
    from oracle import amg as oamg
    n, A, _ = q1_laplacian(m, dirichlet=True, seed=seed)
    levels, off, perm, h = amg_plan(lib, n, A)
    assert off[-1] == n and sorted(perm.tolist()) == list(range(n))
    assert levels[-1]["nf"] == 1
    Ap = A[perm][:, perm]  # the matrix in the plan's order
    rng = np.random.default_rng(3)
    b = rng.standard_normal(n)
    x_or = oamg.amg_exec(levels, off, b)
    x_h = np.zeros(n)
    bb = b.copy()
    assert lib.nekmesh_amg_apply(C.byref(h), x_h.ctypes.data_as(C.c_void_p),
                                 bb.ctypes.data_as(C.c_void_p)) == 0
    assert np.max(np.abs(x_h - x_or)) <= 1e-12 * np.max(np.abs(x_or))
    # stationary iteration x += B (b - A x): error contraction per cycle
    xs = np.zeros(n)
    x_true = np.linalg.solve(Ap.toarray(), b)
    errs = []
    for _ in range(8):
        xs = xs + oamg.amg_exec(levels, off, b - Ap @ xs)
        errs.append(np.linalg.norm(xs - x_true))
    rate = (errs[-1] / errs[2]) ** (1.0 / 5)
    assert rate < 0.7, (rate, errs)
    # as a GMRES preconditioner: far fewer iterations than without
    spla = pytest.importorskip("scipy.sparse.linalg")
    M = spla.LinearOperator((n, n), matvec=lambda v: oamg.amg_exec(levels, off, v))
    counts = []
    for prec in (M, None):
        its = [0]
        x, info = spla.gmres(Ap, b, M=prec, rtol=1e-10, restart=60, maxiter=400,
                             callback=lambda _r: its.__setitem__(0, its[0] + 1),
                             callback_type="pr_norm")
        assert info == 0
        counts.append(its[0])
    assert counts[0] <= 30 and counts[0] < counts[1], counts
    lib.nekmesh_amg_free(C.byref(h))


def test_null_space_form(lib):
    """crs_solve's null-space step in the oracle: the pinned unknown and the
    mean removal give a zero-mean result that solves the singular system up
    to a constant."""
    from oracle import amg as oamg
    n, A, _ = q1_laplacian(6, dirichlet=False)
    Ared = A[: n - 1, : n - 1]
    levels, off, perm, h = amg_plan(lib, n - 1, Ared.tocsr())
    rng = np.random.default_rng(4)
    v = rng.standard_normal(n)
    v -= v.mean()
    x = oamg.crs_solve(levels, off, perm, v, n, True)
    assert abs(x.sum()) <= 1e-10 * np.abs(x).sum()
    lib.nekmesh_amg_free(C.byref(h))
