"""The algebraic multigrid coarse solve on the device (amg.cu): the
reference's crs_amg interface (crs_amg_setup / crs_amg_solve,
core/crs_amg.c:531, :186) through nekgpu_crs_amg_setup / _solve_dev, against
the oracle's restatement of the V-cycle (oracle/amg.py) on the hierarchy the
library's host setup builds for the same matrix (nekmesh_amg_*): the device
sums in another order, so results agree to 1e-12 relative.  Then the
pressure preconditioner with its coarse solve switched to AMG
(NEKGPU_OPT_COARSE = 1, the reference's param(40) = 1): GMRES and flexible
CG still converge to 1e-10, in at most 1.5 times the iterations (plus 2) of
the exact X X^T coarse solve."""
import ctypes as C

import numpy as np
import pytest

from amg_util import amg_plan, q1_laplacian
from conftest import rng_unit_vector

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m,seed,null", [(10, None, False), (13, 5, False), (7, None, True)])
def test_crs_amg_solve_matches_the_oracle(gpu_lib, m, seed, null):
    torch = pytest.importorskip("torch")
    from nek5000_gb300 import _capi
    from oracle import amg as oamg
    L = _capi.load()
    n, A, (ai, aj, av) = q1_laplacian(m, dirichlet=not null, seed=seed)
    Ar = A[: n - 1, : n - 1].tocsr() if null else A
    levels, off, perm, h = amg_plan(L, Ar.shape[0], Ar)
    lib = gpu_lib(0)
    hh = lib._h
    rc = L.nekgpu_crs_amg_setup(C.byref(hh), C.byref(C.c_int64(n)), C.byref(C.c_int64(ai.size)),
                                C.c_void_p(ai.ctypes.data), C.c_void_p(aj.ctypes.data),
                                C.c_void_p(av.ctypes.data), C.byref(C.c_int(int(null))))
    assert rc == 0, lib.last_error()
    rng = np.random.default_rng(9)
    for _ in range(2):  # two calls in a row: no state leaks between them
        v = rng.standard_normal(n)
        if null:
            v -= v.mean()
        want = oamg.crs_solve(levels, off, perm, v, n, null)
        x = torch.zeros(n, dtype=torch.float64, device="cuda")
        rc = L.nekgpu_crs_amg_solve_dev(C.byref(hh), C.c_void_p(x.data_ptr()),
                                        C.c_void_p(torch.tensor(v, device="cuda").data_ptr()))
        assert rc == 0, lib.last_error()
        got = x.cpu().numpy()
        assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    L.nekmesh_amg_free(C.byref(h))


@pytest.mark.parametrize("solver", ["gmres", "flex_cg"])
def test_pressure_solve_with_amg_coarse_solve(gpu_lib, oracle, solver):
    torch = pytest.importorskip("torch")
    from nek5000_gb300 import _capi
    P = oracle.box_problem(6, 4, 4, 3, v=rng_unit_vector(121))
    n = P["n"]
    h1, h2 = np.ones(n), np.zeros(n)
    f = P["ops"].dssum(P["bm1"] * np.random.default_rng(122).standard_normal(n)) * P["mask"]
    dev = lambda a: torch.tensor(a, device="cuda")
    its = {}
    for coarse in (0, 1):
        lib = gpu_lib(0)
        lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
        lib.set_option(_capi.OPT_COARSE, coarse)
        lib.h1mg_setup(P["x"], P["y"], P["z"], P["glo_num"], mask=P["mask"])
        x = dev(f)
        fn = lib.hmh_gmres if solver == "gmres" else lib.hmh_flex_cg
        it, d0, rn, rc = fn(x, dev(h1), dev(h2), dev(P["mult"]), dev(P["mask"]), -1e-10,
                            maxit=2000)
        assert rc == 0 and rn < 1e-10 * d0
        xs = x.cpu().numpy()
        r = f - P["ops"].dssum(P["ops"].axhelm(xs, h1, h2)) * P["mask"]
        assert np.linalg.norm(r) <= 1e-8 * np.linalg.norm(f)
        its[coarse] = it
        lib.close()
    assert its[1] <= 1.5 * its[0] + 2, its
