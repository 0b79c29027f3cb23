"""The pressure solve's GMRES (nekgpu_hmh_gmres_dev) against the oracle's
restatement of hmh_gmres with the same Jacobi stand-in preconditioner.

The GPU's weighted dot products are block sums (the oracle's are serial), so
the Arnoldi coefficients differ in the last bits: iteration counts must agree
to +-2, the initial residual norm to 1e-12, and the solutions, both stopped
at 1e-10 of the initial residual norm, to 1e-8 relative."""
import numpy as np
import pytest

from conftest import rng_unit_vector

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case,kmax", [("dirichlet", 30), ("periodic", 30), ("periodic", 7),
                                       ("null", 30)])
def test_gmres_matches_the_oracle(gpu_lib, oracle, case, kmax):
    torch = pytest.importorskip("torch")
    if case == "dirichlet":
        P = oracle.box_problem(8, 3, 3, 3, v=rng_unit_vector(71))
        h2v = 0.0
    elif case == "periodic":
        P = oracle.box_problem(6, 3, 4, 3, periodic=(False, True, True), v=rng_unit_vector(72))
        h2v = 10.0
    else:  # pure Neumann, h2 = 0: the constant null space (ortho)
        P = oracle.box_problem(6, 3, 3, 2, dirichlet=(False,) * 6, v=rng_unit_vector(73))
        h2v = 0.0
    n, ops = P["n"], P["ops"]
    h1, h2 = np.ones(n), np.full(n, h2v)
    f = ops.dssum(P["bm1"] * np.random.default_rng(74).standard_normal(n)) * P["mask"]
    null = case == "null"
    if null:
        f = f - np.sum(f * P["mult"]) / np.sum(P["mult"])
    x_ref, it_ref, d0_ref, rn_ref = ops.gmres(f, h1, h2, P["mult"], P["mask"], -1e-10,
                                              maxit=20000, m=kmax, null_space=null)
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    dev = lambda a: torch.tensor(a, device="cuda")
    x = dev(f)
    it, d0, rn, rc = lib.hmh_gmres(x, dev(h1), dev(h2), dev(P["mult"]), dev(P["mask"]), -1e-10,
                                   maxit=20000, kmax=kmax, null_space=null)
    assert rc == 0
    assert abs(it - it_ref) <= 2, (it, it_ref)
    assert abs(d0 - d0_ref) <= 1e-12 * d0_ref
    assert rn < 1e-10 * d0
    xh = x.cpu().numpy()
    assert np.linalg.norm(xh - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
    r = f - ops.dssum(ops.axhelm(xh, h1, h2)) * P["mask"]
    assert np.sqrt(np.sum(r * r * P["mult"]) / np.sum(P["bm1"])) <= 2e-10 * d0
    if null:
        assert abs(np.mean(xh)) < 1e-13
    print(case, kmax, "iterations", it, "oracle", it_ref)


def test_gmres_reports_the_iteration_cap(gpu_lib, oracle):
    torch = pytest.importorskip("torch")
    from nek5000_gb300 import _capi
    P = oracle.box_problem(6, 2, 2, 2, v=rng_unit_vector(75))
    n = P["n"]
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    dev = lambda a: torch.tensor(a, device="cuda")
    f = P["ops"].dssum(P["bm1"] * np.random.default_rng(76).standard_normal(n)) * P["mask"]
    it, d0, rn, rc = lib.hmh_gmres(dev(f), dev(np.ones(n)), dev(np.zeros(n)), dev(P["mult"]),
                                   dev(P["mask"]), -1e-10, maxit=5, kmax=30)
    assert rc == _capi.ENOTCONV and it == 5 and rn > 1e-10 * d0


def test_gmres_host_entry_point(gpu_lib, oracle):
    """nekgpu_hmh_gmres (host arrays) returns what the device entry point does."""
    torch = pytest.importorskip("torch")
    P = oracle.box_problem(6, 2, 3, 2, v=rng_unit_vector(77))
    n = P["n"]
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    f = P["ops"].dssum(P["bm1"] * np.random.default_rng(78).standard_normal(n)) * P["mask"]
    h1, h2 = np.ones(n), np.full(n, 3.0)
    xh = f.copy()
    ith, d0h, rnh, rch = lib.hmh_gmres(xh, h1, h2, P["mult"], P["mask"], -1e-10, kmax=20)
    dev = lambda a: torch.tensor(a, device="cuda")
    xd = dev(f)
    itd, d0d, rnd, rcd = lib.hmh_gmres(xd, dev(h1), dev(h2), dev(P["mult"]), dev(P["mask"]),
                                       -1e-10, kmax=20)
    assert rch == rcd == 0 and ith == itd and d0h == d0d and rnh == rnd
    assert np.array_equal(xh, xd.cpu().numpy())


@pytest.mark.parametrize("case", ["dirichlet", "periodic", "null"])
def test_flex_cg_matches_the_oracle(gpu_lib, oracle, case):
    """nekgpu_hmh_flex_cg_dev against the oracle's hmh_flex_cg restatement:
    iterations to +-2, div0 to 1e-12, solutions to 1e-8 relative."""
    torch = pytest.importorskip("torch")
    if case == "dirichlet":
        P = oracle.box_problem(8, 3, 3, 3, v=rng_unit_vector(81))
        h2v = 0.0
    elif case == "periodic":
        P = oracle.box_problem(6, 3, 4, 3, periodic=(False, True, True), v=rng_unit_vector(82))
        h2v = 10.0
    else:
        P = oracle.box_problem(6, 3, 3, 2, dirichlet=(False,) * 6, v=rng_unit_vector(83))
        h2v = 0.0
    n, ops = P["n"], P["ops"]
    h1, h2 = np.ones(n), np.full(n, h2v)
    f = ops.dssum(P["bm1"] * np.random.default_rng(84).standard_normal(n)) * P["mask"]
    null = case == "null"
    if null:
        f = f - np.sum(f * P["mult"]) / np.sum(P["mult"])
    x_ref, it_ref, d0_ref, rn_ref = ops.flex_cg(f, h1, h2, P["mult"], P["mask"], -1e-10,
                                                maxit=20000, null_space=null)
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    dev = lambda a: torch.tensor(a, device="cuda")
    x = dev(f)
    it, d0, rn, rc = lib.hmh_flex_cg(x, dev(h1), dev(h2), dev(P["mult"]), dev(P["mask"]),
                                     -1e-10, maxit=20000, null_space=null)
    assert rc == 0
    assert abs(it - it_ref) <= 2, (it, it_ref)
    assert abs(d0 - d0_ref) <= 1e-12 * d0_ref
    assert rn < 1e-10 * d0
    xh = x.cpu().numpy()
    assert np.linalg.norm(xh - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
    if null:
        assert abs(np.mean(xh)) < 1e-13
    print(case, "flex cg iterations", it, "oracle", it_ref)


def test_flex_cg_host_entry_point_and_zero_rhs(gpu_lib, oracle):
    """nekgpu_hmh_flex_cg (host arrays) returns what the device entry point
    does; a zero right-hand side gives x = 0 after no iteration; the cap is
    reported."""
    torch = pytest.importorskip("torch")
    from nek5000_gb300 import _capi
    P = oracle.box_problem(6, 2, 3, 2, v=rng_unit_vector(85))
    n = P["n"]
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    f = P["ops"].dssum(P["bm1"] * np.random.default_rng(86).standard_normal(n)) * P["mask"]
    h1, h2 = np.ones(n), np.full(n, 3.0)
    xh = f.copy()
    ith, d0h, rnh, rch = lib.hmh_flex_cg(xh, h1, h2, P["mult"], P["mask"], -1e-10)
    dev = lambda a: torch.tensor(a, device="cuda")
    xd = dev(f)
    itd, d0d, rnd, rcd = lib.hmh_flex_cg(xd, dev(h1), dev(h2), dev(P["mult"]), dev(P["mask"]),
                                         -1e-10)
    assert rch == rcd == 0 and ith == itd and d0h == d0d and rnh == rnd
    assert np.array_equal(xh, xd.cpu().numpy())
    z = np.zeros(n)
    it0, d00, _, rc0 = lib.hmh_flex_cg(z, h1, h2, P["mult"], P["mask"], -1e-10)
    assert rc0 == 0 and it0 == 0 and d00 == 0.0 and not np.any(z)
    it5, d05, rn5, rc5 = lib.hmh_flex_cg(f.copy(), h1, h2, P["mult"], P["mask"], -1e-10, maxit=5)
    assert rc5 == _capi.ENOTCONV and it5 == 5 and rn5 > 1e-10 * d05
