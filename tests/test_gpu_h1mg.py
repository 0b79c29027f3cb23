"""The pressure preconditioner h1mg_solve on the device (h1mg.cu) against
the oracle's restatement (oracle/h1mg.c): one application z = M r, and
hmh_gmres / hmh_flex_cg preconditioned by it.

Tolerances: the device sums in a different order and its 1-D eigenvectors
come from the library's own host setup, so z agrees to 1e-10 relative;
Krylov iteration counts to +-1 and solutions to 1e-8 relative."""
import numpy as np
import pytest

from conftest import rng_unit_vector

pytestmark = pytest.mark.gpu

CASES = {
    "dirichlet": dict(args=(8, 3, 3, 2), kw={}, h2=0.0, null=False),
    "periodic": dict(args=(6, 3, 4, 3), kw=dict(periodic=(False, True, True)), h2=10.0, null=False),
    "null": dict(args=(6, 3, 3, 2), kw=dict(dirichlet=(False,) * 6), h2=0.0, null=True),
    "lx4": dict(args=(4, 3, 3, 3), kw={}, h2=0.0, null=False),
}


def _problem(oracle, case, seed):
    c = CASES[case]
    P = oracle.box_problem(*c["args"], v=rng_unit_vector(seed), **c["kw"])
    fbc = oracle.face_types(P["nx1"], P["nel"], P["glo_num"], P["mask"])
    mg = oracle.H1mg(P["ops"], P["x"], P["y"], P["z"], fbc, P["vertex"], null_space=c["null"])
    return P, mg, c


def _lib(gpu_lib, P, null):
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    lib.h1mg_setup(P["x"], P["y"], P["z"], P["glo_num"], mask=P["mask"], null_space=null)
    return lib


@pytest.mark.parametrize("case", list(CASES))
def test_h1mg_apply_matches_the_oracle(gpu_lib, oracle, case):
    torch = pytest.importorskip("torch")
    P, mg, c = _problem(oracle, case, 111)
    n = P["n"]
    r = P["ops"].dssum(P["bm1"] * np.random.default_rng(112).standard_normal(n)) * P["mask"]
    zo, ro = mg.solve(r)
    lib = _lib(gpu_lib, P, c["null"])
    rd = torch.tensor(r, device="cuda")
    zd = torch.zeros(n, dtype=torch.float64, device="cuda")
    lib.h1mg_apply(zd, rd)
    z = zd.cpu().numpy()
    assert np.abs(z - zo).max() <= 1e-10 * np.abs(zo).max()
    assert np.array_equal(rd.cpu().numpy(), ro)
    # linear in the right-hand side
    zd2 = torch.zeros_like(zd)
    lib.h1mg_apply(zd2, torch.tensor(2.0 * r, device="cuda"))
    assert np.allclose(zd2.cpu().numpy(), 2.0 * z, rtol=0, atol=1e-12 * np.abs(z).max())


@pytest.mark.parametrize("case", ["dirichlet", "periodic", "null"])
@pytest.mark.parametrize("solver", ["gmres", "flex_cg"])
def test_preconditioned_pressure_solve(gpu_lib, oracle, case, solver):
    torch = pytest.importorskip("torch")
    P, mg, c = _problem(oracle, case, 113)
    n, ops, null = P["n"], P["ops"], c["null"]
    h1, h2 = np.ones(n), np.full(n, c["h2"])
    f = ops.dssum(P["bm1"] * np.random.default_rng(114).standard_normal(n)) * P["mask"]
    if null:
        f = f - np.sum(f * P["mult"]) / np.sum(P["mult"])
    x_ref, it_ref, d0_ref, _ = getattr(ops, solver)(f, h1, h2, P["mult"], P["mask"], -1e-10,
                                                     maxit=2000, null_space=null, mg=mg)
    lib = _lib(gpu_lib, P, null)
    dev = lambda a: torch.tensor(a, device="cuda")
    x = dev(f)
    fn = lib.hmh_gmres if solver == "gmres" else lib.hmh_flex_cg
    it, d0, rn, rc = fn(x, dev(h1), dev(h2), dev(P["mult"]), dev(P["mask"]), -1e-10, maxit=2000,
                        null_space=null)
    assert rc == 0
    assert abs(it - it_ref) <= 1, (it, it_ref)
    assert abs(d0 - d0_ref) <= 1e-12 * d0_ref
    assert rn < 1e-10 * d0
    xh = x.cpu().numpy()
    assert np.linalg.norm(xh - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
    print(case, solver, "iterations", it, "oracle", it_ref)


def test_free_returns_to_jacobi_and_errors(gpu_lib, oracle):
    torch = pytest.importorskip("torch")
    from nek5000_gb300 import _capi
    P, mg, c = _problem(oracle, "dirichlet", 115)
    n, ops = P["n"], P["ops"]
    h1, h2 = np.ones(n), np.zeros(n)
    f = ops.dssum(P["bm1"] * np.random.default_rng(116).standard_normal(n)) * P["mask"]
    _, it_j, _, _ = ops.gmres(f, h1, h2, P["mult"], P["mask"], -1e-10, maxit=20000)
    lib = _lib(gpu_lib, P, False)
    lib.h1mg_free()
    dev = lambda a: torch.tensor(a, device="cuda")
    it, _, _, rc = lib.hmh_gmres(dev(f), dev(h1), dev(h2), dev(P["mult"]), dev(P["mask"]), -1e-10,
                                 maxit=20000)
    assert rc == 0 and abs(it - it_j) <= 2
    with pytest.raises(_capi.NekGpuError) as ei:
        lib.h1mg_apply(dev(f), dev(f))
    assert ei.value.code == _capi.ENOSETUP
