"""The stress formulation's coupled velocity operator and solve on the device
(nekgpu_axhmsf_dev, nekgpu_hmhzsf_dev) against the oracle's restatement
(oracle/gradops.c: ref_axsf of core/subs1.f:2031-2116, ref_hmhzsf of
:1093-1147 with chktcgs and cggosf): the operator bit for bit (both round
every product and sum in the reference's order); the solve with the same
iteration count within 1 and the solution within 1e-10 (its dot products are
block-order sums on the device, serial in the oracle)."""
import numpy as np
import pytest

from conftest import rng_unit_vector

pytestmark = pytest.mark.gpu


def _setup(gpu_lib, oracle, nx1, k, seed):
    P = oracle.box_problem(nx1, *k, v=rng_unit_vector(seed))
    rst, jac = oracle.geom_rst(P["nx1"], P["nel"], P["x"], P["y"], P["z"])
    lib = gpu_lib(0)
    lib.setup_xyz(P["nx1"], P["nel"], P["D"], P["wgll"], P["x"], P["y"], P["z"], P["glo_num"])
    return P, rst, jac, lib


@pytest.mark.parametrize("nx1", [3, 6, 8])
def test_stress_operator_bit_for_bit(gpu_lib, oracle, nx1):
    torch = pytest.importorskip("torch")
    P, rst, jac, lib = _setup(gpu_lib, oracle, nx1, (3, 2, 2), 171 + nx1)
    n = P["n"]
    rng = np.random.default_rng(172)
    u = [rng.standard_normal(n) for _ in range(3)]
    h1 = 1.0 + 0.2 * np.abs(rng.standard_normal(n))
    h2 = np.abs(rng.standard_normal(n))
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")
    au = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    lib.axhmsf(au, [dev(a) for a in u], dev(h1), dev(h2))
    want = oracle.axsf(P["ops"], u, h1, h2, rst, jac, P["bm1"])
    for a, b in zip(au, want):
        assert np.array_equal(a.cpu().numpy(), b)


@pytest.mark.parametrize("case", ["walls", "mixed"])
def test_stress_solve_matches_the_oracle(gpu_lib, oracle, case):
    torch = pytest.importorskip("torch")
    P, rst, jac, lib = _setup(gpu_lib, oracle, 6, (3, 3, 2), 175)
    n, ops = P["n"], P["ops"]
    rng = np.random.default_rng(176)
    m = P["mask"]
    if case == "walls":
        masks = [m, m, m]
    else:  # the third component free on the faces the other two hold
        masks = [m, m, np.ones(n)]
    r = [ops.dssum(P["bm1"] * rng.standard_normal(n)) for _ in range(3)]
    h1 = 1.0 + 0.1 * np.abs(rng.standard_normal(n))
    h2 = np.full(n, 20.0)
    vol = float(np.sum(P["bm1"]))
    tol = 1e-9
    u_ref, r_ref, it_ref, r0_ref, r2_ref = oracle.hmhzsf(ops, r, h1, h2, masks, P["mult"],
                                                         P["binv"], rst, jac, P["bm1"], vol, tol)
    assert it_ref > 0
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")
    u = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(3)]
    rd = [dev(a) for a in r]
    it, r0, r2, rc = lib.hmhzsf(u, rd, dev(h1), dev(h2), [dev(a) for a in masks], dev(P["mult"]),
                                dev(P["binv"]), tol)
    assert rc == 0
    assert abs(it - it_ref) <= 1, (it, it_ref)
    assert abs(r0 - r0_ref) <= 1e-12 * r0_ref
    assert r2 < tol
    num = sum(np.sum((u[c].cpu().numpy() - u_ref[c]) ** 2) for c in range(3))
    den = sum(np.sum(u_ref[c] ** 2) for c in range(3))
    err = np.sqrt(num / den)
    print(f"stress solve ({case}): {it} iterations (oracle {it_ref}), rel. error {err:.2e}")
    assert err < 1e-10
