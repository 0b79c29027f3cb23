"""Mixed precision: FP32 inner PCG inside FP64 defect correction, against the
FP64 oracle on the same seeded mesh and right-hand side.

Both forms of the defect correction are run: mode 1 (default) keeps one FP32
PCG and replaces its residual by the FP64 one each time it has dropped by
inner_tol; mode 0 starts a fresh FP32 PCG at every outer step.

Each mode runs with its default inner tolerance (1e-2 for mode 1, 1e-5 for
mode 0).

Pass criteria (per solve):
  * the FP64 residual of the returned x, recomputed by the oracle's operator
    (r = f - mask*dssum(A x), cggo's norm), is <= 1.05 * 1e-10 * rbn0;
  * the error against the oracle's FP64 solution is reported and bounded by
    1e-8 relative (both solutions satisfy the same 1e-10 residual bound; their
    difference is the conditioning of A times that bound, not rounding).
"""
import numpy as np
import pytest

from conftest import rng_unit_vector

pytestmark = pytest.mark.gpu


def fp64_residual_norm(P, x, f, h1, h2):
    ops = P["ops"]
    w = ops.dssum(ops.axhelm(x, h1, h2)) * P["mask"]
    r = f - w
    return np.sqrt(np.sum(P["mult"] * P["binv"] * r * r) / np.sum(P["bm1"]))


@pytest.mark.parametrize("mode", [1, 0])
@pytest.mark.parametrize("case", [
    dict(nx1=10, k=(3, 3, 3), periodic=(False, False, False), h2=0.0, seed=2),   # N=9 Poisson
    dict(nx1=8, k=(3, 4, 3), periodic=(False, True, True), h2=10.0, seed=1),     # Helmholtz, periodic
    dict(nx1=6, k=(2, 2, 2), periodic=(False, False, False), h2=1500.0, seed=3), # velocity-like h2
])
def test_mixed_meets_fp64_tolerance(gpu_lib, oracle, case, mode):
    torch = pytest.importorskip("torch")
    from nek5000_gb300 import _capi
    kx, ky, kz = case["k"]
    P = oracle.box_problem(case["nx1"], kx, ky, kz, periodic=case["periodic"],
                           v=rng_unit_vector(case["seed"]))
    n = P["n"]
    rng = np.random.default_rng(case["seed"])
    f = P["ops"].dssum(P["bm1"] * (P["ops"].dssum(rng.standard_normal(n)) * P["mult"])) * P["mask"]
    h1, h2 = np.ones(n), np.full(n, case["h2"])
    x_ref, it_ref, r0_ref, r2_ref = P["ops"].cggo(f, h1, h2, P["mask"], P["mult"], P["binv"], -1e-10,
                                                  maxcg=10 ** 6)
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    lib.set_option(_capi.OPT_MIXED_MODE, mode)
    dev = lambda a: torch.tensor(a, device="cuda")
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    outer, inner, r0, r2, rc = lib.cggo_mixed(x, dev(f), dev(h1), dev(h2), dev(P["mask"]),
                                              dev(P["mult"]), 1, -1e-10, 10 ** 6, 1, dev(P["binv"]),
                                              inner_tol=None)
    assert rc == 0, lib.last_error()
    xs = x.cpu().numpy()
    assert abs(r0 - r0_ref) <= 1e-12 * r0_ref
    rn = fp64_residual_norm(P, xs, f, h1, h2)
    assert rn <= 1.05e-10 * r0_ref, (rn / r0_ref, outer, inner)
    err = np.linalg.norm(xs - x_ref) / np.linalg.norm(x_ref)
    print(f"mixed mode {mode}: outer {outer} inner {inner} (FP64 cggo {it_ref}), rel. error vs FP64 oracle {err:.2e}")
    assert err <= 1e-8
    assert 2 <= outer <= (12 if mode == 1 else 6)
    if mode == 1:  # the kept search direction: no more FP32 iterations than FP64 ones, +10%
        assert inner <= 1.1 * it_ref + 5, (inner, it_ref)


def test_mixed_host_entry_point(gpu_lib, oracle):
    P = oracle.box_problem(8, 2, 2, 2, v=rng_unit_vector(5))
    n = P["n"]
    rhs = P["bm1"] * (P["ops"].dssum(np.random.default_rng(5).uniform(-1, 1, n)) * P["mult"])
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    u = np.zeros(n)
    r = rhs.copy()
    h1, h2 = np.ones(n), np.zeros(n)
    outer, inner, r0, r2, rc = lib.hmholtz_mixed("TEMP", u, r, h1, h2, P["mask"], P["mult"], 1,
                                                 -1e-10, 10 ** 6, 1, P["binv"])
    u_ref, rhs_ref, it_ref, r0_ref, _ = P["ops"].hmholtz(rhs, h1, h2, P["mask"], P["mult"],
                                                         P["binv"], -1e-10, maxcg=10 ** 6)
    assert rc == 0
    assert np.array_equal(r, rhs_ref)
    assert fp64_residual_norm(P, u, rhs_ref, h1, h2) <= 1.05e-10 * r0_ref


@pytest.mark.parametrize("nx1,k,periodic,h2", [
    (8, (4, 3, 3), (False, True, True), 10.0),
    (4, (5, 4, 3), (False, False, False), 0.0),
    (7, (3, 3, 3), (False, False, False), 0.0),   # odd lx1: the element-local form runs
])
def test_assembled_boundary_layout_matches_element_local_form(gpu_lib, oracle, nx1, k, periodic,
                                                              h2):
    """The residual-replacement solve with its FP32 vectors stored once per
    global node (NEKGPU_OPT_SPLIT 1, the default) and element-locally (0):
    both meet the FP64 tolerance, and their FP32 iteration counts agree to a
    few percent (the same PCG; only the order of its FP32 sums differs)."""
    torch = pytest.importorskip("torch")
    from nek5000_gb300 import _capi
    P = oracle.box_problem(nx1, *k, periodic=periodic, v=rng_unit_vector(31))
    n = P["n"]
    rng = np.random.default_rng(31)
    f = P["ops"].dssum(P["bm1"] * (P["ops"].dssum(rng.standard_normal(n)) * P["mult"])) * P["mask"]
    h1, h2a = np.ones(n), np.full(n, h2)
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    dev = lambda a: torch.tensor(a, device="cuda")
    out = {}
    for split in (1, 0):
        lib.set_option(_capi.OPT_SPLIT, split)
        x = torch.zeros(n, dtype=torch.float64, device="cuda")
        outer, inner, r0, r2, rc = lib.cggo_mixed(x, dev(f), dev(h1), dev(h2a), dev(P["mask"]),
                                                  dev(P["mult"]), 1, -1e-10, 10 ** 6, 1,
                                                  dev(P["binv"]), inner_tol=None)
        assert rc == 0, lib.last_error()
        xs = x.cpu().numpy()
        assert fp64_residual_norm(P, xs, f, h1, h2a) <= 1.05e-10 * r0
        out[split] = (inner, xs)
    (i1, x1), (i0, x0) = out[1], out[0]
    assert abs(i1 - i0) <= max(3, 0.03 * i0), (i1, i0)
    assert np.linalg.norm(x1 - x0) <= 1e-8 * np.linalg.norm(x0)


@pytest.mark.parametrize("nx1,k,periodic,h2", [
    (8, (4, 3, 3), (False, True, True), 10.0),
    (7, (3, 3, 2), (False, False, False), 0.0),
    (10, (2, 3, 2), (False, False, False), 1500.0),
])
def test_face_ordered_layout_matches_natural_order(gpu_lib, oracle, nx1, k, periodic, h2):
    """The residual-replacement solve with its FP32 vectors in the
    face-ordered element layout (NEKGPU_OPT_FACE_ORDER 1, the default) and in
    the natural order (0): both meet the FP64 tolerance and their FP32
    iteration counts agree to a few percent (the same PCG; the FP32 sums run
    in another order)."""
    torch = pytest.importorskip("torch")
    from nek5000_gb300 import _capi
    P = oracle.box_problem(nx1, *k, periodic=periodic, v=rng_unit_vector(33))
    n = P["n"]
    rng = np.random.default_rng(33)
    f = P["ops"].dssum(P["bm1"] * (P["ops"].dssum(rng.standard_normal(n)) * P["mult"])) * P["mask"]
    h1, h2a = np.ones(n), np.full(n, h2)
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    dev = lambda a: torch.tensor(a, device="cuda")
    out = {}
    for fo in (1, 0):
        lib.set_option(_capi.OPT_FACE_ORDER, fo)
        x = torch.zeros(n, dtype=torch.float64, device="cuda")
        outer, inner, r0, r2, rc = lib.cggo_mixed(x, dev(f), dev(h1), dev(h2a), dev(P["mask"]),
                                                  dev(P["mult"]), 1, -1e-10, 10 ** 6, 1,
                                                  dev(P["binv"]), inner_tol=None)
        assert rc == 0, lib.last_error()
        xs = x.cpu().numpy()
        assert fp64_residual_norm(P, xs, f, h1, h2a) <= 1.05e-10 * r0
        out[fo] = (inner, xs)
    (i1, x1), (i0, x0) = out[1], out[0]
    assert abs(i1 - i0) <= max(3, 0.03 * i0), (i1, i0)
    assert np.linalg.norm(x1 - x0) <= 1e-8 * np.linalg.norm(x0)
