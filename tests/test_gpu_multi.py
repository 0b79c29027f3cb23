"""Several fields of one mesh solved together by the mixed solve
(nekgpu_cggo_mixed_multi_dev): the velocity components of a time step.

Each field is a separate FP32 PCG with its own mask, scalars and residual
replacements; the fused kernels only share the reads of the geometric
factors, diagonal, mass and weights.  So every field must return exactly what
the single-field mixed solve returns (every launch shape of the single-field
kernels gives the same result), and meet the FP64 tolerance against the oracle.
"""
import numpy as np
import pytest

from conftest import rng_unit_vector

pytestmark = pytest.mark.gpu

DIRICHLET = [None,                                         # every face
             (True, True, False, False, False, False),     # x faces only
             (True, True, True, True, True, False)]        # all but z+


def _fields(oracle, nx1, k, seed):
    P0 = oracle.box_problem(nx1, *k, v=rng_unit_vector(seed))
    masks = [oracle.box_problem(nx1, *k, dirichlet=dr, v=rng_unit_vector(seed))["mask"]
             for dr in DIRICHLET]
    n = P0["n"]
    ops = P0["ops"]
    rng = np.random.default_rng(seed)
    fs = [ops.dssum(P0["bm1"] * (ops.dssum(rng.standard_normal(n)) * P0["mult"])) * m
          for m in masks]
    return P0, masks, fs


@pytest.mark.parametrize("nx1", [8, 7])
def test_multi_field_mixed_solve(gpu_lib, oracle, nx1):
    torch = pytest.importorskip("torch")
    P, masks, fs = _fields(oracle, nx1, (3, 3, 2), 41)
    n = P["n"]
    x_, y_, z_ = P["x"], P["y"], P["z"]
    h1 = np.exp(0.2 * np.sin(3 * x_) * np.cos(2 * y_ + z_))  # per-point h1
    h2 = np.full(n, 10.0)
    dev = lambda a: torch.tensor(a, device="cuda")
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    xs = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in fs]
    res = lib.cggo_mixed_multi(xs, [dev(f) for f in fs], dev(h1), dev(h2), [dev(m) for m in masks],
                               dev(P["mult"]), 1, -1e-10, 10 ** 6, 1, dev(P["binv"]))
    assert res["status"] == [0, 0, 0], res
    ops = P["ops"]
    for c, (f, m) in enumerate(zip(fs, masks)):
        x = xs[c].cpu().numpy()
        w = ops.dssum(ops.axhelm(x, h1, h2)) * m
        r = f - w
        rn = np.sqrt(np.sum(P["mult"] * P["binv"] * r * r) / np.sum(P["bm1"]))
        assert rn <= 1.05e-10 * res["rbn0"][c], (c, rn / res["rbn0"][c])
        x_ref, it_ref, _, _ = ops.cggo(f, h1, h2, m, P["mult"], P["binv"], -1e-10, maxcg=10 ** 6)
        assert np.linalg.norm(x - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
        # the single-field mixed solve of the same field: identical
        x1 = torch.zeros(n, dtype=torch.float64, device="cuda")
        no, ni, r0, r2, rc = lib.cggo_mixed(x1, dev(f), dev(h1), dev(h2), dev(m), dev(P["mult"]), 1,
                                            -1e-10, 10 ** 6, 1, dev(P["binv"]))
        assert rc == 0
        assert (no, ni) == (res["nouter"][c], res["ninner"][c]), (c, no, ni, res)
        assert torch.equal(x1, xs[c]), c
    print("multi-field: outer", res["nouter"], "inner", res["ninner"])


def test_multi_field_argument_errors(gpu_lib, oracle):
    torch = pytest.importorskip("torch")
    from nek5000_gb300 import _capi
    P, masks, fs = _fields(oracle, 6, (2, 2, 2), 42)
    n = P["n"]
    dev = lambda a: torch.tensor(a, device="cuda")
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    xs = [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(4)]
    with pytest.raises(ValueError):
        lib.cggo_mixed_multi(xs, [dev(fs[0])] * 4, dev(np.ones(n)), dev(np.ones(n)),
                             [dev(masks[0])] * 4, dev(P["mult"]), 1, -1e-10, 100, 1, dev(P["binv"]))
    # a singular field (no Dirichlet point, h2 = 0) is refused per field
    ones = np.ones(n)
    res = lib.cggo_mixed_multi(xs[:2], [dev(fs[0]), dev(fs[0] * masks[0])], dev(ones),
                               dev(np.zeros(n)), [dev(masks[0]), dev(ones)], dev(P["mult"]), 1,
                               -1e-10, 10 ** 6, 1, dev(P["binv"]))
    assert res["status"] == [0, _capi.EINVAL]
