"""The FP64 operator with double-float contractions (NEKGPU_OPT_DF): FP64 in
and out, every product and sum of the tensor contractions in pairs of FP32
values with compensated products and sums (axhelm_df.cuh).  It must agree
with the oracle's FP64 operator (ref_axhelm, core/hmholtz.f:72-259) to
1e-13 relative in the max norm, the tolerance of the fused multiply-add FP64
form, on every order lx1 = 2..12 and every coefficient mode; a Jacobi-PCG
solve that uses it must reach the reference's stopping rule with the
oracle's iteration count within 1 and its solution within 1e-10."""
import numpy as np
import pytest

from conftest import rng_unit_vector

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("nx1", [2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12])
def test_df_operator_within_fp64_tolerance(gpu_lib, oracle, nx1):
    from nek5000_gb300 import _capi
    P = oracle.box_problem(nx1, 3, 2, 2, v=rng_unit_vector(60 + nx1))
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    lib.set_option(_capi.OPT_DF, 1)
    n = P["n"]
    rng = np.random.default_rng(61)
    u = rng.standard_normal(n)
    worst = 0.0
    for h1, h2 in ((np.ones(n), np.zeros(n)), (np.ones(n), np.full(n, 10.0)),
                   (np.exp(0.3 * rng.standard_normal(n)), rng.uniform(0, 5, n))):
        au = np.zeros(n)
        lib.axhelm(au, u, h1, h2)
        e = rel(au, P["ops"].axhelm(u, h1, h2))
        worst = max(worst, e)
        assert e < 1e-13, e
    print(f"lx1={nx1}: double-float operator, max rel. difference from the oracle {worst:.2e}")


def test_df_solve_matches_the_oracle(gpu_lib, oracle):
    torch = pytest.importorskip("torch")
    from nek5000_gb300 import _capi
    P = oracle.box_problem(8, 4, 4, 4, periodic=(False, True, True), v=rng_unit_vector(62))
    n = P["n"]
    rng = np.random.default_rng(62)
    f = P["ops"].dssum(P["bm1"] * (P["ops"].dssum(rng.standard_normal(n)) * P["mult"])) * P["mask"]
    h1, h2 = np.ones(n), np.full(n, 10.0)
    x_ref, it_ref, r0_ref, _ = P["ops"].cggo(f, h1, h2, P["mask"], P["mult"], P["binv"], -1e-10,
                                             maxcg=10 ** 6)
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    lib.set_option(_capi.OPT_DF, 1)
    dev = lambda a: torch.tensor(a, device="cuda")
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    it, r0, r2, rc = lib.cggo(x, dev(f), dev(h1), dev(h2), dev(P["mask"]), dev(P["mult"]), 1,
                              -1e-10, 10 ** 6, 1, dev(P["binv"]), maxcg=10 ** 6)
    assert rc == 0
    assert abs(it - it_ref) <= 1, (it, it_ref)
    assert abs(r0 - r0_ref) <= 1e-13 * r0_ref
    err = np.linalg.norm(x.cpu().numpy() - x_ref) / np.linalg.norm(x_ref)
    print(f"double-float PCG: {it} iterations (oracle {it_ref}), rel. error {err:.2e}")
    assert err < 1e-10
