"""The splitting step's right-hand sides on the device (nekgpu_cresvsp_dev,
nekgpu_cresvsp_weak_dev, nekgpu_crespsp_dev) against the oracle (oracle/gradops.c): bit for bit with
the handle's exact option (every product and sum rounded in the reference's
order), to 1e-12 with the default fused operator; the null-space mean of
crespsp is a block-order sum, so that case is compared to 1e-13."""
import numpy as np
import pytest

from conftest import rng_unit_vector

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("exact", [True, False])
def test_residuals_match_the_oracle(gpu_lib, oracle, exact):
    torch = pytest.importorskip("torch")
    P = oracle.box_problem(6, 3, 2, 2, v=rng_unit_vector(161))
    nx1, nel, n, ops = P["nx1"], P["nel"], P["n"], P["ops"]
    rst, jac = oracle.geom_rst(nx1, nel, P["x"], P["y"], P["z"])
    rng = np.random.default_rng(162)
    rnd = lambda: rng.standard_normal(n)
    v, bf = [rnd() for _ in range(3)], [rnd() for _ in range(3)]
    h1, h2 = 1.0 + 0.1 * np.abs(rnd()), np.abs(rnd())
    vdiff, qtl, pr = 1.0 + 0.1 * np.abs(rnd()), rnd(), rnd()
    vtrans = 1.0 + 0.2 * np.abs(rnd())
    lib = gpu_lib(0)
    lib.setup_xyz(nx1, nel, P["D"], P["wgll"], P["x"], P["y"], P["z"], P["glo_num"])
    lib.set_exact(exact)
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")
    zeros = lambda: torch.zeros(n, dtype=torch.float64, device="cuda")
    cmp = (lambda a, b: np.array_equal(a, b)) if exact else \
        (lambda a, b: np.allclose(a, b, rtol=0, atol=1e-12 * np.abs(b).max()))
    r = [zeros() for _ in range(3)]
    lib.cresvsp(r, [dev(a) for a in v], dev(h1), dev(h2), dev(vdiff), dev(qtl), dev(pr),
                [dev(a) for a in bf])
    want = oracle.cresvsp(ops, v, h1, h2, vdiff, qtl, pr, bf, rst)
    for a, b in zip(r, want):
        assert cmp(a.cpu().numpy(), b)
    for stress in (True, False):  # the weak-gradient form (plan4.f:308)
        r = [zeros() for _ in range(3)]
        lib.cresvsp_weak(r, [dev(a) for a in v], dev(h1), dev(h2), dev(vdiff), dev(qtl),
                         dev(pr), [dev(a) for a in bf], stress=stress)
        want = oracle.cresvsp_weak(ops, v, h1, h2, vdiff, qtl, pr, bf, rst, jac, P["bm1"],
                                   stress=stress)
        for a, b in zip(r, want):
            assert cmp(a.cpu().numpy(), b), stress
    vc = [rnd() for _ in range(3)]  # the current velocity (face terms)
    fbc = rng.integers(0, 4, size=(nel, 6)).astype(np.int32)  # all four face kinds
    for null, faces in ((False, None), (True, None), (False, fbc)):
        respr = zeros()
        lib.crespsp(respr, [dev(a) for a in v], dev(pr), dev(qtl), dev(vdiff), dev(vtrans),
                    [dev(a) for a in bf], dev(P["binv"]), 1.5, null_space=null,
                    v=[dev(a) for a in vc], fbc=faces)
        want = oracle.crespsp(ops, v, pr, qtl, vdiff, vtrans, bf, P["bm1"], P["binv"], 1.5,
                              null, rst, jac, v=vc, fbc=faces)
        got = respr.cpu().numpy()
        if null:
            assert np.allclose(got, want, rtol=0, atol=1e-13 * np.abs(want).max())
        else:
            assert cmp(got, want)


def test_time_integration_bookkeeping_bit_for_bit(gpu_lib, oracle):
    torch = pytest.importorskip("torch")
    P = oracle.box_problem(5, 2, 2, 2, v=rng_unit_vector(163))
    n = P["n"]
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    rng = np.random.default_rng(164)
    r = lambda: rng.standard_normal(n)
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")
    host = lambda t: t.cpu().numpy()
    bf, a1, a2, vt = r(), r(), r(), 1.0 + np.abs(r())
    ab = [1.8, -1.0, 0.2]
    bfd, a1d, a2d = dev(bf), dev(a1), dev(a2)
    lib.makeabf(bfd, a1d, a2d, dev(vt), ab)
    for got, want in zip((bfd, a1d, a2d), oracle.makeabf(bf, a1, a2, vt, np.array(ab))):
        assert np.array_equal(host(got), want)
    v, l1, l2 = r(), r(), r()
    bd = [11 / 6, 3.0, -1.5, 1 / 3]
    bfd = dev(bf)
    lib.makebdf(bfd, dev(v), dev(np.concatenate([l1, l2])), dev(vt), bd, 3, 0.01)
    assert np.array_equal(host(bfd), oracle.makebdf(bf, v, [l1, l2], P["bm1"], vt,
                                                    np.array(bd), 3, 0.01))
    out = torch.zeros(n, dtype=torch.float64, device="cuda")
    lib.sumab(out, dev(v), dev(np.concatenate([l1, l2])), ab, 3)
    assert np.array_equal(host(out), oracle.sumab(v, [l1, l2], np.array(ab), 3))
