"""The oracle's restatement of the stress formulation (oracle/gradops.c:
ref_axsf of core/subs1.f:2031-2116, ref_hmhzsf of :1093-1147) checked by
properties on the CPU: the coupled operator is symmetric and positive on
continuous fields, a rigid translation has no strain (only the h2 B u term
remains), and the solve reaches its tolerance with the true residual equal to
the recurrence's."""
import numpy as np

from conftest import rng_unit_vector


def _problem(oracle, k, seed):
    P = oracle.box_problem(6, *k, v=rng_unit_vector(seed))
    rst, jac = oracle.geom_rst(P["nx1"], P["nel"], P["x"], P["y"], P["z"])
    return P, rst, jac


def test_operator_symmetric_positive_and_strain_free_on_translations(oracle):
    P, rst, jac = _problem(oracle, (2, 2, 2), 173)
    n, ops = P["n"], P["ops"]
    rng = np.random.default_rng(174)
    cont = lambda: ops.dssum(rng.standard_normal(n) * P["mult"])
    u, v = [cont() for _ in range(3)], [cont() for _ in range(3)]
    h1, h2 = 1.0 + 0.1 * np.abs(rng.standard_normal(n)), np.full(n, 2.0)
    au = oracle.axsf(ops, u, h1, h2, rst, jac, P["bm1"])
    av = oracle.axsf(ops, v, h1, h2, rst, jac, P["bm1"])
    a = sum(np.dot(v[c], au[c]) for c in range(3))
    b = sum(np.dot(u[c], av[c]) for c in range(3))
    assert abs(a - b) <= 1e-12 * abs(a)
    assert sum(np.dot(u[c], au[c]) for c in range(3)) > 0
    # a constant velocity: no strain, A u = h2 B u exactly up to rounding
    t = [np.full(n, 0.3), np.full(n, -1.2), np.full(n, 0.7)]
    at = oracle.axsf(ops, t, h1, h2, rst, jac, P["bm1"])
    for c in range(3):
        want = h2 * P["bm1"] * t[c]
        assert np.max(np.abs(at[c] - want)) <= 1e-12 * np.max(np.abs(want))


def test_solve_reaches_its_tolerance(oracle):
    P, rst, jac = _problem(oracle, (3, 3, 2), 175)
    n, ops = P["n"], P["ops"]
    rng = np.random.default_rng(176)
    m = P["mask"]
    r = [ops.dssum(P["bm1"] * rng.standard_normal(n)) for _ in range(3)]
    h1, h2 = 1.0 + 0.1 * np.abs(rng.standard_normal(n)), np.full(n, 20.0)
    vol = float(np.sum(P["bm1"]))
    masks = [m, m, np.ones(n)]
    u, _, it, r0, r2 = oracle.hmhzsf(ops, r, h1, h2, masks, P["mult"], P["binv"], rst, jac,
                                     P["bm1"], vol, 1e-9)
    assert 0 < it < 200 and r2 < 1e-9
    au = oracle.axsf(ops, u, h1, h2, rst, jac, P["bm1"])
    res = [ops.dssum(r[c] * masks[c]) - ops.dssum(au[c] * masks[c]) for c in range(3)]
    rn = np.sqrt(sum(np.sum(res[c] ** 2 * P["binv"] * P["mult"]) for c in range(3)) / vol)
    assert abs(rn - r2) <= 1e-6 * r2
