"""The package's box mesher produces the data the reference's setup would:
checked against the oracle's restatement of speclib / coef / setvert3d."""
import numpy as np
import pytest

from conftest import rng_unit_vector


def groups(glo):
    order = np.lexsort((np.arange(len(glo)), glo))
    g = glo[order]
    keep = g != 0
    order, g = order[keep], g[keep]
    cuts = np.flatnonzero(np.diff(g)) + 1
    return sorted(tuple(x) for x in np.split(order, cuts))


@pytest.mark.parametrize("N", [1, 2, 4, 7, 9, 11])
def test_gll_and_derivative_match_oracle(oracle, N):
    from nek5000_gb300 import mesh
    z, w = mesh.gll(N + 1)
    zr, wr = oracle.zwgll(N + 1)
    assert np.max(np.abs(z - zr)) < 4e-16
    assert np.max(np.abs(w - wr)) < 1e-15
    D = mesh.deriv_matrix(z)
    Dr, _ = oracle.dgll(zr)
    assert np.max(np.abs(D - Dr)) < 2e-13 * N * N


@pytest.mark.parametrize("case", [
    dict(N=7, k=(4, 4, 4), periodic=(False, False, False)),
    dict(N=5, k=(3, 4, 5), periodic=(False, True, True)),
    dict(N=3, k=(2, 3, 3), periodic=(False, False, True)),
])
def test_box_mesh_matches_oracle(oracle, case):
    from nek5000_gb300 import mesh
    v = rng_unit_vector(1)
    kx, ky, kz = case["k"]
    M = mesh.box_mesh(case["N"], kx, ky, kz, periodic=case["periodic"], v=v)
    P = oracle.box_problem(case["N"] + 1, kx, ky, kz, periodic=case["periodic"], v=v)
    assert np.max(np.abs(M["g"] - P["g"])) <= 1e-12 * np.max(np.abs(P["g"]))
    assert np.max(np.abs(M["bm1"] - P["bm1"])) <= 1e-12 * np.max(P["bm1"])
    assert np.array_equal(M["mask"], P["mask"])
    assert np.array_equal(M["mult"], P["mult"])
    assert np.max(np.abs(M["binv"] - P["binv"])) <= 1e-12 * np.max(P["binv"])
    assert groups(M["glo_num"]) == groups(P["glo_num"])
