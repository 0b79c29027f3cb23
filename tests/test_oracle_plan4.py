"""The oracle's splitting step (oracle/plan4.py) on the CPU: identities the
step must keep whatever its arithmetic order.  Without convection or forcing
the kinetic energy of a wall-bounded flow decays at every step; the velocity
stays zero on the walls; ortho leaves the pressure with zero mean (the
closed box's pressure is defined up to a constant).  Both velocity forms:
three Helmholtz solves, and the stress formulation's coupled one."""
import numpy as np
import pytest

from conftest import rng_unit_vector


@pytest.mark.parametrize("stress", [False, True])
def test_oracle_step_identities(oracle, stress):
    from oracle.plan4 import SplittingStepOracle
    P = oracle.box_problem(5, 2, 2, 2, v=rng_unit_vector(172))
    n = P["n"]
    x, y, z = P["x"], P["y"], P["z"]
    pi = np.pi
    g = np.sin(pi * z)
    v0 = [g * 2 * pi * np.sin(pi * x) ** 2 * np.sin(pi * y) * np.cos(pi * y) * P["mask"],
          -g * 2 * pi * np.sin(pi * x) * np.cos(pi * x) * np.sin(pi * y) ** 2 * P["mask"],
          np.zeros(n)]
    S = SplittingStepOracle(P, P["mask"], np.ones(n), np.ones(n), np.full(n, 0.05),
                            np.zeros(n), 1e-3, convection=False, stress=stress)
    S.v = [a.copy() for a in v0]
    ke = [sum(np.sum(a * a * P["bm1"] * P["mult"]) for a in S.v)]
    for _ in range(4):
        S.step()
        ke.append(sum(np.sum(a * a * P["bm1"] * P["mult"]) for a in S.v))
        for a in S.v:
            assert np.abs(a[P["mask"] == 0]).max() == 0.0
        assert abs(np.sum(S.pr)) <= 1e-12 * n * np.abs(S.pr).max()
    assert all(b < a for a, b in zip(ke, ke[1:])), ke
