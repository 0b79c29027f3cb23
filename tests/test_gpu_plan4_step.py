"""The whole splitting step (plan4, core/plan4.f:2-97) on the device:
nek5000_gb300.plan4.SplittingStep strings the library's entry points together
in the reference's order (makef, sumab, lagvel, bcdirvc, crespsp, the
projected pressure solve, ortho, cresvsp, ophinv; with the stress
formulation cresvsp_weak and the coupled hmhzsf) and is compared after every
one of six steps (the BDF/extrapolation order ramping from 1 to 3) with the
oracle's restatement of the same step (oracle/plan4.py), on a deformed box
with walls on every face and a divergence-free initial field that vanishes on
them.  Both solve their pressure and velocity systems to an absolute
tolerance of 1e-10 in cggo's norm, so the fields agree to that level
amplified by the conditioning: the test asks for 1e-8 relative."""
import numpy as np
import pytest

from conftest import rng_unit_vector

pytestmark = pytest.mark.gpu


def _initial(P):
    x, y, z = P["x"], P["y"], P["z"]
    pi = np.pi
    g = np.sin(pi * z)
    vx = g * 2 * pi * np.sin(pi * x) ** 2 * np.sin(pi * y) * np.cos(pi * y)
    vy = -g * 2 * pi * np.sin(pi * x) * np.cos(pi * x) * np.sin(pi * y) ** 2
    return [vx * P["mask"], vy * P["mask"], np.zeros(P["n"])]


@pytest.mark.parametrize("convection,stress", [(True, False), (False, False), (True, True)])
def test_splitting_step_matches_the_oracle(gpu_lib, oracle, convection, stress):
    torch = pytest.importorskip("torch")
    from oracle.plan4 import SplittingStepOracle
    from nek5000_gb300.plan4 import SplittingStep
    P = oracle.box_problem(6, 3, 3, 3, v=rng_unit_vector(171))
    n = P["n"]
    lib = gpu_lib(0)
    lib.setup_xyz(P["nx1"], P["nel"], P["D"], P["wgll"], P["x"], P["y"], P["z"], P["glo_num"])
    vtrans, vdiff, qtl = np.ones(n), np.full(n, 0.01), np.zeros(n)
    kw = dict(dt=1e-3, tolhv=1e-10, tolpdf=1e-10, convection=convection, stress=stress)
    ref = SplittingStepOracle(P, P["mask"], np.ones(n), vtrans, vdiff, qtl, **kw)
    dev = SplittingStep(lib, P["bm1"], P["binv"], P["mask"], np.ones(n), P["mult"], vtrans,
                        vdiff, qtl, **kw)
    v0 = _initial(P)
    ref.v = [a.copy() for a in v0]
    dev.set_velocity(*v0)
    for step in range(6):
        itp_r, itv_r = ref.step()
        itp, itv = dev.step()
        assert abs(itp - itp_r) <= 3 and all(abs(a - b) <= 1 for a, b in zip(itv, itv_r)), \
            (step, itp, itp_r, itv, itv_r)
        for c in range(3):
            got, want = dev.v[c].cpu().numpy(), ref.v[c]
            scale = max(np.abs(want).max(), 1e-30)
            assert np.abs(got - want).max() <= 1e-8 * max(scale, np.abs(v0[0]).max()), (step, c)
        got = dev.pr.cpu().numpy()
        assert np.abs(got - ref.pr).max() <= 1e-8 * np.abs(ref.pr).max(), step
