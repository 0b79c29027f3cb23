"""Projection onto previous solutions (hsolve, core/navier4.f:562-1188) against
the oracle's restatement, over a sequence of solves like a time-stepping run.

The right-hand sides vary smoothly (f0 + sin(0.3 t) f1 + 0.01 t^2 f2 plus a
small seeded perturbation), so the space fills up to its capacity (8) and the
O(nm) update with its Givens rotations runs; h2 changes at step 6, which
makes project1 rebuild B = A X and re-orthonormalise the space fully (CGS2).
Per step the GPU must report the oracle's iteration count (+-1: the dot
products are tree sums, not the reference's serial ones) and the same space
size, and its solution must agree with the oracle's to 1e-10 relative (the
oracle's own spread across rank counts is ~1e-15 here; the bound leaves room
for a one-iteration difference of a CG stopped at an absolute 1e-9).
"""
import numpy as np
import pytest

from conftest import rng_unit_vector

pytestmark = pytest.mark.gpu

STEPS = 10


def _rhs_sequence(P, seed=7):
    ops = P["ops"]
    n = P["n"]
    rng = np.random.default_rng(seed)
    f0, f1, f2 = (rng.standard_normal(n) for _ in range(3))
    for t in range(STEPS):
        g = np.random.default_rng(100 + t).standard_normal(n)
        f = f0 + np.sin(0.3 * t) * f1 + 0.01 * t * t * f2 + 1e-3 * g
        h2 = np.full(n, 100.0 if t < 6 else 120.0)
        yield t, P["bm1"] * ops.dssum(f * P["mult"]), h2


@pytest.mark.parametrize("exact", [False, True])
def test_hsolve_sequence_matches_oracle(gpu_lib, oracle, exact):
    torch = pytest.importorskip("torch")
    P = oracle.box_problem(8, 3, 3, 3, v=rng_unit_vector(11))
    n = P["n"]
    proj = oracle.Projection(P["ops"], 8)
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    lib.set_exact(exact)
    dev = lambda a: torch.tensor(a, device="cuda")
    h1 = np.ones(n)
    sizes = []
    for t, rhs, h2 in _rhs_sequence(P):
        u_ref, r_ref, it_ref, r0_ref, r2_ref = proj.hsolve(rhs, h1, h2, P["mask"], P["mult"],
                                                           P["binv"], 1e-9)
        u = torch.zeros(n, dtype=torch.float64, device="cuda")
        r = dev(rhs)
        it, r0, r2, m, rc = lib.hsolve("VELX", u, r, dev(h1), dev(h2), dev(P["mask"]),
                                       dev(P["mult"]), 1, 1e-9, 10 ** 6, 1, dev(P["binv"]), space=2,
                                       maxcg=10 ** 6)
        assert rc == 0
        assert m == proj.m, (t, m, proj.m)
        assert abs(it - it_ref) <= 1, (t, it, it_ref)
        assert abs(r0 - r0_ref) <= 1e-9 * max(r0_ref, 1e-300), (t, r0, r0_ref)
        err = np.linalg.norm(u.cpu().numpy() - u_ref) / np.linalg.norm(u_ref)
        assert err <= 1e-10, (t, err)
        # the projected right-hand side handed to cggo
        rerr = np.linalg.norm(r.cpu().numpy() - r_ref) / np.linalg.norm(r_ref)
        assert rerr <= 1e-10, (t, rerr)
        sizes.append((m, it))
    print("hsolve (m, niter) per step:", sizes)
    assert max(m for m, _ in sizes) == 8       # the space filled up
    assert sizes[-1][1] < sizes[0][1]          # and projection pays off
    assert lib.proj_count(2) == sizes[-1][0]
    assert lib.proj_count(0) == 0              # other spaces untouched


def test_hsolve_host_entry_point_and_reset(gpu_lib, oracle):
    P = oracle.box_problem(6, 2, 3, 2, v=rng_unit_vector(12))
    n = P["n"]
    proj = oracle.Projection(P["ops"], 4)
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    lib.proj_setup(0, 4)
    h1 = np.ones(n)
    for t, rhs, h2 in _rhs_sequence(P, seed=8):
        if t == 6:
            break
        u_ref, r_ref, it_ref, _, _ = proj.hsolve(rhs, h1, h2, P["mask"], P["mult"], P["binv"],
                                                 1e-9)
        u = np.zeros(n)
        r = rhs.copy()
        it, r0, r2, m, rc = lib.hsolve("TEMP", u, r, h1, h2, P["mask"], P["mult"], 1, 1e-9,
                                       10 ** 6, 1, P["binv"], space=0, maxcg=10 ** 6)
        assert rc == 0 and m == proj.m and abs(it - it_ref) <= 1
        assert np.linalg.norm(u - u_ref) <= 1e-10 * np.linalg.norm(u_ref)
        assert np.linalg.norm(r - r_ref) <= 1e-10 * np.linalg.norm(r_ref)
    assert lib.proj_count(0) == 4  # capacity 4 reached
    lib.proj_setup(0, 4)           # emptied
    assert lib.proj_count(0) == 0
