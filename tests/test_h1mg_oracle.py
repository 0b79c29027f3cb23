"""The oracle's restatement of the pressure preconditioner h1mg_solve
(oracle/h1mg.c): level orders, face types, the coarse Galerkin solve and
GMRES / flexible CG preconditioned by it."""
import numpy as np
import pytest

from conftest import rng_unit_vector


def test_level_orders(oracle):
    """h1mg_setup_mg_nx (core/hsmg.f:2272-2338) for lx1 = 3..14: orders
    1, min(3, mgn2(lx1)), lx1 - 1 (two levels at lx1 = 4)."""
    got = {lx: oracle.h1mg_levels(lx) for lx in range(3, 15)}
    want = {3: [1, 2, 2], 4: [1, 3], 5: [1, 2, 4], 6: [1, 3, 5], 7: [1, 3, 6], 8: [1, 3, 7]}
    for lx in range(9, 15):
        want[lx] = [1, 3, lx - 1]
    assert got == want


def test_face_types(oracle):
    """Interior and periodic faces 0, masked boundary faces 1, unmasked 2."""
    P = oracle.box_problem(4, 3, 3, 2, periodic=(False, True, False),
                           dirichlet=(True, False, False, False, False, True))
    fbc = oracle.face_types(P["nx1"], P["nel"], P["glo_num"], P["mask"]).reshape(2, 3, 3, 6)
    # [ez, ey, ex, face]; r-: x = 0 Dirichlet; r+: x = 1 Neumann; s: periodic;
    # t-: z = 0 Neumann; t+: z = 1 Dirichlet
    assert (fbc[:, :, 0, 0] == 1).all() and (fbc[:, :, 1:, 0] == 0).all()
    assert (fbc[:, :, 2, 1] == 2).all() and (fbc[:, :, :2, 1] == 0).all()
    assert (fbc[..., 2] == 0).all() and (fbc[..., 3] == 0).all()
    assert (fbc[0, :, :, 4] == 2).all() and (fbc[1, :, :, 4] == 0).all()
    assert (fbc[1, :, :, 5] == 1).all() and (fbc[0, :, :, 5] == 0).all()


def _galerkin_residual(oracle, P, e1):
    """Assembled b_i^T A (sum_j e_j b_j) minus nothing: the coarse operator
    applied to the element-local coarse vector e1 (8 per element)."""
    nx1, nel, ops = P["nx1"], P["nel"], P["ops"]
    z, _ = oracle.zwgll(nx1)
    lo, hi = 0.5 * (1 - z), 0.5 * (1 + z)
    B = np.empty((8, nx1, nx1, nx1))  # [j, t, s, r]
    for j in range(8):
        br, bs, bt = (hi if j & 1 else lo), (hi if j & 2 else lo), (hi if j & 4 else lo)
        B[j] = bt[:, None, None] * bs[None, :, None] * br[None, None, :]
    B = B.reshape(8, -1)
    u = (e1.reshape(nel, 8) @ B).reshape(-1)
    w = ops.axhelm(u, np.ones(P["n"]), np.zeros(P["n"])).reshape(nel, -1)
    return (w @ B.T).reshape(-1)


@pytest.mark.parametrize("case", ["dirichlet", "null"])
def test_coarse_solve_is_exact(oracle, case):
    """e = A_c^-1 r: the Galerkin operator of e, assembled over the vertices,
    equals the assembled r on every unmasked vertex; with a null space the
    pinned solution has zero mean over the coarse unknowns."""
    if case == "dirichlet":
        P = oracle.box_problem(5, 3, 2, 2, v=rng_unit_vector(91))
    else:
        P = oracle.box_problem(5, 2, 2, 3, dirichlet=(False,) * 6, v=rng_unit_vector(92))
    null = case == "null"
    fbc = oracle.face_types(P["nx1"], P["nel"], P["glo_num"], P["mask"])
    mg = oracle.H1mg(P["ops"], P["x"], P["y"], P["z"], fbc, P["vertex"], null_space=null)
    mask1 = mg.level(0)[0]
    r = np.random.default_rng(93).standard_normal(8 * P["nel"]) * mask1
    vid = np.asarray(P["vertex"]).reshape(-1)
    ids, inv = np.unique(vid, return_inverse=True)
    rg = np.zeros(len(ids))
    np.add.at(rg, inv, r)
    if null:
        rg -= rg.mean()  # a consistent right-hand side
        r = np.zeros_like(r)
        first = np.unique(inv, return_index=True)[1]
        r[first] = rg
    e = mg.coarse(r)
    ag = np.zeros(len(ids))
    np.add.at(ag, inv, _galerkin_residual(oracle, P, e))
    free = np.zeros(len(ids), bool)
    free[inv[mask1 > 0]] = True
    assert np.allclose(ag[free], rg[free], rtol=0, atol=1e-11 * np.abs(rg).max())
    eg = np.zeros(len(ids))
    eg[inv] = e
    assert np.all(e[mask1 == 0] == 0.0)
    if null:
        assert abs(eg.mean()) < 1e-14 * np.abs(eg).max()


@pytest.mark.parametrize("case", ["dirichlet", "periodic", "null"])
def test_preconditioned_krylov(oracle, case):
    """GMRES(30) and flexible CG with h1mg_solve reach the tolerance in a
    small fraction of the Jacobi iterations, on the same solution."""
    if case == "dirichlet":
        P = oracle.box_problem(8, 3, 3, 3, v=rng_unit_vector(71))
        h2v = 0.0
    elif case == "periodic":
        P = oracle.box_problem(6, 3, 4, 3, periodic=(False, True, True), v=rng_unit_vector(72))
        h2v = 10.0
    else:
        P = oracle.box_problem(6, 3, 3, 2, dirichlet=(False,) * 6, v=rng_unit_vector(73))
        h2v = 0.0
    n, ops = P["n"], P["ops"]
    null = case == "null"
    fbc = oracle.face_types(P["nx1"], P["nel"], P["glo_num"], P["mask"])
    mg = oracle.H1mg(ops, P["x"], P["y"], P["z"], fbc, P["vertex"], null_space=null)
    h1, h2 = np.ones(n), np.full(n, h2v)
    f = ops.dssum(P["bm1"] * np.random.default_rng(74).standard_normal(n)) * P["mask"]
    if null:
        f = f - np.sum(f * P["mult"]) / np.sum(P["mult"])
    xj, itj, _, _ = ops.gmres(f, h1, h2, P["mult"], P["mask"], -1e-10, maxit=20000,
                              null_space=null)
    for solver in ("gmres", "flex_cg"):
        x, it, d0, rn = getattr(ops, solver)(f, h1, h2, P["mult"], P["mask"], -1e-10,
                                             maxit=2000, null_space=null, mg=mg)
        r = f - ops.dssum(ops.axhelm(x, h1, h2)) * P["mask"]
        true = np.sqrt(np.sum(r * r * P["mult"]) / np.sum(P["bm1"]))
        assert rn < 1e-10 * d0 and abs(true - rn) <= 1e-3 * rn, solver
        assert it * 5 < itj, (solver, it, itj)
        assert np.linalg.norm(x - xj) <= 1e-8 * np.linalg.norm(xj), solver
        if null:
            assert abs(np.mean(x)) < 1e-13


def test_schwarz_weights_count_overlaps(oracle):
    """Schwarz weights are 1 / (number of extended subdomains covering the
    point): 1 deep inside an element, 1/2 on the first layer off an
    interior face, smaller near edges and corners."""
    P = oracle.box_problem(6, 3, 3, 3, amp=0.0, v=rng_unit_vector(94))
    fbc = oracle.face_types(P["nx1"], P["nel"], P["glo_num"], P["mask"])
    mg = oracle.H1mg(P["ops"], P["x"], P["y"], P["z"], fbc, P["vertex"])
    _, rwt, swt = mg.level(2)
    s = swt.reshape(27, 6, 6, 6)
    c = 13  # the middle element
    assert s[c, 3, 3, 3] == 1.0 and s[c, 2, 2, 2] == 1.0
    assert s[c, 3, 3, 1] == 0.5 and s[c, 3, 1, 3] == 0.5 and s[c, 1, 3, 3] == 0.5
    assert s[c, 3, 1, 1] == pytest.approx(1 / 3) and s[c, 1, 1, 1] == pytest.approx(1 / 4)
    # on the face: 2 elements, and each one's first layer of the other
    assert s[c, 3, 3, 0] == pytest.approx(1 / 2)
    assert np.allclose(rwt, P["mult"])
