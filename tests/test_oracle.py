"""CPU oracle: known-answer tests that pin the restatement of the reference.

The reference ships no function-level golden vectors for this path, so the
oracle is pinned by mathematics (GLL quadrature and differentiation
exactness, operator symmetry and null space, spectral convergence to a
manufactured solution), by internal consistency with the reference's own
alternative forms (local_grad3 / local_grad3_t vs axhelm's inline mxm
contractions), and by the committed fixtures in tests/golden/.
"""
import numpy as np
import pytest

from conftest import rng_unit_vector


@pytest.mark.parametrize("np_", [2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12])
def test_gll_quadrature_exactness(oracle, np_):
    z, w = oracle.zwgll(np_)
    N = np_ - 1
    assert z[0] == -1.0 and z[-1] == 1.0
    assert np.all(np.diff(z) > 0)
    # GLL integrates polynomials up to degree 2N-1 exactly
    for k in range(0, 2 * N):
        exact = 0.0 if k % 2 else 2.0 / (k + 1)
        assert abs(np.dot(w, z ** k) - exact) < 5e-15 * max(1, np_)


@pytest.mark.parametrize("np_", [3, 5, 8, 10, 12])
def test_gll_nodes_against_sympy(oracle, np_):
    sympy = pytest.importorskip("sympy")
    x = sympy.symbols("x")
    N = np_ - 1
    dP = sympy.diff(sympy.legendre(N, x), x)
    roots = sorted(float(r) for r in sympy.Poly(dP, x).nroots(n=30))
    z, _ = oracle.zwgll(np_)
    assert np.max(np.abs(z[1:-1] - np.array(roots))) < 4e-16


@pytest.mark.parametrize("np_", [2, 4, 6, 8, 10, 12])
def test_dgll_differentiates_polynomials(oracle, np_):
    z, _ = oracle.zwgll(np_)
    D, DT = oracle.dgll(z)
    assert np.array_equal(D.T, DT)
    N = np_ - 1
    for k in range(0, N + 1):
        d = D @ z ** k
        ex = k * z ** (k - 1) if k else np.zeros_like(z)
        assert np.max(np.abs(d - ex)) < 2e-13 * N ** 2


def test_mxm_order_is_left_to_right(oracle):
    a = np.array([[1e16, 1.0, -1e16]])
    b = np.array([[1.0], [1.0], [1.0]])
    # ((1e16 + 1) - 1e16) = 0 in left-to-right FP64, not 1
    assert oracle.mxm(a, b)[0, 0] == 0.0


def test_local_grad3_matches_axhelm_contractions(oracle):
    """axhelm's inline mxm forms (hmholtz.f:191-217) equal local_grad3/_t."""
    N = 6
    z, w = oracle.zwgll(N + 1)
    D, _ = oracle.dgll(z)
    rng = np.random.default_rng(3)
    u = rng.standard_normal((N + 1) ** 3)
    ur, us, ut = oracle.local_grad3(u, D)
    U = u.reshape(N + 1, N + 1, N + 1)  # [k, j, i]
    assert np.allclose(ur.reshape(U.shape), np.einsum("il,kjl->kji", D, U), rtol=0, atol=1e-12)
    assert np.allclose(us.reshape(U.shape), np.einsum("jl,kli->kji", D, U), rtol=0, atol=1e-12)
    assert np.allclose(ut.reshape(U.shape), np.einsum("kl,lji->kji", D, U), rtol=0, atol=1e-12)
    v = oracle.local_grad3_t(ur, us, ut, D)
    V = (np.einsum("li,kjl->kji", D, ur.reshape(U.shape)) + np.einsum("lj,kli->kji", D, us.reshape(U.shape))
         + np.einsum("lk,lji->kji", D, ut.reshape(U.shape)))
    assert np.allclose(v.reshape(U.shape), V, rtol=0, atol=1e-11)


@pytest.fixture(scope="module")
def small(oracle):
    return oracle.box_problem(6, 3, 3, 3, v=rng_unit_vector(0))


def test_setvert3d_groups_equal_geometric_coincidence(oracle, small):
    P = small
    glo = P["glo_num"]
    nx = P["nx1"]
    # interior ids are 0, boundary ids non-zero
    gl = glo.reshape(P["nel"], nx, nx, nx)
    assert np.all(gl[:, 1:-1, 1:-1, 1:-1] == 0)
    bnd = np.ones((nx, nx, nx), bool)
    bnd[1:-1, 1:-1, 1:-1] = False
    assert np.all(gl[:, bnd] > 0)
    # equal ids <=> equal undeformed lattice coordinates
    x, y, zc = P["x"], P["y"], P["z"]
    key = np.round(np.stack([x, y, zc], 1) * 1e9).astype(np.int64)
    nz = glo > 0
    ids = {}
    for g, k in zip(glo[nz], map(tuple, key[nz])):
        ids.setdefault(g, set()).add(k)
    assert all(len(s) == 1 for s in ids.values())
    keys = {}
    for g, k in zip(glo[nz], map(tuple, key[nz])):
        keys.setdefault(k, set()).add(g)
    assert all(len(s) == 1 for s in keys.values())
    # the id count equals unique nodes minus element interiors
    nn = (3 * 5 + 1) ** 3 - P["nel"] * 4 ** 3
    assert len(ids) == nn == P["ngv"]


def test_gs_semantics(oracle, small):
    P = small
    gs = oracle.GS(P["glo_num"])
    u = np.random.default_rng(1).standard_normal(P["n"])
    v = u.copy()
    gs.op(v, "+")
    start, idx, _ = gs.maps()
    for s in range(len(start) - 1):
        members = idx[start[s]:start[s + 1]]
        assert np.all(np.diff(members) > 0)
        tot = u[members[0]]
        for m in members[1:]:
            tot = tot + u[m]
        assert np.all(v[members] == tot)
    untouched = np.ones(P["n"], bool)
    untouched[idx] = False
    assert np.array_equal(v[untouched], u[untouched])


def test_axhelm_symmetric_and_null_space(oracle, small):
    P = small
    ops = P["ops"]
    n = P["n"]
    rng = np.random.default_rng(2)
    h1 = np.ones(n)
    h2 = np.zeros(n)
    uc = ops.dssum(rng.standard_normal(n)) * P["mult"]
    vc = ops.dssum(rng.standard_normal(n)) * P["mult"]
    a = ops.axhelm(uc, h1, h2)
    b = ops.axhelm(vc, h1, h2)
    assert abs(np.dot(vc, a) - np.dot(uc, b)) < 1e-12 * abs(np.dot(vc, a))
    assert np.max(np.abs(ops.axhelm(np.ones(n), h1, h2))) < 1e-13
    # h2 term adds exactly h2 * bm1 * u
    h2c = np.full(n, 10.0)
    d = ops.axhelm(uc, h1, h2c) - a
    assert np.allclose(d, 10.0 * P["bm1"] * uc, rtol=1e-12, atol=1e-14)


def test_poisson_spectral_convergence(oracle):
    """-lap u = 3 pi^2 u for u = sin(pi x) sin(pi y) sin(pi z) on the undeformed cube."""
    errs = []
    for N in (3, 5, 7):
        P = oracle.box_problem(N + 1, 2, 2, 2, amp=0.0)
        ops, n = P["ops"], P["n"]
        x, y, z = P["x"], P["y"], P["z"]
        ue = np.sin(np.pi * x) * np.sin(np.pi * y) * np.sin(np.pi * z)
        f = 3 * np.pi ** 2 * ue
        rhs = P["bm1"] * f
        u, _, it, r0, r2 = ops.hmholtz(rhs, np.ones(n), np.zeros(n), P["mask"], P["mult"],
                                       P["binv"], -1e-12, maxcg=10 ** 6)
        errs.append(np.max(np.abs(u - ue)))
    assert errs[0] > errs[1] > errs[2]
    assert errs[2] < 1e-5


def test_cggo_converges_and_counts(oracle, small):
    P = small
    ops, n = P["ops"], P["n"]
    rng = np.random.default_rng(0)
    f = ops.dssum(rng.uniform(-1, 1, n)) * P["mult"]
    rhs = P["bm1"] * f
    u, rhs2, it, r0, r2 = ops.hmholtz(rhs, np.ones(n), np.zeros(n), P["mask"], P["mult"], P["binv"],
                                       -1e-10, maxcg=10 ** 6)
    assert r2 <= 1e-10 * r0
    assert 10 < it < 500
    # the residual of the returned solution is small in the reference norm
    w = ops.axhelm(u, np.ones(n), np.zeros(n))
    w = ops.dssum(w) * P["mask"]
    res = rhs2 - w
    rn = np.sqrt(np.sum(res * res * P["mult"] * P["binv"]) / P["bm1"].sum())
    assert rn < 2e-10 * r0
    # the reference's 900-iteration cap (maxcg)
    _, _, it2, _, r22 = ops.hmholtz(rhs, np.ones(n), np.zeros(n), P["mask"], P["mult"], P["binv"],
                                    -1e-10, maxcg=5)
    assert it2 == 5 and r22 > 1e-10 * r0


def test_threaded_oracle_matches_serial(oracle):
    if oracle.max_threads() < 2:
        pytest.skip("oracle built without OpenMP threads")
    P1 = oracle.box_problem(5, 3, 3, 2, v=rng_unit_vector(4), nthreads=1)
    P4 = oracle.box_problem(5, 3, 3, 2, v=rng_unit_vector(4), nthreads=4)
    n = P1["n"]
    u = np.random.default_rng(5).standard_normal(n)
    a1 = P1["ops"].axhelm(u, np.ones(n), np.zeros(n))
    a4 = P4["ops"].axhelm(u, np.ones(n), np.zeros(n))
    assert np.array_equal(a1, a4)  # per-element work is order-independent


def test_projection_restatement_properties(oracle):
    """project1/project2 (navier4.f:636-1187): after a sequence of hsolve calls
    the space is B-orthonormal in (x, y)_mult, the projected right-hand side
    is orthogonal to it, and every returned u solves the masked system."""
    from conftest import rng_unit_vector
    P = oracle.box_problem(5, 2, 2, 3, v=rng_unit_vector(13))
    ops, n = P["ops"], P["n"]
    proj = oracle.Projection(ops, 4)
    rng = np.random.default_rng(13)
    f0, f1 = rng.standard_normal(n), rng.standard_normal(n)
    h1, h2 = np.ones(n), np.full(n, 50.0)
    its = []
    for t in range(7):
        f = f0 + np.cos(0.5 * t) * f1 + 1e-2 * np.random.default_rng(t).standard_normal(n)
        rhs = P["bm1"] * ops.dssum(f * P["mult"])
        u, r, it, r0, r2 = proj.hsolve(rhs, h1, h2, P["mask"], P["mult"], P["binv"], 1e-11)
        its.append(it)
        w = P["mult"]
        if proj.m > 1 and t < 6:
            X, B = proj.basis()
            G = (X * w) @ B.T
            assert np.abs(G - np.eye(len(G))).max() < 1e-12
        # u solves mask * dssum(A u) = mask * dssum(rhs*mask) (hsolve's rhs)
        b = ops.dssum(rhs * P["mask"])
        res = ops.dssum(ops.axhelm(u, h1, h2)) * P["mask"] - b
        assert np.sqrt(np.sum(P["mult"] * P["binv"] * res ** 2) / P["bm1"].sum()) < 1e-9
    assert proj.m == 4 and its[-1] < its[0]


def test_oracle_matches_committed_golden_fixtures(oracle):
    """tests/golden/oracle_golden.npz (made by tests/golden/make_golden.py)
    pins the restatement against itself: integer outputs and iteration counts
    exactly, floating-point outputs to 1e-12 relative (exact on the machine
    that made them; libm and numpy's vector math may round differently on
    another architecture)."""
    import importlib.util
    import os
    here = os.path.dirname(os.path.abspath(__file__))
    spec = importlib.util.spec_from_file_location("make_golden",
                                                  os.path.join(here, "golden", "make_golden.py"))
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    ref = np.load(os.path.join(here, "golden", "oracle_golden.npz"))
    got = mg.compute()
    assert set(ref.files) == set(got)
    for k in ref.files:
        a, b = ref[k], np.asarray(got[k])
        assert a.shape == b.shape, k
        if a.dtype.kind in "iu":
            assert np.array_equal(a, b), k
        elif k.endswith("_stats"):
            cnt = a[..., 0] if k != "proj_stats" else a[:, :2]
            cnt_b = b[..., 0] if k != "proj_stats" else b[:, :2]
            assert np.array_equal(cnt, cnt_b), k  # iteration counts (and space sizes)
            assert np.allclose(a, b, rtol=1e-10, atol=0), k
        else:
            scale = np.max(np.abs(a)) if a.size else 1.0
            assert np.max(np.abs(a - b)) <= 1e-12 * max(scale, 1e-300), k


def test_gmres_restatement_solves_the_system(oracle):
    """hmh_gmres restated (Jacobi stand-in preconditioner): its residual
    estimate equals the true weighted residual, restarts do not change the
    solution beyond the tolerance, and the null-space case returns a
    zero-mean solution of a consistent system."""
    from conftest import rng_unit_vector
    P = oracle.box_problem(5, 3, 2, 2, v=rng_unit_vector(61))
    n, ops = P["n"], P["ops"]
    h1, h2 = np.ones(n), np.zeros(n)
    f = ops.dssum(P["bm1"] * np.random.default_rng(61).standard_normal(n)) * P["mask"]
    x, it, d0, rn = ops.gmres(f, h1, h2, P["mult"], P["mask"], -1e-10, m=30)
    r = f - ops.dssum(ops.axhelm(x, h1, h2)) * P["mask"]
    true = np.sqrt(np.sum(r * r * P["mult"]) / np.sum(P["bm1"]))
    assert rn < 1e-10 * d0 and abs(true - rn) <= 1e-3 * rn
    x5, it5, _, _ = ops.gmres(f, h1, h2, P["mult"], P["mask"], -1e-10, m=5)
    assert it5 > it and np.linalg.norm(x5 - x) <= 1e-8 * np.linalg.norm(x)
    Q = oracle.box_problem(5, 2, 2, 2, dirichlet=(False,) * 6, v=rng_unit_vector(62))
    nq, oq = Q["n"], Q["ops"]
    g = oq.dssum(Q["bm1"] * np.random.default_rng(62).standard_normal(nq))
    g = g - np.sum(g * Q["mult"]) / np.sum(Q["mult"])
    xq, itq, d0q, rnq = oq.gmres(g, np.ones(nq), np.zeros(nq), Q["mult"], Q["mask"], -1e-10,
                                 maxit=4000, null_space=True)
    assert rnq < 1e-10 * d0q and abs(np.mean(xq)) < 1e-14


def test_flex_cg_restatement_solves_the_system(oracle):
    """hmh_flex_cg restated (Jacobi stand-in preconditioner): its residual
    norm is the true weighted residual, it agrees with GMRES on the same
    system, the null-space case returns a zero-mean solution and a zero
    right-hand side gives x = 0 after no iteration."""
    from conftest import rng_unit_vector
    P = oracle.box_problem(5, 3, 2, 2, v=rng_unit_vector(63))
    n, ops = P["n"], P["ops"]
    h1, h2 = np.ones(n), np.full(n, 2.0)
    f = ops.dssum(P["bm1"] * np.random.default_rng(63).standard_normal(n)) * P["mask"]
    x, it, d0, rn = ops.flex_cg(f, h1, h2, P["mult"], P["mask"], -1e-10)
    r = f - ops.dssum(ops.axhelm(x, h1, h2)) * P["mask"]
    true = np.sqrt(np.sum(r * r * P["mult"]) / np.sum(P["bm1"]))
    assert rn < 1e-10 * d0 and abs(true - rn) <= 1e-3 * rn
    xg, _, _, _ = ops.gmres(f, h1, h2, P["mult"], P["mask"], -1e-10, m=30)
    assert np.linalg.norm(xg - x) <= 1e-8 * np.linalg.norm(x)
    Q = oracle.box_problem(5, 2, 2, 2, dirichlet=(False,) * 6, v=rng_unit_vector(64))
    nq, oq = Q["n"], Q["ops"]
    g = oq.dssum(Q["bm1"] * np.random.default_rng(64).standard_normal(nq))
    g = g - np.sum(g * Q["mult"]) / np.sum(Q["mult"])
    xq, itq, d0q, rnq = oq.flex_cg(g, np.ones(nq), np.zeros(nq), Q["mult"], Q["mask"], -1e-10,
                                   maxit=4000, null_space=True)
    assert rnq < 1e-10 * d0q and abs(np.mean(xq)) < 1e-14
    x0, it0, d00, _ = ops.flex_cg(np.zeros(n), h1, h2, P["mult"], P["mask"], -1e-10)
    assert it0 == 0 and d00 == 0.0 and not np.any(x0)
