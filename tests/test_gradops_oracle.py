"""The oracle's gradient-type operators (oracle/gradops.c) on a deformed
box, through identities a correct restatement must satisfy: linear fields
are exact in the GLL interpolant, so the strong derivative is the constant
gradient, the weak gradient is bm1 times it, the curl of (-y, x, 0) is
(0, 0, 2), and cdtp is the transpose of bm1 * dudxyz."""
import numpy as np

from conftest import rng_unit_vector


def _mesh(oracle):
    P = oracle.box_problem(6, 3, 2, 2, v=rng_unit_vector(141))
    rst, jac = oracle.geom_rst(P["nx1"], P["nel"], P["x"], P["y"], P["z"])
    assert np.allclose(jac, P["jac"], rtol=0, atol=0)
    return P, rst, jac


def test_linear_fields_are_differentiated_exactly(oracle):
    P, rst, jac = _mesh(oracle)
    nx1, nel = P["nx1"], P["nel"]
    a = np.array([0.3, -1.2, 2.5])
    u = a[0] * P["x"] + a[1] * P["y"] + a[2] * P["z"]
    for isd in (1, 2, 3):
        du = oracle.dudxyz(nx1, nel, u, rst, jac, isd)
        assert np.allclose(du, a[isd - 1], rtol=0, atol=1e-11)
    ux, uy, uz = oracle.wgradm1(nx1, nel, u, rst)
    for c, g in enumerate((ux, uy, uz)):
        assert np.allclose(g, a[c] * P["bm1"], rtol=1e-11, atol=1e-14)


def test_curl_of_a_rotation(oracle):
    P, rst, jac = _mesh(oracle)
    ops = P["ops"]
    w1, w2, w3 = oracle.op_curl(ops, -P["y"], P["x"], np.zeros(P["n"]), rst, jac, P["bm1"],
                                P["binv"], ifavg=True)
    assert np.abs(w1).max() < 1e-11 and np.abs(w2).max() < 1e-11
    assert np.allclose(w3, 2.0, rtol=0, atol=1e-11)


def test_cdtp_is_the_transpose_of_the_weighted_derivative(oracle):
    P, rst, jac = _mesh(oracle)
    nx1, nel, n = P["nx1"], P["nel"], P["n"]
    rng = np.random.default_rng(142)
    x, v = rng.standard_normal(n), rng.standard_normal(n)
    for isd in (1, 2, 3):
        lhs = np.dot(v, oracle.cdtp(nx1, nel, x, rst, jac, P["bm1"], isd))
        rhs = np.dot(x, P["bm1"] * oracle.dudxyz(nx1, nel, v, rst, jac, isd))
        assert abs(lhs - rhs) <= 1e-12 * (abs(lhs) + abs(rhs))


def test_splitting_residuals_on_known_fields(oracle):
    """cresvsp with v = 0, qtl = 0: r = bf - bm1 grad(pr), exact for a linear
    pr; crespsp with a rigid rotation (curl curl = 0), bf = 0 and qtl = 0:
    respr = -A(1/vtrans, 0) pr."""
    P, rst, jac = _mesh(oracle)
    n, ops = P["n"], P["ops"]
    z0 = np.zeros(n)
    pr = 0.7 * P["x"] - 0.2 * P["z"]
    bf = [np.full(n, 0.1), np.full(n, -0.3), np.full(n, 0.5)]
    r = oracle.cresvsp(ops, [z0, z0, z0], np.ones(n), z0, np.ones(n), z0, pr, bf, rst)
    for c, g in enumerate((0.7, 0.0, -0.2)):
        assert np.allclose(r[c], bf[c] - g * P["bm1"], rtol=0, atol=1e-11)
    vtrans = np.full(n, 2.0)
    ve = [-P["y"], P["x"], z0]
    respr = oracle.crespsp(ops, ve, pr, z0, np.ones(n), vtrans, [z0, z0, z0], P["bm1"],
                           P["binv"], 1.5, False, rst, jac)
    want = -ops.axhelm(pr, 1.0 / vtrans, z0)
    assert np.allclose(respr, want, rtol=0, atol=1e-10 * np.abs(want).max())


def test_convection_of_a_linear_field(oracle):
    """conv1 of u = a.x in the velocity field v: v.a, exact for linear u;
    advab subtracts bm1 times it from the forcing."""
    P, rst, jac = _mesh(oracle)
    nx1, nel, n = P["nx1"], P["nel"], P["n"]
    rng = np.random.default_rng(143)
    v = [rng.standard_normal(n) for _ in range(3)]
    a = np.array([0.5, -0.25, 1.5])
    u = a[0] * P["x"] + a[1] * P["y"] + a[2] * P["z"]
    c = oracle.conv1(nx1, nel, u, v, rst, jac)
    assert np.allclose(c, a[0] * v[0] + a[1] * v[1] + a[2] * v[2], rtol=0, atol=1e-10)
    bf = [np.ones(n), np.zeros(n), -np.ones(n)]
    out = oracle.advab(nx1, nel, bf, v, P["bm1"], rst, jac)
    for k in range(3):
        ck = oracle.conv1(nx1, nel, v[k], v, rst, jac)
        assert np.array_equal(out[k], bf[k] - P["bm1"] * ck)


def test_time_integration_bookkeeping(oracle):
    """makeabf, makebdf and sumab restated: equal, bit for bit, to the same
    formulas evaluated by numpy in the reference's order."""
    rng = np.random.default_rng(144)
    n = 1000
    r = lambda: rng.standard_normal(n)
    bf, a1, a2, vt, bm1 = r(), r(), r(), 1.0 + np.abs(r()), np.abs(r())
    ab = np.array([1.8, -1.0, 0.2])
    b, n1, n2 = oracle.makeabf(bf, a1, a2, vt, ab)
    ta = ab[1] * a1 + ab[2] * a2
    assert np.array_equal(b, (ab[0] * bf + ta) * vt)
    assert np.array_equal(n1, bf) and np.array_equal(n2, a1)
    v, l1, l2 = r(), r(), r()
    bd = np.array([11 / 6, 3.0, -1.5, 1 / 3])
    got = oracle.makebdf(bf, v, [l1, l2], bm1, vt, bd, 3, 0.01)
    tb = v * bm1 * bd[1]
    tb = tb + l1 * bm1 * bd[2]
    tb = tb + l2 * bm1 * bd[3]
    assert np.array_equal(got, bf + tb * (vt * (1.0 / 0.01)))
    s = oracle.sumab(v, [l1, l2], ab, 3)
    assert np.array_equal(s, (ab[0] * v + ab[1] * l1) + ab[2] * l2)


def test_dealiased_convection(oracle):
    """convop with dealiasing: for a linear u and a constant velocity the
    product is a polynomial the Gauss grid integrates exactly, so it equals
    v . a; for general fields it tends to the undealiased conv1 as the
    fields resolve (here: polynomial velocity of degree 1 and u of degree
    2 on an affine mesh, where both are exact)."""
    P = oracle.box_problem(6, 3, 2, 2, amp=0.0, v=rng_unit_vector(145))
    nx1, nel, n = P["nx1"], P["nel"], P["n"]
    rst, jac = oracle.geom_rst(nx1, nel, P["x"], P["y"], P["z"])
    lxd = (3 * nx1) // 2
    a = np.array([0.5, -0.25, 1.5])
    u = a[0] * P["x"] + a[1] * P["y"] + a[2] * P["z"]
    v = [np.full(n, 0.3), np.full(n, -0.7), np.full(n, 0.2)]
    c = oracle.convect_new(nx1, nel, lxd, u, v, rst, P["bm1"])
    assert np.allclose(c, 0.3 * a[0] - 0.7 * a[1] + 0.2 * a[2], rtol=0, atol=1e-11)
    u2 = P["x"] ** 2 + P["y"] * P["z"]
    v2 = [P["y"], P["z"] - 0.5, P["x"]]
    c2 = oracle.convect_new(nx1, nel, lxd, u2, v2, rst, P["bm1"])
    c1 = oracle.conv1(nx1, nel, u2, v2, rst, jac)
    assert np.allclose(c2, c1, rtol=0, atol=1e-10)


def test_crespsp_face_terms_close_over_the_boundary(oracle):
    """With every boundary face an 'shl' velocity face, a constant velocity
    and nothing else, crespsp is minus the flux c . n dA at the face points,
    which sums to zero over a closed boundary; one face alone gives minus the
    flux through it (here the plane face x = 0 of an undeformed box)."""
    P = oracle.box_problem(5, 3, 2, 2, amp=0.0, v=rng_unit_vector(146))
    nx1, nel, n, ops = P["nx1"], P["nel"], P["n"], P["ops"]
    rst, jac = oracle.geom_rst(nx1, nel, P["x"], P["y"], P["z"])
    fb = oracle.face_types(nx1, nel, P["glo_num"], P["mask"])  # r-, r+, s-, s+, t-, t+
    pre = np.zeros((nel, 6), dtype=np.int32)  # preprocessor order 1..6: s- r+ s+ r- t- t+
    for f_pre, f_fast in ((0, 2), (1, 1), (2, 3), (3, 0), (4, 4), (5, 5)):
        pre[:, f_pre] = np.where(fb[:, f_fast] != 0, 2, 0)
    z0 = np.zeros(n)
    c = np.array([0.3, -1.1, 0.7])
    v = [np.full(n, c[0]), np.full(n, c[1]), np.full(n, c[2])]
    args = (ops, [z0] * 3, z0, z0, np.ones(n), np.ones(n), [z0] * 3, P["bm1"], P["binv"], 1.5,
            False, rst, jac)
    r = oracle.crespsp(*args, v=v, fbc=pre)
    assert abs(r.sum()) < 1e-12 * np.abs(r).sum() and np.abs(r).sum() > 0.1
    one = np.zeros_like(pre)
    one[:, 3] = pre[:, 3]  # the x = 0 faces (r-, preprocessor face 4) only
    r1 = oracle.crespsp(*args, v=v, fbc=one)
    area = (P["y"].max() - P["y"].min()) * (P["z"].max() - P["z"].min())
    assert abs(r1.sum() - c[0] * area) < 1e-12


def test_conservative_convection(oracle):
    """The conservative form div(v u) equals the advective one v . grad u
    for a divergence-free velocity (a rigid rotation) when both are exact
    (u linear, affine mesh)."""
    P = oracle.box_problem(6, 3, 2, 2, amp=0.0, v=rng_unit_vector(147))
    nx1, nel, n = P["nx1"], P["nel"], P["n"]
    rst, jac = oracle.geom_rst(nx1, nel, P["x"], P["y"], P["z"])
    lxd = (3 * nx1) // 2
    u = 0.4 * P["x"] - 0.9 * P["y"] + 0.2 * P["z"]
    v = [-P["y"], P["x"], np.zeros(n)]
    cc = oracle.convect_cons(nx1, nel, lxd, u, v, rst, P["bm1"])
    ca = oracle.convect_new(nx1, nel, lxd, u, v, rst, P["bm1"])
    assert np.allclose(cc, ca, rtol=0, atol=1e-11)
    assert np.allclose(ca, -P["y"] * 0.4 + P["x"] * (-0.9), rtol=0, atol=1e-11)


def test_conv2_is_the_transpose_of_conv1(oracle):
    """sum bm1 psi conv2(phi) = sum bm1 phi conv1(psi) on every element
    (conv2 is the weak transposed form); with no outflow face the
    skew-symmetric form is (conv1 - conv2) / 2 and is skew:
    sum bm1 phi convopo(phi) = 0."""
    P = oracle.box_problem(5, 3, 2, 2, v=rng_unit_vector(148))
    nx1, nel, n = P["nx1"], P["nel"], P["n"]
    rst, jac = oracle.geom_rst(nx1, nel, P["x"], P["y"], P["z"])
    rng = np.random.default_rng(149)
    v = [rng.standard_normal(n) for _ in range(3)]
    phi, psi = rng.standard_normal(n), rng.standard_normal(n)
    lhs = np.sum(P["bm1"] * psi * oracle.conv2(nx1, nel, phi, v, rst, P["bm1"]))
    rhs = np.sum(P["bm1"] * phi * oracle.conv1(nx1, nel, psi, v, rst, jac))
    assert abs(lhs - rhs) <= 1e-11 * (abs(lhs) + abs(rhs))
    none = np.zeros((nel, 6), dtype=np.int32)
    c = oracle.convopo(nx1, nel, phi, v, rst, jac, P["bm1"], none)
    want = 0.5 * oracle.conv1(nx1, nel, phi, v, rst, jac) - 0.5 * oracle.conv2(nx1, nel, phi, v, rst, P["bm1"])
    assert np.allclose(c, want, rtol=0, atol=1e-12 * np.abs(want).max())
    skew = np.sum(P["bm1"] * phi * c)
    assert abs(skew) <= 1e-11 * np.sum(np.abs(P["bm1"] * phi * c))
