"""Mesh ingestion (include/nekmesh.h): .re2 / .co2 readers, connectivity from
element corners, set_vert numbering and the trilinear GLL coordinates, on
the host (no GPU).

The .re2 layout is pinned on the reference's own genbox output
(short_tests/lpm_one/uniform.re2, written from uniform.box: a 5x5x5 box on
the unit cube with walls on every side) when the reference tree is present;
tests/golden/re2_reference.json holds what was read from it.  set_vert is
compared with the oracle's restatement bit for bit."""
import json
import os

import numpy as np
import pytest

from re2_util import box_elements, rotate_elements, same_partition, write_re2

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden", "re2_reference.json")
# the reference's Nek5000 source tree, when the environment names it
_REF_ROOT = os.environ.get("NEK5000_REFERENCE", "")
REF_RE2 = (os.path.join(_REF_ROOT, "short_tests", "lpm_one", "uniform.re2") if _REF_ROOT
           else "")


@pytest.fixture(scope="module")
def mio():
    from nek5000_gb300 import build
    build.build()
    from nek5000_gb300 import meshio
    return meshio


@pytest.mark.parametrize("version,big", [("#v002", False), ("#v002", True), ("#v001", False)])
def test_re2_round_trip(mio, tmp_path, version, big):
    xc, yc, zc, _, bcs = box_elements(3, 2, 2, jitter=0.2, seed=3)
    curves = [(2, 5, (0.1, 0.2, 0.3, 0.4, 0.5), "m"), (7, 11, (1.0, 0, 0, 0, 0), "C")]
    thermal = [(1, 4, (3.5, 0, 0, 0, 0), "t  ")]
    p = tmp_path / "box.re2"
    write_re2(p, xc, yc, zc, bcs, version=version, big_endian=big, curves=curves,
              groups=np.arange(12) % 3, extra_bc_sections=(thermal,))
    R = mio.read_re2(p)
    assert (R["nelgt"], R["ndim"], R["nelgv"]) == (12, 3, 12)
    assert R["wdsize"] == (4 if version == "#v001" else 8)
    rtol = 1e-7 if version == "#v001" else 0.0
    for a, b in ((R["xc"], xc), (R["yc"], yc), (R["zc"], zc)):
        np.testing.assert_allclose(a, b, rtol=rtol, atol=rtol)
    assert list(R["group"]) == list(np.arange(12) % 3)
    assert list(R["curves"]["elem"]) == [2, 7] and list(R["curves"]["side"]) == [5, 11]
    assert R["curves"]["ccurve"] == "mC"
    np.testing.assert_allclose(R["curves"]["curve"][0], [0.1, 0.2, 0.3, 0.4, 0.5], rtol=rtol)
    assert len(R["bcs"]) == 2
    cbc, bc = R["bcs"][0]
    for (el, f, vals, t) in bcs:
        assert cbc[el - 1, f - 1] == t
    assert (cbc == "W  ").sum() == len(bcs) and (cbc == "E  ").sum() == 12 * 6 - len(bcs)
    cbc2, bc2 = R["bcs"][1]
    assert cbc2[0, 3] == "t  " and bc2[0, 3, 0] == pytest.approx(3.5)


def test_re2_errors(mio, tmp_path):
    from nek5000_gb300 import _capi
    with pytest.raises(_capi.NekGpuError) as ei:
        mio.read_re2(tmp_path / "missing.re2")
    assert ei.value.code == _capi.EIO
    xc, yc, zc, _, bcs = box_elements(2, 2, 2)
    p = tmp_path / "t.re2"
    write_re2(p, xc, yc, zc, bcs)
    data = open(p, "rb").read()
    for bad in (data[:500], b"#x002" + data[5:], data[:80] + b"\0\0\0\0" + data[84:]):
        open(p, "wb").write(bad)
        with pytest.raises(_capi.NekGpuError) as ei:
            mio.read_re2(p)
        assert ei.value.code == _capi.EIO


def test_reference_genbox_file(mio):
    """The reference's uniform.re2 holds the box uniform.box describes: 5^3
    elements of 0.2, x fastest, corners in preprocessor order, W on every
    outside face (150 records) and E inside."""
    ref = json.load(open(GOLDEN))["uniform.re2"]
    if not REF_RE2 or not os.path.exists(REF_RE2):
        pytest.skip("NEK5000_REFERENCE does not name a Nek5000 tree (the golden digest was "
                    "checked by its generator)")
    R = mio.read_re2(REF_RE2)
    assert (R["nelgt"], R["ndim"], R["nelgv"], R["wdsize"]) == tuple(ref["header"])
    xc, yc, zc, _, bcs = box_elements(5, 5, 5)
    np.testing.assert_allclose(R["xc"], xc, atol=1e-15)
    np.testing.assert_allclose(R["yc"], yc, atol=1e-15)
    np.testing.assert_allclose(R["zc"], zc, atol=1e-15)
    cbc, bc = R["bcs"][0]
    assert (cbc == "W  ").sum() == ref["n_wall_faces"] == len(bcs)
    for (el, f, vals, t) in bcs:
        assert cbc[el - 1, f - 1] == "W  "
    assert float(np.sum(R["xc"] + 2 * R["yc"] + 3 * R["zc"])) == pytest.approx(ref["corner_sum"])


@pytest.mark.parametrize("periodic_y", [False, True])
def test_connectivity_matches_the_lattice(mio, periodic_y):
    perm = np.random.default_rng(5).permutation(4 * 3 * 3)
    xc, yc, zc, lattice, bcs = box_elements(4, 3, 3, periodic_y=periodic_y, jitter=0.25, seed=5,
                                            perm=perm)
    nel = xc.shape[0]
    cbc = np.full((nel, 6), "E  ")
    bc = np.zeros((nel, 6, 5))
    for (el, f, vals, t) in bcs:
        cbc[el - 1, f - 1] = t
        bc[el - 1, f - 1] = vals
    vertex, nv = mio.connect(xc, yc, zc, cbc, bc)
    assert same_partition(vertex, lattice)
    assert nv == len(np.unique(lattice))
    assert vertex.min() == 1 and vertex.max() == nv


def test_connectivity_errors(mio):
    from nek5000_gb300 import _capi
    xc, yc, zc, _, bcs = box_elements(2, 2, 2, periodic_y=True)
    nel = 8
    cbc = np.full((nel, 6), "E  ")
    bc = np.zeros((nel, 6, 5))
    for (el, f, vals, t) in bcs:
        cbc[el - 1, f - 1] = t
        bc[el - 1, f - 1] = vals
    with pytest.raises(_capi.NekGpuError):  # a tolerance that merges whole elements
        mio.connect(xc, yc, zc, cbc, bc, tol=3.0)
    bad = bc.copy()
    q = np.argwhere(cbc == "P  ")[0]
    bad[q[0], q[1], 0] = (q[0] + 1) % nel + 1  # partner that does not point back
    with pytest.raises(_capi.NekGpuError):
        mio.connect(xc, yc, zc, cbc, bad)


@pytest.mark.parametrize("nx", [2, 3, 5, 8])
def test_setvert3d_matches_the_oracle(mio, oracle, nx):
    xc, yc, zc, lattice, _ = box_elements(3, 2, 2, periodic_y=True, seed=1,
                                          perm=np.random.default_rng(1).permutation(12))
    # relabel the vertices at random: the numbering must follow them
    relabel = np.random.default_rng(2).permutation(lattice.max()) + 1
    vertex = relabel[lattice - 1]
    glo, ngv = mio.setvert3d(nx, vertex)
    glo_ref, ngv_ref = oracle.setvert3d(nx, 12, vertex.reshape(-1))
    assert ngv == ngv_ref
    assert np.array_equal(glo, glo_ref)


def test_xyzlin_is_the_trilinear_map(mio):
    from nek5000_gb300.mesh import gll
    xc, yc, zc, _, _ = box_elements(2, 2, 1, jitter=0.3, seed=4)
    nx = 6
    zg, _ = gll(nx)
    x, y, z = mio.xyzlin(nx, zg, xc, yc, zc)
    h = np.stack([(1 - zg) / 2, (1 + zg) / 2])  # (2, nx)
    pre = [0, 1, 3, 2, 4, 5, 7, 6]  # tensor corner -> preprocessor corner
    for arr, c in ((x, xc), (y, yc), (z, zc)):
        u = c[:, pre].reshape(-1, 2, 2, 2)  # (e, k, j, i)
        want = np.einsum("ekji,kz,jy,ix->ezyx", u, h, h, h).reshape(-1)
        np.testing.assert_allclose(arr, want, rtol=0, atol=1e-15)


def test_co2_round_trip_and_load_mesh(mio, tmp_path):
    from nek5000_gb300 import mesh
    xc, yc, zc, lattice, bcs = box_elements(3, 3, 2)
    p = tmp_path / "box.re2"
    write_re2(p, xc, yc, zc, bcs)
    M = mio.load_mesh(p, N=5)
    c2 = tmp_path / "box.co2"
    mio.write_co2(c2, M["vertex"])
    C2 = mio.read_co2(c2)
    assert np.array_equal(C2["vertex"], M["vertex"]) and C2["nv"] == 8
    M2 = mio.load_mesh(p, N=5, co2=c2)
    assert np.array_equal(M2["glo_num"], M["glo_num"])
    # the same box from the box mesher (undeformed, walls everywhere)
    B = mesh.box_mesh(5, 3, 3, 2, amp=0.0)
    np.testing.assert_allclose(M["g"], B["g"], rtol=1e-12, atol=1e-13)
    np.testing.assert_allclose(M["bm1"], B["bm1"], rtol=1e-13)
    assert same_partition(M["glo_num"] + (M["glo_num"] == 0) * (10 ** 9 + np.arange(M["n"])),
                          B["glo_num"] + (B["glo_num"] == 0) * (10 ** 9 + np.arange(B["n"])))
    np.testing.assert_array_equal(M["mask"], B["mask"])
    np.testing.assert_allclose(M["mult"], B["mult"], rtol=1e-15)
    np.testing.assert_allclose(M["binv"], B["binv"], rtol=1e-13)


def test_rotated_elements_give_a_continuous_numbering(mio, tmp_path):
    """Elements whose corner lists start at different corners (mixed local
    frames): the numbering must still join exactly the coincident points, so
    the average over copies of a smooth field is the field itself and every
    point's copy count is its geometric multiplicity."""
    xc, yc, zc, _, _ = box_elements(3, 3, 3, jitter=0.2, seed=9,
                                    perm=np.random.default_rng(9).permutation(27))
    xc, yc, zc = rotate_elements(xc, yc, zc, seed=9)
    p = tmp_path / "rot.re2"
    write_re2(p, xc, yc, zc, [])
    M = mio.load_mesh(p, N=4)
    assert np.all(M["jac"] > 0)
    f = np.sin(2 * M["x"]) * np.cos(3 * M["y"]) + M["z"] ** 2
    avg = mio._dsop(M["glo_num"], f, "+") * M["mult"]
    np.testing.assert_allclose(avg, f, rtol=0, atol=1e-13)
    # copy counts: 8 at interior lattice vertices, 4 on interior edges, 2 on faces
    cnt = np.rint(1 / M["mult"]).astype(int)
    key = np.round(np.stack([M["x"], M["y"], M["z"]], 1), 9)
    _, inv, counts = np.unique(key, axis=0, return_inverse=True, return_counts=True)
    assert np.array_equal(cnt, counts[inv.reshape(-1)])


def test_face_repair_joins_a_displaced_corner(mio):
    """One element's copy of an interior vertex moved by 0.3 h (beyond the
    0.2 tolerance): its faces share three of four corners with their
    neighbours, and the repair step (gencon face_chk) joins the fourth."""
    xc, yc, zc, lattice, _ = box_elements(3, 3, 3)
    e = 0  # element (0,0,0): its preprocessor corner 7 (index 6) is lattice vertex (1,1,1)
    xc[e, 6] += 0.3 / 3
    vertex, nv = mio.connect(xc, yc, zc)
    assert same_partition(vertex, lattice) and nv == lattice.max()


# edges of an element (preprocessor numbering 1..12) as pairs of preprocessor corners
PRE_EDGES = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 4), (1, 5),
             (2, 6), (3, 7)]


def _quad_map(p):
    """A map whose every component is linear plus univariate quadratics:
    reproduced exactly by vertex + edge Gordon-Hall blending."""
    x, y, z = p[..., 0], p[..., 1], p[..., 2]
    return np.stack([x + 0.3 * y * y, y + 0.2 * z * z - 0.1 * x * x, z + 0.25 * x * x], -1)


def _midside_mesh(kx, ky, kz, mapf, straight=False):
    xc, yc, zc, lattice, bcs = box_elements(kx, ky, kz)
    P = np.stack([xc, yc, zc], -1)  # (nel, 8, 3) box corners
    curves = []
    for e in range(P.shape[0]):
        for k, (a, b) in enumerate(PRE_EDGES):
            m = 0.5 * (P[e, a] + P[e, b])
            node = m if straight else mapf(m)
            curves.append((e + 1, k + 1, (node[0], node[1], node[2], 0.0, 0.0), "m"))
    Q = P if straight else mapf(P)
    return Q[..., 0], Q[..., 1], Q[..., 2], curves, bcs


def _curves_dict(curves):
    return dict(elem=np.array([c[0] for c in curves]), side=np.array([c[1] for c in curves]),
                curve=np.array([c[2] for c in curves]), ccurve="".join(c[3] for c in curves))


def test_midside_nodes_reproduce_quadratic_maps(mio):
    """xyzquad + Gordon-Hall: on an element whose map is the composition of a
    map with univariate-quadratic components with the trilinear box map, the
    GLL points are that map's values; with midpoints of straight edges the
    result is the trilinear map."""
    from nek5000_gb300.mesh import gll
    nx = 7
    zg, _ = gll(nx)
    xc, yc, zc, curves, _ = _midside_mesh(2, 2, 1, _quad_map)
    x, y, z = mio.genxyz(nx, zg, xc, yc, zc, _curves_dict(curves))
    # the box points at the GLL nodes (trilinear map of the box corners), mapped
    bx, by, bz, _, _ = box_elements(2, 2, 1)
    px, py, pz = mio.xyzlin(nx, zg, bx, by, bz)
    want = _quad_map(np.stack([px, py, pz], -1))
    got = np.stack([x, y, z], -1)
    np.testing.assert_allclose(got, want, rtol=0, atol=4e-15)
    # straight midpoints: the trilinear map
    xc, yc, zc, curves, _ = _midside_mesh(2, 2, 1, None, straight=True)
    got = np.stack(mio.genxyz(nx, zg, xc, yc, zc, _curves_dict(curves)), -1)
    np.testing.assert_allclose(got, np.stack([px, py, pz], -1), rtol=0, atol=4e-16)


def test_midside_mesh_loads_continuous(mio, tmp_path):
    """A .re2 mesh with 'm' records on every edge: load_mesh gives positive
    Jacobians and a numbering under which a smooth field is continuous."""
    xc, yc, zc, curves, bcs = _midside_mesh(3, 2, 2, _quad_map)
    p = tmp_path / "quad.re2"
    write_re2(p, xc, yc, zc, bcs, curves=curves)
    M = mio.load_mesh(p, N=6)
    assert np.all(M["jac"] > 0)
    f = np.cos(M["x"]) * np.sin(2 * M["y"]) + M["z"]
    avg = mio._dsop(M["glo_num"], f, "+") * M["mult"]
    np.testing.assert_allclose(avg, f, rtol=0, atol=1e-13)
    # other curve types are refused
    write_re2(p, xc, yc, zc, bcs, curves=[(1, 1, (0.5, 0, 0, 0, 0), "s")])
    from nek5000_gb300 import _capi
    with pytest.raises(_capi.NekGpuError) as ei:
        mio.load_mesh(p, N=6)
    assert ei.value.code == _capi.EINVAL


def _annulus(nt=8, nr=2, nz=1, ri=0.5, ro=1.0, h=0.5, arcs=True):
    """Elements of an annular ring (nt around, nr across, nz high): corners in
    file order (bottom counter-clockwise seen from +z, then top), the
    circular-arc records of their inner and outer edges (positive radius where
    the centre is on the element's side), walls on every outside face."""
    xc, yc, zc, curves, bcs = [], [], [], [], []
    e = 0
    for kz in range(nz):
        for jt in range(nt):
            t0, t1 = 2 * np.pi * jt / nt, 2 * np.pi * (jt + 1) / nt
            for ir in range(nr):
                r0, r1 = ri + (ro - ri) * ir / nr, ri + (ro - ri) * (ir + 1) / nr
                quad = [(r0, t0), (r1, t0), (r1, t1), (r0, t1)]
                xs = [r * np.cos(t) for r, t in quad]
                ys = [r * np.sin(t) for r, t in quad]
                xc.append(xs + xs)
                yc.append(ys + ys)
                zc.append([h * kz / nz] * 4 + [h * (kz + 1) / nz] * 4)
                e += 1
                if arcs:
                    for edge, rad in ((2, r1), (4, -r0), (6, r1), (8, -r0)):
                        curves.append((e, edge, (rad, 0.0, 0.0, 0.0, 0.0), "C"))
                if ir == 0:
                    bcs.append((e, 4, (0.0,) * 5, "W  "))
                if ir == nr - 1:
                    bcs.append((e, 2, (0.0,) * 5, "W  "))
                if kz == 0:
                    bcs.append((e, 5, (0.0,) * 5, "W  "))
                if kz == nz - 1:
                    bcs.append((e, 6, (0.0,) * 5, "W  "))
    return np.array(xc), np.array(yc), np.array(zc), curves, bcs


def test_arc_edges_make_an_exact_annulus(mio, tmp_path):
    """Circular-arc edges (arcsrf): the GLL points of the bent edges lie on
    their circles, the numbering is continuous around the ring, and the mesh
    volume converges to the annulus' (a polygonal ring misses it by 2.6%)."""
    ri, ro, h = 0.5, 1.0, 0.5
    exact = np.pi * (ro * ro - ri * ri) * h
    vols = {}
    for arcs in (True, False):
        xc, yc, zc, curves, bcs = _annulus(ri=ri, ro=ro, h=h, arcs=arcs)
        p = tmp_path / f"ring{arcs}.re2"
        write_re2(p, xc, yc, zc, bcs, curves=curves)
        M = mio.load_mesh(p, N=7)
        assert np.all(M["jac"] > 0)
        vols[arcs] = M["vol"]
        f = M["x"] * M["y"] + np.cos(M["z"])
        avg = mio._dsop(M["glo_num"], f, "+") * M["mult"]
        np.testing.assert_allclose(avg, f, rtol=0, atol=1e-13)
        if arcs:
            rad = np.hypot(M["x"], M["y"]).reshape(M["nel"], 8, 8, 8)
            np.testing.assert_allclose(rad[1::2, :, :, -1], ro, rtol=0, atol=1e-14)  # outer edges
            np.testing.assert_allclose(rad[0::2, :, :, 0], ri, rtol=0, atol=1e-14)   # inner edges
    assert abs(vols[True] - exact) <= 1e-8 * exact, (vols[True], exact)
    assert abs(vols[False] - exact) > 1e-2 * exact


def test_single_element_periodicity(mio, tmp_path):
    """'p  ' on both z faces of a one-element-high box (check_p_bc): the
    points of each element's z faces share ids, so a z-periodic field stays
    continuous and those points count twice as often."""
    xc, yc, zc, lattice, bcs = box_elements(3, 2, 1, jitter=0.0)
    bcs = [b for b in bcs if b[1] not in (5, 6)]
    for e in range(6):
        bcs += [(e + 1, 5, (0.0,) * 5, "p  "), (e + 1, 6, (0.0,) * 5, "p  ")]
    p = tmp_path / "p.re2"
    write_re2(p, xc, yc, zc, bcs)
    M = mio.load_mesh(p, N=4)
    nx = 5
    g = M["glo_num"].reshape(6, nx, nx, nx)
    assert np.array_equal(g[:, 0], g[:, -1])
    f = np.cos(2 * np.pi * M["z"]) + M["x"] * M["y"]   # periodic in z with period 1
    avg = mio._dsop(M["glo_num"], f, "+") * M["mult"]
    np.testing.assert_allclose(avg, f, rtol=0, atol=1e-13)
    cnt = np.rint(1 / M["mult"]).reshape(6, nx, nx, nx)
    assert np.all(cnt[:, 0, 1:-1, 1:-1] == 2) and np.all(cnt[:, 1:-1, 1:-1, 1:-1] == 1)


def _cubed_shell(ri=0.5, ro=1.0, k=2, spheres=True):
    """A spherical shell from the six faces of a cube (k x k elements per face,
    one across): corners on the spheres, 's' records on the inner (face 5) and
    outer (face 6) sides, walls there."""
    frames = [((1, 0, 0), (0, 1, 0), (0, 0, 1)), ((-1, 0, 0), (0, 0, 1), (0, 1, 0)),
              ((0, 1, 0), (0, 0, 1), (1, 0, 0)), ((0, -1, 0), (1, 0, 0), (0, 0, 1)),
              ((0, 0, 1), (1, 0, 0), (0, 1, 0)), ((0, 0, -1), (0, 1, 0), (1, 0, 0))]
    us = np.linspace(-1, 1, k + 1)
    xc, yc, zc, curves, bcs = [], [], [], [], []
    e = 0
    for nrm, eu, ev in frames:
        nrm, eu, ev = (np.array(a, dtype=float) for a in (nrm, eu, ev))
        for jv in range(k):
            for iu in range(k):
                pts = []
                for r in (ri, ro):
                    for (a, b) in ((0, 0), (1, 0), (1, 1), (0, 1)):
                        p = nrm + us[iu + a] * eu + us[jv + b] * ev
                        pts.append(r * p / np.linalg.norm(p))
                pts = np.array(pts)
                xc.append(pts[:, 0])
                yc.append(pts[:, 1])
                zc.append(pts[:, 2])
                e += 1
                if spheres:
                    curves += [(e, 5, (0.0, 0.0, 0.0, ri, 0.0), "s"),
                               (e, 6, (0.0, 0.0, 0.0, ro, 0.0), "s")]
                bcs += [(e, 5, (0.0,) * 5, "W  "), (e, 6, (0.0,) * 5, "W  ")]
    return np.array(xc), np.array(yc), np.array(zc), curves, bcs


def test_spherical_faces_make_an_exact_shell(mio, tmp_path):
    """Spherical faces (sphsrf): the GLL points of the inner and outer faces
    lie on their spheres, the numbering is continuous, and the volume
    converges to the shell's (straight-sided elements miss it by percents)."""
    ri, ro = 0.5, 1.0
    exact = 4.0 / 3.0 * np.pi * (ro ** 3 - ri ** 3)
    vols = {}
    for sph in (True, False):
        xc, yc, zc, curves, bcs = _cubed_shell(ri, ro, spheres=sph)
        p = tmp_path / f"shell{sph}.re2"
        write_re2(p, xc, yc, zc, bcs, curves=curves)
        M = mio.load_mesh(p, N=7)
        assert np.all(M["jac"] > 0)
        vols[sph] = M["vol"]
        f = M["x"] * M["y"] + np.sin(M["z"])
        avg = mio._dsop(M["glo_num"], f, "+") * M["mult"]
        np.testing.assert_allclose(avg, f, rtol=0, atol=1e-13)
        if sph:
            rad = np.sqrt(M["x"] ** 2 + M["y"] ** 2 + M["z"] ** 2).reshape(M["nel"], 8, 8, 8)
            np.testing.assert_allclose(rad[:, 0], ri, rtol=0, atol=1e-14)
            np.testing.assert_allclose(rad[:, -1], ro, rtol=0, atol=1e-14)
    assert abs(vols[True] - exact) <= 1e-11 * exact, (vols[True], exact)  # 1.8e-13 at N = 7
    assert abs(vols[False] - exact) > 1e-1 * exact                          # 23 % off


def test_ma2_reader(mio, tmp_path):
    """A .ma2 map file as genmap writes it (#v001 header a5,7i12, the test
    value, then partition and eight vertex ids per element, either byte
    order): read back, and load_mesh numbers the mesh as from the corners."""
    import struct
    xc, yc, zc, lattice, bcs = box_elements(3, 2, 2)
    p = tmp_path / "box.re2"
    write_re2(p, xc, yc, zc, bcs)
    M = mio.load_mesh(p, N=4)
    part = np.arange(12) % 3
    for big in (False, True):
        e = ">" if big else "<"
        hdr = f"#v001{12:12d}{M['vertex'].max():12d}{1:12d}{2:12d}{0:12d}{0:12d}{0:12d}"
        out = hdr.ljust(132).encode() + struct.pack(e + "f", 6.54321)
        for q in range(12):
            out += struct.pack(e + "9i", part[q], *M["vertex"][q])
        m2 = tmp_path / f"box{big}.ma2"
        m2.write_bytes(out)
        R = mio.read_ma2(m2)
        assert R["nel"] == 12 and R["nv"] == 8
        assert np.array_equal(R["vertex"], M["vertex"]) and np.array_equal(R["part"], part)
    M2 = mio.load_mesh(p, N=4, ma2=m2)
    assert np.array_equal(M2["glo_num"], M["glo_num"])
