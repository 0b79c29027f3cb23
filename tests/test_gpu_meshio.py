"""Meshes read from .re2 files through the solve path: the numbering comes
from the library's connectivity (tools/gencon algorithm) and set_vert, the
geometry from the trilinear map of the file's corners.  The GPU solves must
match the oracle on the same arrays as the box meshes do (tolerances as in
test_gpu_parity.py): gather-scatter maps bit-identical, FP64 PCG within
max(1e-12, 2 x the oracle's own rank spread), the mixed solve to the FP64
tolerance."""
import numpy as np
import pytest

from conftest import rank_spread
from re2_util import box_elements, rotate_elements, write_re2

pytestmark = pytest.mark.gpu


def _mesh(tmp_path, case):
    from nek5000_gb300 import meshio
    if case == "rotated":  # mixed local frames, natural boundaries
        xc, yc, zc, _, _ = box_elements(4, 3, 3, jitter=0.2, seed=21,
                                        perm=np.random.default_rng(21).permutation(36))
        xc, yc, zc = rotate_elements(xc, yc, zc, seed=21)
        bcs = []
    elif case == "periodic":  # periodic in y, walls on the x and z faces
        xc, yc, zc, _, bcs = box_elements(4, 3, 3, periodic_y=True, jitter=0.2, seed=22,
                                          perm=np.random.default_rng(22).permutation(36))
    elif case == "shell":  # a spherical shell with spherical faces, walls inside and outside
        from test_meshio import _cubed_shell
        xc, yc, zc, curves, bcs = _cubed_shell()
        p = tmp_path / "shell.re2"
        write_re2(p, xc, yc, zc, bcs, curves=curves)
        return meshio.load_mesh(p, N=7)
    else:  # an annular ring with circular-arc edges, walls inside and outside
        from test_meshio import _annulus
        xc, yc, zc, curves, bcs = _annulus(nt=12, nr=3, nz=2)
        p = tmp_path / "annulus.re2"
        write_re2(p, xc, yc, zc, bcs, curves=curves)
        return meshio.load_mesh(p, N=7)
    p = tmp_path / f"{case}.re2"
    write_re2(p, xc, yc, zc, bcs)
    return meshio.load_mesh(p, N=7)


@pytest.mark.parametrize("case", ["rotated", "periodic", "annulus", "shell"])
def test_re2_mesh_solves_match_the_oracle(gpu_lib, oracle, tmp_path, case):
    torch = pytest.importorskip("torch")
    M = _mesh(tmp_path, case)
    n = M["n"]
    ops = oracle.Ops(M["lx1"], M["nel"], M["D"], M["g"], M["bm1"], M["glo_num"])
    P = dict(nx1=M["lx1"], nel=M["nel"], D=M["D"], g=M["g"], bm1=M["bm1"],
             glo_num=M["glo_num"], ops=ops)
    lib = gpu_lib(0)
    lib.setup(M["lx1"], M["nel"], M["D"], M["g"], M["bm1"], M["glo_num"])
    start, idx = lib.gs_maps()
    rs, ri, _ = oracle.GS(M["glo_num"]).maps()
    assert np.array_equal(start, rs) and np.array_equal(idx, ri)
    h1, h2 = np.ones(n), np.full(n, 10.0)
    rng = np.random.default_rng(30)
    f = ops.dssum(M["bm1"] * rng.standard_normal(n)) * M["mask"]
    x_ref, it_ref, r0_ref, _ = ops.cggo(f, h1, h2, M["mask"], M["mult"], M["binv"], -1e-10,
                                        maxcg=10 ** 6)
    dev = lambda a: torch.tensor(a, device="cuda")
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    it, r0, r2, rc = lib.cggo(x, dev(f), dev(h1), dev(h2), dev(M["mask"]), dev(M["mult"]), 1,
                              -1e-10, 10 ** 6, 1, dev(M["binv"]), maxcg=10 ** 6)
    assert rc == 0 and abs(it - it_ref) <= 1, (it, it_ref)
    assert abs(r0 - r0_ref) <= 1e-13 * r0_ref
    _, spread = rank_spread(oracle, P, lambda o: o.cggo(
        f, h1, h2, M["mask"], M["mult"], M["binv"], -1e-10, maxcg=10 ** 6)[0])
    err = np.linalg.norm(x.cpu().numpy() - x_ref) / np.linalg.norm(x_ref)
    assert err <= max(1e-12, 2 * spread), (err, spread)
    # the mixed solve on the same mesh: FP64 residual and agreement
    xm = torch.zeros(n, dtype=torch.float64, device="cuda")
    no, ni, r0m, r2m, rcm = lib.cggo_mixed(xm, dev(f), dev(h1), dev(h2), dev(M["mask"]),
                                           dev(M["mult"]), 1, -1e-10, 10 ** 6, 1, dev(M["binv"]))
    assert rcm == 0
    xmh = xm.cpu().numpy()
    r = f - ops.dssum(ops.axhelm(xmh, h1, h2)) * M["mask"]
    rn = np.sqrt(np.sum(M["mult"] * M["binv"] * r * r) / M["vol"])
    assert rn <= 1.05e-10 * r0m
    assert np.linalg.norm(xmh - x_ref) <= 1e-8 * np.linalg.norm(x_ref)
    print(case, "fp64 iterations", it, "mixed", no, ni)


@pytest.mark.parametrize("nx1", [2, 3, 5, 8, 10, 12])
def test_device_geometry_is_the_reference_bit_for_bit(gpu_lib, oracle, nx1):
    """nekgpu_setup_xyz: G1..G6 and bm1 formed on the GPU from xm1, ym1, zm1
    equal the oracle's xyzrst / glmapm1 / geodat1 restatement exactly."""
    from conftest import rng_unit_vector
    P = oracle.box_problem(nx1, 3, 2, 2, v=rng_unit_vector(nx1 + 40), amp=0.08)
    lib = gpu_lib(0)
    lib.setup_xyz(P["nx1"], P["nel"], P["D"], P["wgll"], P["x"], P["y"], P["z"], P["glo_num"])
    g, bm1 = lib.geometry()
    assert np.array_equal(g, P["g"].reshape(6, -1))
    assert np.array_equal(bm1, P["bm1"])


def test_moving_mesh_geometry_update(gpu_lib, oracle):
    """nekgpu_geom_update_dev: new coordinates of the same mesh give the
    oracle's geometry of the moved mesh, and the solve sees it (volume and
    operator both updated)."""
    torch = pytest.importorskip("torch")
    from conftest import rng_unit_vector
    P = oracle.box_problem(8, 3, 3, 2, v=rng_unit_vector(50), amp=0.05)
    Q = oracle.box_problem(8, 3, 3, 2, v=rng_unit_vector(51), amp=0.09)  # the moved mesh
    lib = gpu_lib(0)
    lib.setup_xyz(P["nx1"], P["nel"], P["D"], P["wgll"], P["x"], P["y"], P["z"], P["glo_num"])
    dev = lambda a: torch.tensor(a, device="cuda")
    lib.geom_update(P["wgll"], dev(Q["x"]), dev(Q["y"]), dev(Q["z"]))
    g, bm1 = lib.geometry()
    assert np.array_equal(g, Q["g"].reshape(6, -1)) and np.array_equal(bm1, Q["bm1"])
    n = Q["n"]
    h1, h2 = np.ones(n), np.full(n, 10.0)
    f = Q["ops"].dssum(Q["bm1"] * np.random.default_rng(52).standard_normal(n)) * Q["mask"]
    x_ref, it_ref, r0_ref, _ = Q["ops"].cggo(f, h1, h2, Q["mask"], Q["mult"], Q["binv"], -1e-10,
                                             maxcg=10 ** 6)
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    it, r0, r2, rc = lib.cggo(x, dev(f), dev(h1), dev(h2), dev(Q["mask"]), dev(Q["mult"]), 1,
                              -1e-10, 10 ** 6, 1, dev(Q["binv"]), maxcg=10 ** 6)
    assert rc == 0 and abs(it - it_ref) <= 1
    assert abs(r0 - r0_ref) <= 1e-13 * r0_ref  # the volume was updated too
    assert np.linalg.norm(x.cpu().numpy() - x_ref) <= 1e-10 * np.linalg.norm(x_ref)
    # a tangled element map is refused, not computed
    bad = Q["x"].copy()
    P3 = Q["nx1"] ** 3
    bad[:P3] = bad[:P3][::-1].copy()  # mirror element 0
    from nek5000_gb300 import _capi
    with pytest.raises(_capi.NekGpuError) as ei:
        lib.geom_update(P["wgll"], dev(bad), dev(Q["y"]), dev(Q["z"]))
    assert ei.value.code == _capi.EINVAL
