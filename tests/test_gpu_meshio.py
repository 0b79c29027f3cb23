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
    else:  # periodic in y, walls on the x and z faces
        xc, yc, zc, _, bcs = box_elements(4, 3, 3, periodic_y=True, jitter=0.2, seed=22,
                                          perm=np.random.default_rng(22).permutation(36))
    p = tmp_path / f"{case}.re2"
    write_re2(p, xc, yc, zc, bcs)
    return meshio.load_mesh(p, N=7)


@pytest.mark.parametrize("case", ["rotated", "periodic"])
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
