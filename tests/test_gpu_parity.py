"""GPU parity: libnekgpu.so (through its C ABI) against the CPU oracle.

Tolerances:
  * EXACT mode (FP64 products and sums rounded one by one in the reference's
    order): axhelm, dssum, setprec are bit-identical to the oracle.
  * default mode (fused multiply-adds): axhelm within 1e-13 relative (max
    norm).
  * PCG: the same iteration count as the oracle (+-1 allowed only at the
    stopping threshold), rbn0 within 1e-13 relative, and the solution within
    max(1e-12, 2 * spread) relative (L2) of the single-rank oracle, where
    spread is how far the reference's own solution moves when its dot
    products are summed as P ranks would (P = 2, 3, 4, 7, 8): the GPU sums in
    a tree, which no serial order reproduces, and CG carries that rounding
    into the iterates at the 1e-12 level.
"""
import numpy as np
import pytest

from conftest import rank_spread, rng_unit_vector

pytestmark = pytest.mark.gpu


def _setup(NekGpu, P):
    lib = NekGpu(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    return lib


@pytest.fixture(scope="module")
def cfg1(oracle):
    """Config-1 shape: 4x4x4 elements, N=7, Dirichlet on all faces, seed 0."""
    return oracle.box_problem(8, 4, 4, 4, v=rng_unit_vector(0))


@pytest.fixture(scope="module")
def cfgp(oracle):
    """Config-2 shape at small size: Dirichlet x, periodic y/z, N=5."""
    return oracle.box_problem(6, 3, 4, 3, periodic=(False, True, True), v=rng_unit_vector(1))


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_gs_maps_bit_exact(gpu_lib, oracle, cfg1, cfgp):
    for P in (cfg1, cfgp):
        lib = _setup(gpu_lib, P)
        start, idx = lib.gs_maps()
        rs, ri, _ = oracle.GS(P["glo_num"]).maps()
        assert np.array_equal(start, rs)
        assert np.array_equal(idx, ri)


def test_dssum_and_dsop_bit_exact(gpu_lib, oracle, cfgp):
    torch = pytest.importorskip("torch")
    P = cfgp
    lib = _setup(gpu_lib, P)
    u = np.random.default_rng(7).standard_normal(P["n"])
    ref = P["ops"].dssum(u)
    got = u.copy()
    lib.dssum(got)
    assert np.array_equal(got, ref)
    for op in ("*", "M", "m"):
        t = torch.tensor(u, device="cuda")
        lib.dsop(t, op)
        assert np.array_equal(t.cpu().numpy(), P["ops"].dsop(u, op)), op


@pytest.mark.parametrize("nx1", [2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12])
def test_axhelm_exact_bitwise_all_orders(gpu_lib, oracle, nx1):
    P = oracle.box_problem(nx1, 2, 2, 3, v=rng_unit_vector(nx1))
    lib = _setup(gpu_lib, P)
    lib.set_exact(True)
    n = P["n"]
    rng = np.random.default_rng(nx1)
    u = rng.standard_normal(n)
    for h1, h2 in ((np.ones(n), np.zeros(n)), (np.ones(n), np.full(n, 10.0)),
                   (np.exp(0.3 * rng.standard_normal(n)), rng.uniform(0, 5, n))):
        au = np.zeros(n)
        lib.axhelm(au, u, h1, h2)
        assert np.array_equal(au, P["ops"].axhelm(u, h1, h2))


@pytest.mark.parametrize("df", [1, 0])
@pytest.mark.parametrize("tma", [1, 0])
@pytest.mark.parametrize("nx1", [2, 3, 4, 6, 8, 9, 10, 12])
def test_axhelm_fma_within_tolerance(gpu_lib, oracle, nx1, tma, df):
    """Default (fused multiply-add) operator, TMA-staged (even lx1) or plain
    loads, with double-float contractions (the default) or FP64 ones."""
    P = oracle.box_problem(nx1, 3, 2, 2, v=rng_unit_vector(20 + nx1))
    lib = _setup(gpu_lib, P)
    lib.set_option(5, tma)
    lib.set_option(10, df)
    n = P["n"]
    rng = np.random.default_rng(11)
    u = rng.standard_normal(n)
    for h1, h2 in ((np.ones(n), np.zeros(n)), (np.ones(n), np.full(n, 10.0)),
                   (np.exp(0.3 * rng.standard_normal(n)), rng.uniform(0, 5, n))):
        au = np.zeros(n)
        lib.axhelm(au, u, h1, h2)
        assert rel(au, P["ops"].axhelm(u, h1, h2)) < 1e-13


def test_axhelm_device_path_equals_host_path(gpu_lib, oracle, cfg1):
    torch = pytest.importorskip("torch")
    P = cfg1
    lib = _setup(gpu_lib, P)
    n = P["n"]
    u = np.random.default_rng(12).standard_normal(n)
    h1, h2 = np.ones(n), np.zeros(n)
    au = np.zeros(n)
    lib.axhelm(au, u, h1, h2)
    tu = torch.tensor(u, device="cuda")
    tau = torch.zeros(n, dtype=torch.float64, device="cuda")
    lib.axhelm(tau, tu, torch.tensor(h1, device="cuda"), torch.tensor(h2, device="cuda"))
    assert np.array_equal(tau.cpu().numpy(), au)


def test_setprec_bit_exact(gpu_lib, oracle, cfgp):
    P = cfgp
    lib = _setup(gpu_lib, P)
    n = P["n"]
    rng = np.random.default_rng(5)
    for h1, h2 in ((np.ones(n), np.zeros(n)), (np.ones(n), np.full(n, 10.0)),
                   (np.exp(0.3 * rng.standard_normal(n)), rng.uniform(0, 5, n))):
        d = np.zeros(n)
        lib.setprec(d, h1, h2)
        assert np.array_equal(d, P["ops"].setprec(h1, h2))


def _rhs(P, seed, dist="uniform"):
    rng = np.random.default_rng(seed)
    ops = P["ops"]
    f = rng.uniform(-1, 1, P["n"]) if dist == "uniform" else rng.standard_normal(P["n"])
    f = ops.dssum(f) * P["mult"]  # one value per global node
    return P["bm1"] * f


@pytest.mark.parametrize("exact,graph", [(True, 1), (False, 1), (False, 0)])
def test_hmholtz_poisson_config1(gpu_lib, oracle, cfg1, exact, graph):
    P = cfg1
    lib = _setup(gpu_lib, P)
    lib.set_exact(exact)
    lib.set_option(6, graph)
    n = P["n"]
    h1, h2 = np.ones(n), np.zeros(n)
    rhs = _rhs(P, 0)
    u_ref, rhs_ref, it_ref, r0_ref, r2_ref = P["ops"].hmholtz(rhs, h1, h2, P["mask"], P["mult"],
                                                              P["binv"], -1e-10, maxcg=10 ** 6)
    u = np.zeros(n)
    r = rhs.copy()
    it, r0, r2, rc = lib.hmholtz("TEMP", u, r, h1, h2, P["mask"], P["mult"], 1, -1e-10, 10 ** 6, 1,
                                 P["binv"], maxcg=10 ** 6)
    assert rc == 0
    assert np.array_equal(r, rhs_ref)  # dssum + mask of the rhs, in place
    assert abs(r0 - r0_ref) <= 1e-13 * r0_ref
    assert abs(it - it_ref) <= 1, (it, it_ref)
    assert r2 <= 1e-10 * r0
    base, spread = rank_spread(oracle, P, lambda ops: ops.hmholtz(
        rhs, h1, h2, P["mask"], P["mult"], P["binv"], -1e-10, maxcg=10 ** 6)[0])
    assert np.array_equal(base, u_ref)
    err = np.linalg.norm(u - u_ref) / np.linalg.norm(u_ref)
    assert err <= max(1e-12, 2 * spread), (err, spread)


def test_cggo_helmholtz_periodic(gpu_lib, oracle, cfgp):
    torch = pytest.importorskip("torch")
    P = cfgp
    lib = _setup(gpu_lib, P)
    n = P["n"]
    h1, h2 = np.ones(n), np.full(n, 10.0)
    f = P["ops"].dssum(_rhs(P, 3, "normal")) * P["mask"]
    x_ref, it_ref, r0_ref, r2_ref = P["ops"].cggo(f, h1, h2, P["mask"], P["mult"], P["binv"], -1e-10,
                                                  maxcg=10 ** 6)
    dev = lambda a: torch.tensor(a, device="cuda")
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    it, r0, r2, rc = lib.cggo(x, dev(f), dev(h1), dev(h2), dev(P["mask"]), dev(P["mult"]), 1, -1e-10,
                              10 ** 6, 1, dev(P["binv"]), maxcg=10 ** 6)
    assert rc == 0
    assert abs(it - it_ref) <= 1
    _, spread = rank_spread(oracle, P, lambda ops: ops.cggo(
        f, h1, h2, P["mask"], P["mult"], P["binv"], -1e-10, maxcg=10 ** 6)[0])
    err = np.linalg.norm(x.cpu().numpy() - x_ref) / np.linalg.norm(x_ref)
    assert err <= max(1e-12, 2 * spread), (err, spread)


def test_cggo_iteration_cap_reports_not_converged(gpu_lib, oracle, cfg1):
    P = cfg1
    lib = _setup(gpu_lib, P)
    n = P["n"]
    f = P["ops"].dssum(_rhs(P, 0)) * P["mask"]
    x = np.zeros(n)
    it, r0, r2, rc = lib.cggo(x, f, np.ones(n), np.zeros(n), P["mask"], P["mult"], 1, -1e-10, 10 ** 6,
                              1, P["binv"], maxcg=7)
    x_ref, it_ref, _, r2_ref = P["ops"].cggo(f, np.ones(n), np.zeros(n), P["mask"], P["mult"],
                                             P["binv"], -1e-10, maxcg=7)
    assert rc == -5 and it == 7 == it_ref
    assert abs(r2 - r2_ref) <= 1e-10 * r2_ref
    assert np.linalg.norm(x - x_ref) <= 1e-12 * np.linalg.norm(x_ref)


def test_zero_rhs_returns_zero(gpu_lib, oracle, cfg1):
    P = cfg1
    lib = _setup(gpu_lib, P)
    n = P["n"]
    x = np.ones(n)
    it, r0, r2, rc = lib.cggo(x, np.zeros(n), np.ones(n), np.zeros(n), P["mask"], P["mult"], 1,
                              -1e-10, 100, 1, P["binv"])
    assert rc == 0 and it == 0 and np.all(x == 0)


def test_errors_are_status_codes(gpu_lib, oracle, cfg1):
    from nek5000_gb300 import _capi
    lib = gpu_lib(0)
    n = cfg1["n"]
    with pytest.raises(_capi.NekGpuError) as e:
        lib.axhelm(np.zeros(n), np.zeros(n), np.ones(n), np.zeros(n))
    assert e.value.code == _capi.ENOSETUP
    with pytest.raises(_capi.NekGpuError) as e:
        lib.setup(13, 1, np.eye(13), np.zeros((6, 13 ** 3)), np.ones(13 ** 3),
                  np.zeros(13 ** 3, np.int64))
    assert e.value.code == _capi.EINVAL
    P = cfg1
    lib = _setup(gpu_lib, P)
    f = P["ops"].dssum(_rhs(P, 0)) * P["mask"]
    f[123] = np.nan
    with pytest.raises(_capi.NekGpuError) as e:
        lib.cggo(np.zeros(n), f, np.ones(n), np.zeros(n), P["mask"], P["mult"], 1, -1e-10, 100, 1,
                 P["binv"])
    assert e.value.code == _capi.ENAN


def test_cggo_irregular_group_sizes(gpu_lib, oracle):
    """Groups of 3 and 5 copies (as unstructured meshes have) take the generic
    path of the boundary-group kernel; the solve still matches the oracle."""
    torch = pytest.importorskip("torch")
    P0 = oracle.box_problem(6, 3, 3, 3, v=rng_unit_vector(9))
    nx, nel = P0["nx1"], P0["nel"]
    glo = P0["glo_num"].copy().reshape(nel, nx, nx, nx)
    rng = np.random.default_rng(9)
    # give interior points of some elements the id of a node on an interior
    # face of the same element: that group grows from 2 to 3 (or 4 -> 5)
    for e in rng.choice(nel, 10, replace=False):
        glo[e, 2, 2, 2] = glo[e, 2, 2, 0] if glo[e, 2, 2, 0] else glo[e, 2, 2, -1]
        glo[e, 3, 1, 1] = glo[e, 3, 0, 0]
    glo = glo.reshape(-1)
    ops = oracle.Ops(nx, nel, P0["D"], P0["g"], P0["bm1"], glo, 1)
    n = P0["n"]
    mask = ops.dsop(P0["mask"], "*")
    mult = 1.0 / ops.dssum(np.ones(n))
    binv = 1.0 / ops.dssum(P0["bm1"])
    sizes = np.bincount(np.unique(glo[glo > 0], return_counts=True)[1])
    assert sizes[3:].sum() - sizes[4] - (sizes[8] if len(sizes) > 8 else 0) > 0
    f = ops.dssum(P0["bm1"] * rng.standard_normal(n)) * mask
    h1, h2 = np.ones(n), np.full(n, 3.0)
    x_ref, it_ref, _, _ = ops.cggo(f, h1, h2, mask, mult, binv, -1e-10, maxcg=10 ** 6)
    lib = gpu_lib(0)
    lib.setup(nx, nel, P0["D"], P0["g"], P0["bm1"], glo)
    dev = lambda a: torch.tensor(a, device="cuda")
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    it, r0, r2, rc = lib.cggo(x, dev(f), dev(h1), dev(h2), dev(mask), dev(mult), 1, -1e-10,
                              10 ** 6, 1, dev(binv), maxcg=10 ** 6)
    assert rc == 0 and abs(it - it_ref) <= 1
    assert np.linalg.norm(x.cpu().numpy() - x_ref) <= 1e-11 * np.linalg.norm(x_ref)


@pytest.mark.parametrize("exact", [False, True])
def test_cggo_null_space_correction(gpu_lib, oracle, exact):
    """No Dirichlet point and h2 = 0 (Neumann in x, periodic in y and z): cggo
    applies its mean correction (hmholtz.f:705-750) -- r += rmean dssum(bm1)
    before the loop, z += smean sum(z bm1) in every iteration.  The GPU must
    follow the oracle's iterations and solution; the mixed and batched solves
    refuse the singular system."""
    torch = pytest.importorskip("torch")
    from nek5000_gb300 import _capi, NekGpuBatch
    P = oracle.box_problem(7, 3, 3, 3, periodic=(False, True, True),
                           dirichlet=(False,) * 6, v=rng_unit_vector(31))
    n = P["n"]
    assert P["mask"].min() == 1.0
    rng = np.random.default_rng(31)
    f = P["ops"].dssum(P["bm1"] * (P["ops"].dssum(rng.standard_normal(n)) * P["mult"]))
    h1, h2 = np.ones(n), np.zeros(n)
    x_ref, it_ref, r0_ref, r2_ref = P["ops"].cggo(f, h1, h2, P["mask"], P["mult"], P["binv"],
                                                  -1e-10, maxcg=10 ** 6)
    _, spread = rank_spread(oracle, P, lambda ops: ops.cggo(
        f, h1, h2, P["mask"], P["mult"], P["binv"], -1e-10, maxcg=10 ** 6)[0])
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    lib.set_exact(exact)
    dev = lambda a: torch.tensor(a, device="cuda")
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    it, r0, r2, rc = lib.cggo(x, dev(f), dev(h1), dev(h2), dev(P["mask"]), dev(P["mult"]), 1,
                              -1e-10, 10 ** 6, 1, dev(P["binv"]), maxcg=10 ** 6)
    assert rc == 0
    assert abs(it - it_ref) <= 1, (it, it_ref)
    assert abs(r0 - r0_ref) <= 1e-12 * r0_ref
    err = np.linalg.norm(x.cpu().numpy() - x_ref) / np.linalg.norm(x_ref)
    print(f"null-space correction: {it} iterations (oracle {it_ref}), rel. error {err:.2e}, "
          f"oracle spread {spread:.2e}")
    assert err <= max(1e-12, 2 * spread)
    # mixed and batched solves refuse it
    xm = torch.zeros(n, dtype=torch.float64, device="cuda")
    with pytest.raises(_capi.NekGpuError) as e:
        lib.cggo_mixed(xm, dev(f), dev(h1), dev(h2), dev(P["mask"]), dev(P["mult"]), 1, -1e-10,
                       10 ** 6, 1, dev(P["binv"]))
    assert e.value.code == _capi.EINVAL
    B = NekGpuBatch(0)
    B.add(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    res = B.solve([xm], [dev(f)], [dev(h1)], [dev(h2)], [dev(P["mask"])], [dev(P["mult"])],
                  [dev(P["binv"])], tin=-1e-10)
    assert res["status"] == [_capi.EINVAL]


@pytest.mark.parametrize("case", [((7, 3, 3, 3), (False,) * 6),
                                  ((7, 3, 3, 3), (False, True, False, False, False, False)),
                                  ((6, 4, 3, 2), (False,) * 6)])
def test_cggo_neumann_faces(gpu_lib, oracle, case):
    """Unmasked element faces on the domain boundary (Neumann) make singleton
    boundary groups live.  When a size class does not fill its last 16-byte
    run, the entries up to the boundary are padding and belong to no group;
    the mask and multiplicity weights of the class's last group must ignore
    them.  Iteration counts and solutions follow the oracle."""
    torch = pytest.importorskip("torch")
    (nx1, kx, ky, kz), dirichlet = case
    P = oracle.box_problem(nx1, kx, ky, kz, periodic=(False, True, True), dirichlet=dirichlet,
                           v=rng_unit_vector(33))
    n = P["n"]
    rng = np.random.default_rng(33)
    f = P["ops"].dssum(P["bm1"] * (P["ops"].dssum(rng.standard_normal(n)) * P["mult"]))
    f = f * P["mask"]
    h1, h2 = np.ones(n), np.ones(n)
    x_ref, it_ref, r0_ref, r2_ref = P["ops"].cggo(f, h1, h2, P["mask"], P["mult"], P["binv"],
                                                  -1e-10, maxcg=10 ** 6)
    _, spread = rank_spread(oracle, P, lambda ops: ops.cggo(
        f, h1, h2, P["mask"], P["mult"], P["binv"], -1e-10, maxcg=10 ** 6)[0])
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    dev = lambda a: torch.tensor(a, device="cuda")
    x = torch.zeros(n, dtype=torch.float64, device="cuda")
    it, r0, r2, rc = lib.cggo(x, dev(f), dev(h1), dev(h2), dev(P["mask"]), dev(P["mult"]), 1,
                              -1e-10, 10 ** 6, 1, dev(P["binv"]), maxcg=10 ** 6)
    assert rc == 0 and abs(it - it_ref) <= 1, (it, it_ref)
    err = np.linalg.norm(x.cpu().numpy() - x_ref) / np.linalg.norm(x_ref)
    assert err <= max(1e-12, 2 * spread), (err, spread)
