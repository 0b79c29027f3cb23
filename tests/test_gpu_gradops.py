"""The gradient-type operators of the splitting step on the device
(nekgpu_wgradm1_dev, _dudxyz_dev, _cdtp_dev, _op_curl_dev) against the
oracle's restatement (oracle/gradops.c): both evaluate the reference's
arithmetic in its order without fused multiply-adds, so they must agree bit
for bit, on a deformed box and on a periodic one."""
import numpy as np
import pytest

from conftest import rng_unit_vector

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["box", "periodic"])
def test_gradops_match_the_oracle_bit_for_bit(gpu_lib, oracle, case):
    torch = pytest.importorskip("torch")
    if case == "box":
        P = oracle.box_problem(7, 3, 2, 2, v=rng_unit_vector(151))
    else:
        P = oracle.box_problem(6, 3, 3, 3, periodic=(False, True, True), v=rng_unit_vector(152))
    nx1, nel, n = P["nx1"], P["nel"], P["n"]
    rst, jac = oracle.geom_rst(nx1, nel, P["x"], P["y"], P["z"])
    lib = gpu_lib(0)
    lib.setup_xyz(nx1, nel, P["D"], P["wgll"], P["x"], P["y"], P["z"], P["glo_num"])
    rng = np.random.default_rng(153)
    u1, u2, u3 = (rng.standard_normal(n) for _ in range(3))
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")
    zeros = lambda: torch.zeros(n, dtype=torch.float64, device="cuda")
    host = lambda t: t.cpu().numpy()
    # weak gradient
    g = [zeros() for _ in range(3)]
    lib.wgradm1(*g, dev(u1))
    for a, b in zip(g, oracle.wgradm1(nx1, nel, u1, rst)):
        assert np.array_equal(host(a), b)
    for isd in (1, 2, 3):
        du = zeros()
        lib.dudxyz(du, dev(u2), isd)
        assert np.array_equal(host(du), oracle.dudxyz(nx1, nel, u2, rst, jac, isd)), isd
        dt = zeros()
        lib.cdtp(dt, dev(u3), isd)
        assert np.array_equal(host(dt), oracle.cdtp(nx1, nel, u3, rst, jac, P["bm1"], isd)), isd
    for ifavg in (False, True):
        w = [zeros() for _ in range(3)]
        lib.op_curl(*w, dev(u1), dev(u2), dev(u3), ifavg=ifavg, binv=dev(P["binv"]))
        want = oracle.op_curl(P["ops"], u1, u2, u3, rst, jac, P["bm1"], P["binv"], ifavg=ifavg)
        for a, b in zip(w, want):
            assert np.array_equal(host(a), b), ifavg


def test_gradops_need_coordinates(gpu_lib, oracle):
    torch = pytest.importorskip("torch")
    from nek5000_gb300 import _capi
    P = oracle.box_problem(5, 2, 2, 2, v=rng_unit_vector(154))
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    u = torch.zeros(P["n"], dtype=torch.float64, device="cuda")
    with pytest.raises(_capi.NekGpuError) as ei:
        lib.dudxyz(u.clone(), u, 1)
    assert ei.value.code == _capi.ENOSETUP


def test_convection_matches_the_oracle_bit_for_bit(gpu_lib, oracle):
    torch = pytest.importorskip("torch")
    P = oracle.box_problem(7, 3, 2, 2, v=rng_unit_vector(155))
    nx1, nel, n = P["nx1"], P["nel"], P["n"]
    rst, jac = oracle.geom_rst(nx1, nel, P["x"], P["y"], P["z"])
    lib = gpu_lib(0)
    lib.setup_xyz(nx1, nel, P["D"], P["wgll"], P["x"], P["y"], P["z"], P["glo_num"])
    rng = np.random.default_rng(156)
    v = [rng.standard_normal(n) for _ in range(3)]
    u = rng.standard_normal(n)
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")
    du = torch.zeros(n, dtype=torch.float64, device="cuda")
    lib.conv1(du, dev(u), [dev(a) for a in v])
    assert np.array_equal(du.cpu().numpy(), oracle.conv1(nx1, nel, u, v, rst, jac))
    bf = [rng.standard_normal(n) for _ in range(3)]
    bfd = [dev(a) for a in bf]
    lib.advab(bfd, [dev(a) for a in v])
    for a, b in zip(bfd, oracle.advab(nx1, nel, bf, v, P["bm1"], rst, jac)):
        assert np.array_equal(a.cpu().numpy(), b)


@pytest.mark.parametrize("nx1,lxd", [(6, 9), (8, 12)])
def test_dealiased_convection_matches_the_oracle(gpu_lib, oracle, nx1, lxd):
    """convop with dealiasing on the device against the oracle's
    convect_new / bm1 (to 1e-12: both sum the tensor steps in their own
    order); advab follows the dealiased path once it is set up."""
    torch = pytest.importorskip("torch")
    P = oracle.box_problem(nx1, 3, 2, 2, v=rng_unit_vector(157))
    nel, n = P["nel"], P["n"]
    rst, jac = oracle.geom_rst(nx1, nel, P["x"], P["y"], P["z"])
    lib = gpu_lib(0)
    lib.setup_xyz(nx1, nel, P["D"], P["wgll"], P["x"], P["y"], P["z"], P["glo_num"])
    lib.dealias_setup(lxd)
    rng = np.random.default_rng(158)
    v = [rng.standard_normal(n) for _ in range(3)]
    u = rng.standard_normal(n)
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")
    c = torch.zeros(n, dtype=torch.float64, device="cuda")
    lib.convop(c, dev(u), [dev(a) for a in v])
    want = oracle.convect_new(nx1, nel, lxd, u, v, rst, P["bm1"])
    assert np.allclose(c.cpu().numpy(), want, rtol=0, atol=1e-12 * np.abs(want).max())
    bf = [rng.standard_normal(n) for _ in range(3)]
    bfd = [dev(a) for a in bf]
    lib.advab(bfd, [dev(a) for a in v])
    for k in range(3):
        ck = oracle.convect_new(nx1, nel, lxd, v[k], v, rst, P["bm1"])
        want = bf[k] - P["bm1"] * ck
        assert np.allclose(bfd[k].cpu().numpy(), want, rtol=0, atol=1e-12 * np.abs(want).max())


def test_conservative_convection_matches_the_oracle(gpu_lib, oracle):
    torch = pytest.importorskip("torch")
    nx1, lxd = 6, 9
    P = oracle.box_problem(nx1, 3, 2, 2, v=rng_unit_vector(159))
    nel, n = P["nel"], P["n"]
    rst, jac = oracle.geom_rst(nx1, nel, P["x"], P["y"], P["z"])
    lib = gpu_lib(0)
    lib.setup_xyz(nx1, nel, P["D"], P["wgll"], P["x"], P["y"], P["z"], P["glo_num"])
    lib.dealias_setup(lxd)
    rng = np.random.default_rng(160)
    v = [rng.standard_normal(n) for _ in range(3)]
    u = rng.standard_normal(n)
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")
    c = torch.zeros(n, dtype=torch.float64, device="cuda")
    lib.convect_cons(c, dev(u), [dev(a) for a in v])
    want = oracle.convect_cons(nx1, nel, lxd, u, v, rst, P["bm1"])
    assert np.allclose(c.cpu().numpy(), want, rtol=0, atol=1e-12 * np.abs(want).max())


def test_conv2_and_skew_symmetric_form_bit_for_bit(gpu_lib, oracle):
    torch = pytest.importorskip("torch")
    P = oracle.box_problem(6, 3, 2, 2, v=rng_unit_vector(165))
    nx1, nel, n = P["nx1"], P["nel"], P["n"]
    rst, jac = oracle.geom_rst(nx1, nel, P["x"], P["y"], P["z"])
    lib = gpu_lib(0)
    lib.setup_xyz(nx1, nel, P["D"], P["wgll"], P["x"], P["y"], P["z"], P["glo_num"])
    rng = np.random.default_rng(166)
    v = [rng.standard_normal(n) for _ in range(3)]
    fi = rng.standard_normal(n)
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")
    out = torch.zeros(n, dtype=torch.float64, device="cuda")
    lib.conv2(out, dev(fi), [dev(a) for a in v])
    assert np.array_equal(out.cpu().numpy(), oracle.conv2(nx1, nel, fi, v, rst, P["bm1"]))
    ofc = rng.integers(0, 2, size=(nel, 6)).astype(np.int32)
    lib.convopo(out, dev(fi), [dev(a) for a in v], ofc=ofc)
    want = oracle.convopo(nx1, nel, fi, v, rst, jac, P["bm1"], ofc)
    assert np.array_equal(out.cpu().numpy(), want)
