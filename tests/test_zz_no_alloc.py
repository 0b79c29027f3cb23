"""The allocation-free operator entry point, nekgpu_axhelm_dev_noalloc.

It serves callers that cannot let a library allocate device memory (a code
whose device memory belongs to its own pool allocator, a hard memory budget,
a time-step loop that must avoid cudaMalloc's device-wide synchronisation).
Called through the C ABI, it must return what the allocating entry point
nekgpu_axhelm_dev returns for the same arrays, on two calls in a row with
different coefficients (the fixed scratch array keeps the previous call's
contents, which must not leak into the next result), and it must refuse a
mesh larger than its fixed scratch serves.  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rng_unit_vector

pytestmark = pytest.mark.gpu


def _call(L, name, h, au, u, h1, h2):
    one = C.c_int(1)
    return getattr(L, name)(C.byref(h), C.c_void_p(au.data_ptr()), C.c_void_p(u.data_ptr()),
                            C.c_void_p(h1.data_ptr()), C.c_void_p(h2.data_ptr()), C.byref(one),
                            C.byref(one))


def test_noalloc_axhelm_matches_allocating_entry_point(gpu_lib, oracle):
    torch = pytest.importorskip("torch")
    from nek5000_gb300 import _capi
    L = _capi.load()
    P = oracle.box_problem(8, 5, 4, 6, v=rng_unit_vector(40))
    n = P["n"]
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    h = lib._h
    rng = np.random.default_rng(40)
    dev = lambda a: torch.tensor(a, device="cuda")
    cases = [
        (rng.standard_normal(n), np.ones(n), np.full(n, 10.0)),                  # uniform h1, h2
        (rng.standard_normal(n), np.exp(0.3 * rng.standard_normal(n)), rng.uniform(0, 2, n)),
    ]
    for u, h1, h2 in cases:  # two calls in a row, different coefficient modes
        tu, th1, th2 = dev(u), dev(h1), dev(h2)
        ref = torch.zeros(n, dtype=torch.float64, device="cuda")
        got = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
        assert _call(L, "nekgpu_axhelm_dev", h, ref, tu, th1, th2) == 0
        assert _call(L, "nekgpu_axhelm_dev_noalloc", h, got, tu, th1, th2) == 0, lib.last_error()
        # same kernel, same coefficient modes: identical results
        assert torch.equal(got, ref)
        # and the operator itself is right (default fused multiply-add form)
        exp = P["ops"].axhelm(u, h1, h2)
        assert np.max(np.abs(got.cpu().numpy() - exp)) <= 1e-13 * np.max(np.abs(exp))


def test_noalloc_rejects_meshes_beyond_its_scratch(gpu_lib):
    torch = pytest.importorskip("torch")
    from nek5000_gb300 import _capi
    L = _capi.load()
    lx1 = 2
    nel = _capi.NOALLOC_MAX_POINTS // 8 + 1  # one element more than the scratch serves
    n = 8 * nel
    lib = gpu_lib(0)
    lib.setup(lx1, nel, np.array([[-0.5, 0.5], [-0.5, 0.5]]), np.zeros((6, n)), np.ones(n),
              np.zeros(n, dtype=np.int64))
    z = torch.zeros(n, dtype=torch.float64, device="cuda")
    one = torch.ones(n, dtype=torch.float64, device="cuda")
    rc = _call(L, "nekgpu_axhelm_dev_noalloc", lib._h, z, z, one, z)
    assert rc == _capi.EINVAL
    assert "exceed" in lib.last_error()
