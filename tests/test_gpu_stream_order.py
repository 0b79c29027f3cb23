"""Ordering of the device entry points with the caller's own GPU work.

The handle's stream is non-blocking, and include/nekgpu.h promises two
things for every *_dev call: its kernels start after the work the caller has
queued on the legacy default stream (torch's default stream), and the call
returns only when its own kernels have finished.  Here every input is
written by a torch copy queued behind a ~20 ms sleep kernel on the default
stream just before the call, and every output is read by torch at once after
it, with no torch.cuda.synchronize() in between.  A call that broke either
promise would read the NaN the input held before the copy, or hand torch an
output its kernels had not written yet.  The results must equal, bit for
bit, those of the same calls made with full synchronization, on a mesh of
E = 16^3 elements at N = 7 (2.1 M points), large enough that a kernel still
runs when the call would otherwise have returned.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rng_unit_vector

pytestmark = pytest.mark.gpu

SLEEP_CYCLES = 40_000_000  # ~20 ms at 2 GHz


@pytest.fixture(scope="module")
def mesh(gpu_lib, oracle):
    torch = pytest.importorskip("torch")
    P = oracle.box_problem(8, 16, 16, 16, v=rng_unit_vector(161))
    lib = gpu_lib(0)
    lib.setup_xyz(P["nx1"], P["nel"], P["D"], P["wgll"], P["x"], P["y"], P["z"], P["glo_num"])
    rng = np.random.default_rng(162)
    n = P["n"]
    host = {k: rng.standard_normal(n) for k in ("u", "v", "w", "a", "b")}
    host["h1"] = np.exp(0.3 * rng.standard_normal(n))
    host["h2"] = rng.uniform(0.0, 2.0, n)
    host["pos"] = rng.uniform(0.5, 2.0, n)
    for k in ("mask", "mult", "binv"):
        host[k] = P[k]
    dev = {k: torch.tensor(v, device="cuda") for k, v in host.items()}
    torch.cuda.synchronize()
    yield lib, P, dev
    lib.close()


def _late(torch, src):
    """A copy of src whose values land only after a sleep kernel on torch's
    default stream; until then it holds NaN."""
    dst = torch.full_like(src, float("nan"))
    torch.cuda._sleep(SLEEP_CYCLES)
    dst.copy_(src)
    return dst


def _raw(lib, name, *args):
    conv = []
    for a in args:
        if isinstance(a, float):
            conv.append(C.byref(C.c_double(a)))
        elif isinstance(a, int):
            conv.append(C.byref(C.c_int(a)))
        else:
            conv.append(C.c_void_p(a.data_ptr()))
    rc = getattr(lib._L, name)(C.byref(lib._h), *conv)
    assert rc == 0, (name, rc, lib.last_error())


# Each case: (name, inputs, number of outputs, call(lib, outs, ins)).  Outputs
# that the call also reads (in-place operands) start as copies of an input.
CASES = [
    ("axhelm", ("u", "h1", "h2"), 1,
     lambda L, o, i: L.axhelm(o[0], i[0], i[1], i[2])),
    ("axhelm_noalloc", ("u", "h1", "h2"), 1,
     lambda L, o, i: _raw(L, "nekgpu_axhelm_dev_noalloc", o[0], i[0], i[1], i[2], 1, 1)),
    ("setprec", ("h1", "h2"), 1, lambda L, o, i: L.setprec(o[0], i[0], i[1])),
    ("dssum", ("u",), ("u",), lambda L, o, i: L.dssum(o[0])),
    ("col2", ("v",), ("u",), lambda L, o, i: _raw(L, "nekgpu_col2_dev", o[0], i[0])),
    ("col3", ("u", "v"), 1, lambda L, o, i: _raw(L, "nekgpu_col3_dev", o[0], i[0], i[1])),
    ("add2s1", ("v",), ("u",), lambda L, o, i: _raw(L, "nekgpu_add2s1_dev", o[0], i[0], 0.75)),
    ("add2s2", ("v",), ("u",), lambda L, o, i: _raw(L, "nekgpu_add2s2_dev", o[0], i[0], -1.25)),
    ("invcol1", (), ("pos",), lambda L, o, i: _raw(L, "nekgpu_invcol1_dev", o[0])),
    ("setprec_local", ("h1", "h2"), 1,
     lambda L, o, i: _raw(L, "nekgpu_setprec_local_dev", o[0], i[0], i[1])),
    ("wgradm1", ("u",), 3, lambda L, o, i: L.wgradm1(o[0], o[1], o[2], i[0])),
    ("dudxyz", ("u",), 1, lambda L, o, i: L.dudxyz(o[0], i[0], 2)),
    ("cdtp", ("u",), 1, lambda L, o, i: L.cdtp(o[0], i[0], 3)),
    ("op_curl", ("u", "v", "w", "binv"), 3,
     lambda L, o, i: L.op_curl(o[0], o[1], o[2], i[0], i[1], i[2], ifavg=True, binv=i[3])),
    ("conv1", ("u", "a", "b", "w"), 1, lambda L, o, i: L.conv1(o[0], i[0], i[1:4])),
    ("advab", ("u", "v", "w"), ("a", "b", "h2"), lambda L, o, i: L.advab(o, i)),
    ("makeabf", ("u", "v", "pos"), ("a",),
     lambda L, o, i: L.makeabf(o[0], i[0], i[1], i[2], [1.5, -0.5, 0.0])),
    ("cggo", ("v", "h1", "h2", "mask", "mult", "binv"), 1,
     lambda L, o, i: L.cggo(o[0], i[0] * i[3], i[1], i[2], i[3], i[4], 1, -1e-10, 25, 1, i[5],
                            maxcg=25)),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_dev_call_orders_with_torch_default_stream(mesh, case):
    torch = pytest.importorskip("torch")
    lib, P, dev = mesh
    name, ins, outs, call = case
    n = P["n"]

    def outputs(late):
        if isinstance(outs, int):
            return [torch.zeros(n, dtype=torch.float64, device="cuda") for _ in range(outs)]
        return [_late(torch, dev[k]) if late else dev[k].clone() for k in outs]

    # reference: everything synchronized around the call
    o_ref = outputs(False)
    i_ref = [dev[k].clone() for k in ins]
    torch.cuda.synchronize()
    call(lib, o_ref, i_ref)
    torch.cuda.synchronize()
    want = [t.cpu() for t in o_ref]

    # raced: inputs and in-place outputs land late on torch's stream, outputs
    # are read by torch at once
    o = outputs(True)
    i = [_late(torch, dev[k]) for k in ins]
    call(lib, o, i)
    got = [t.cpu() for t in o]
    for g, w in zip(got, want):
        assert not torch.isnan(g).any(), name
        assert torch.equal(g, w), name
