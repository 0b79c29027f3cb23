"""The C ABI library: builds, loads without a GPU, exports every declared symbol,
and reports errors by status code (no GPU compute is called here)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for h in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if h.endswith(".h"):
            src = open(os.path.join(ROOT, "include", h)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            syms |= set(re.findall(r"\bint\s+(nek(?:gpu|mesh)_\w+)\s*\(", src))
    return sorted(syms)


@pytest.fixture(scope="module")
def lib():
    from nek5000_gb300 import _capi, build
    build.build()
    return _capi.load()


def test_header_declares_the_reference_boundary():
    syms = declared_symbols()
    for must in ("nekgpu_axhelm", "nekgpu_dssum", "nekgpu_setprec", "nekgpu_cggo", "nekgpu_hmholtz",
                 "nekgpu_setup", "nekgpu_init", "nekgpu_finalize", "nekmesh_re2_open",
                 "nekmesh_co2_read", "nekmesh_connect", "nekmesh_setvert3d"):
        assert must in syms


def test_library_exports_every_declared_symbol(lib):
    from nek5000_gb300 import _capi
    for s in declared_symbols():
        assert hasattr(lib, s), s
        assert s in _capi.SIGNATURES, f"{s} has no ctypes signature"


def test_bad_handle_is_an_error_code(lib):
    h = C.c_int64(987654)
    out = C.c_double(0)
    rc = lib.nekgpu_dssum(C.byref(h), C.c_void_p(C.addressof(out)))
    assert rc == -2  # NEKGPU_EHANDLE
    buf = C.create_string_buffer(256)
    assert lib.nekgpu_last_error(C.byref(h), buf, C.byref(C.c_int(256))) == 0
    assert b"handle" in buf.value


def test_init_without_gpu_fails_cleanly(lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    h = C.c_int64(0)
    rc = lib.nekgpu_init(C.byref(C.c_int(0)), C.byref(h))
    assert rc in (-3, -1)


def _prototypes(path):
    """name -> parameter list of every int-returning entry point of a header"""
    import re
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", " ", text, flags=re.S)
    out = {}
    for m in re.finditer(r"\bint\s+(nek(?:gpu|mesh)_\w+)\s*\(([^)]*)\)\s*;", text):
        params = [p.strip() for p in m.group(2).split(",") if p.strip() and p.strip() != "void"]
        out[m.group(1)] = params
    return out


def test_ctypes_signatures_match_the_headers():
    """Every ctypes declaration has as many arguments as the header's
    prototype, pointers where the prototype has pointers and ints/doubles
    passed by reference where it has pointers to them: a mismatch would
    hand the library wrong addresses."""
    import ctypes as C
    from nek5000_gb300 import _capi
    protos = {}
    for h in ("nekgpu.h", "nekmesh.h"):
        protos.update(_prototypes(os.path.join(ROOT, "include", h)))
    missing = [n for n in _capi.SIGNATURES if n not in protos]
    assert not missing, missing
    for name, args in _capi.SIGNATURES.items():
        params = protos[name]
        assert len(args) == len(params), (name, len(args), len(params))
        for a, p in zip(args, params):
            is_ptr = "*" in p
            ctype_is_ptr = a is C.c_void_p or a is C.c_char_p or (
                isinstance(a, type) and issubclass(a, C._Pointer))
            assert is_ptr == ctype_is_ptr, (name, p, a)


class _FakeDev:
    """Stands in for a CUDA tensor in a call that must stop at the handle
    check: the library rejects an unknown handle before it reads any array."""
    is_cuda = True
    dtype = "torch.float64"

    def is_contiguous(self):
        return True

    def data_ptr(self):
        return 0


def test_python_wrappers_reach_the_library(lib):
    """Every wrapper of the pressure preconditioner, the shard primitives and
    the splitting-step operators passes the library the argument list its
    ctypes declaration expects: called on an unknown handle each one ends
    in the library's EHANDLE status, not in a ctypes or Python error."""
    import ctypes as C
    import numpy as np
    from nek5000_gb300 import _capi
    from nek5000_gb300.solver import NekGpu
    g = NekGpu.__new__(NekGpu)
    g._L, g._h = lib, C.c_int64(987654321)
    d, h = _FakeDev(), np.zeros(8)
    gl = np.arange(8, dtype=np.int64)
    calls = [
        lambda: g.hmh_flex_cg(d, d, d, d, d, -1e-10),
        lambda: g.hmh_flex_cg(h, h, h, h, h, -1e-10),
        lambda: g.h1mg_setup(h, h, h, gl, mask=h),
        lambda: g.h1mg_free(),
        lambda: g.h1mg_apply(d, d),
        lambda: g.wgradm1(d, d, d, d),
        lambda: g.dudxyz(d, d, 1),
        lambda: g.cdtp(d, d, 2),
        lambda: g.op_curl(d, d, d, d, d, d, ifavg=True, binv=d),
        lambda: g.conv1(d, d, [d, d, d]),
        lambda: g.advab([d, d, d], [d, d, d]),
        lambda: g.dealias_setup(12),
        lambda: g.convop(d, d, [d, d, d]),
        lambda: g.convect_cons(d, d, [d, d, d]),
        lambda: g.conv2(d, d, [d, d, d]),
        lambda: g.convopo(d, d, [d, d, d], ofc=np.zeros((2, 6), dtype=np.int32)),
        lambda: g.cresvsp([d, d, d], [d, d, d], d, d, d, d, d, [d, d, d]),
        lambda: g.crespsp(d, [d, d, d], d, d, d, d, [d, d, d], d, 1.5, True, v=[d, d, d],
                          fbc=np.zeros((1, 6), dtype=np.int32)),
        lambda: g.makeabf(d, d, d, d, [1.0, 0.0, 0.0]),
        lambda: g.makebdf(d, d, d, d, [1.0, 1.0, 0.0, 0.0], 2, 0.1),
        lambda: g.sumab(d, d, d, [1.0, 0.0, 0.0], 2),
    ]
    for k, call in enumerate(calls):
        with pytest.raises(_capi.NekGpuError) as ei:
            call()
        assert ei.value.code == _capi.EHANDLE, k


def test_device_shard_calls_reach_the_library(lib):
    """The element-shard backend's library calls (shard.DeviceShard) pass
    their arguments as the declarations expect: on an unknown handle each
    ends in EHANDLE."""
    import ctypes as C
    import numpy as np
    from nek5000_gb300 import _capi
    from nek5000_gb300.shard import DeviceShard, Interface
    from nek5000_gb300.solver import NekGpu
    g = NekGpu.__new__(NekGpu)
    g._L, g._h = lib, C.c_int64(987654321)
    s = DeviceShard.__new__(DeviceShard)
    s.lib = g
    d = _FakeDev()
    calls = [
        lambda: s.dssum(d), lambda: s.axhelm(d, d, d, d), lambda: s.setprec_local(d, d, d),
        lambda: s.col2(d, d), lambda: s.col3(d, d, d), lambda: s.add2s1(d, d, 0.5),
        lambda: s.add2s2(d, d, -0.5), lambda: s.invcol1(d), lambda: s.vlsc3(d, d, d),
        lambda: s.vlsc32(d, d, d), lambda: s.vlmax(d, 0),
        lambda: s.iface_setup(Interface(np.array([1, 2, 2, 0]), [np.array([1, 2]),
                                                                  np.array([2, 3])])),
    ]
    for k, call in enumerate(calls):
        with pytest.raises(_capi.NekGpuError) as ei:
            call()
        assert ei.value.code == _capi.EHANDLE, k
