"""Operator launch shapes and the autotuner.

Every candidate shape (kernel kind, elements per block) must give the same
solve, bit for bit: the per-point arithmetic does not depend on the block a
point lands in, and the PCG's interior partial sums are per element.  So a
tuned pick changes speed only.  The tuner itself must pick one of the
candidates and report its time.
"""
import numpy as np
import pytest

from conftest import rng_unit_vector

pytestmark = pytest.mark.gpu


def _problem(oracle, nx1, k, h2, seed):
    P = oracle.box_problem(nx1, *k, v=rng_unit_vector(seed))
    n = P["n"]
    rng = np.random.default_rng(seed)
    f = P["ops"].dssum(P["bm1"] * (P["ops"].dssum(rng.standard_normal(n)) * P["mult"])) * P["mask"]
    return P, f, np.ones(n), np.full(n, h2)


@pytest.mark.parametrize("nx1", [8, 7])
def test_fp64_shapes_give_identical_solves(gpu_lib, oracle, nx1):
    torch = pytest.importorskip("torch")
    P, f, h1, h2 = _problem(oracle, nx1, (4, 3, 3), 10.0, 21)
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    dev = lambda a: torch.tensor(a, device="cuda")
    args = [dev(a) for a in (f, h1, h2, P["mask"], P["mult"])]
    cands = lib.ax_candidates(0)
    assert len(cands) >= 2 and all(k == 0 for k, e in cands)
    sols = []
    for kind, epb in cands:
        lib.set_ax_shape(0, kind, epb)
        assert lib.ax_shape(0)[:2] == (kind, epb)
        x = torch.zeros(P["n"], dtype=torch.float64, device="cuda")
        it, r0, r2, rc = lib.cggo(x, *args, 1, -1e-10, 10 ** 6, 1, dev(P["binv"]), maxcg=10 ** 6)
        assert rc == 0
        sols.append((it, r2, x.cpu().numpy()))
    for it, r2, x in sols[1:]:
        assert it == sols[0][0] and r2 == sols[0][1]
        assert np.array_equal(x, sols[0][2])


@pytest.mark.parametrize("nx1", [8, 7, 9, 10])
def test_fp32_shapes_give_identical_inner_solves(gpu_lib, oracle, nx1):
    """27 elements at lx1 = 7, 8, 9, so that the last block of every
    multi-element shape is ragged (at odd lx1 the TMA-staged kernel's last
    block of 4 elements holds 3 and stages them with plain loads), and 20 at
    lx1 = 10 (the one-element kernel with its own register bound)."""
    torch = pytest.importorskip("torch")
    P, f, h1, h2 = _problem(oracle, nx1, (5, 2, 2) if nx1 == 10 else (3, 3, 3), 10.0, 22)
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    dev = lambda a: torch.tensor(a, device="cuda")
    args = [dev(a) for a in (f, h1, h2, P["mask"], P["mult"])]
    cands = lib.ax_candidates(1)
    kinds = {k for k, e in cands}
    assert kinds == {0, 1}  # plain loads and TMA staging (even lx1, odd lx1 <= 9)
    by_kind = {}
    for kind, epb in cands:
        lib.set_ax_shape(1, kind, epb)
        assert lib.ax_shape(1)[:2] == (kind, epb)
        x = torch.zeros(P["n"], dtype=torch.float64, device="cuda")
        no, ni, r0, r2, rc = lib.cggo_mixed(x, *args, 1, -1e-10, 10 ** 6, 1, dev(P["binv"]))
        assert rc == 0
        by_kind.setdefault(kind, []).append((ni, r2, x.cpu().numpy()))
    for kind, runs in by_kind.items():  # within a kernel kind: identical
        for ni, r2, x in runs[1:]:
            assert ni == runs[0][0] and r2 == runs[0][1]
            assert np.array_equal(x, runs[0][2])
    if len(by_kind) == 2:  # across kinds: both meet the same FP64 tolerance
        a, b = by_kind[0][0][2], by_kind[1][0][2]
        assert np.linalg.norm(a - b) <= 1e-8 * np.linalg.norm(a)


def test_autotune_picks_a_candidate(gpu_lib, oracle):
    torch = pytest.importorskip("torch")
    from nek5000_gb300 import _capi
    P, f, h1, h2 = _problem(oracle, 8, (4, 4, 4), 10.0, 23)
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    kind, epb, ms = lib.ax_shape(0)
    assert ms == 0.0  # untuned: the built-in shape
    dev = lambda a: torch.tensor(a, device="cuda")
    x = torch.zeros(P["n"], dtype=torch.float64, device="cuda")
    it, r0, r2, rc = lib.cggo(x, dev(f), dev(h1), dev(h2), dev(P["mask"]), dev(P["mult"]), 1,
                              -1e-10, 10 ** 6, 1, dev(P["binv"]), maxcg=10 ** 6)
    assert rc == 0
    kind, epb, ms = lib.ax_shape(0)  # tuned by the first solve
    assert (kind, epb) in lib.ax_candidates(0) and ms > 0
    k1, e1, ms1 = lib.autotune(1, 0, 1)  # FP32, uniform h1, uniform h2
    assert (k1, e1) in lib.ax_candidates(1) and ms1 > 0
    print(f"autotune E=64 N=7: FP64 kind {kind} epb {epb} {ms * 1e3:.1f} us; "
          f"FP32 kind {k1} epb {e1} {ms1 * 1e3:.1f} us")
    # switching tuning off returns to the built-in shape
    lib.set_option(_capi.OPT_AUTOTUNE, 0)
    assert lib.ax_shape(0)[2] == 0.0
    with pytest.raises(_capi.NekGpuError):
        lib.set_ax_shape(0, 1, 2)  # no TMA kernel in FP64


@pytest.mark.parametrize("nx1", [8, 5])
def test_fp32_boundary_group_shapes_give_identical_solves(gpu_lib, oracle, nx1):
    """The FP32 boundary-group kernel's shape (threads per block, groups per
    thread) changes speed only: group sums run in the same order, and the
    operator's rho partials are folded in fixed chunks."""
    torch = pytest.importorskip("torch")
    P, f, h1, h2 = _problem(oracle, nx1, (4, 3, 3), 10.0, 24)
    lib = gpu_lib(0)
    lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    lib.set_ax_shape(1, *lib.ax_candidates(1)[0])  # operator shape pinned: no tuning
    dev = lambda a: torch.tensor(a, device="cuda")
    args = [dev(a) for a in (f, h1, h2, P["mask"], P["mult"])]
    runs = []
    for threads in (128, 256, 512):
        for gshift in (-1, 0, 1):
            lib.set_gs_shape(threads, gshift)
            assert lib.gs_shape(1)[:2] == (threads, gshift)
            x = torch.zeros(P["n"], dtype=torch.float64, device="cuda")
            no, ni, r0, r2, rc = lib.cggo_mixed(x, *args, 1, -1e-10, 10 ** 6, 1, dev(P["binv"]))
            assert rc == 0
            runs.append((ni, r2, x.cpu().numpy()))
    for ni, r2, x in runs[1:]:
        assert ni == runs[0][0] and r2 == runs[0][1]
        assert np.array_equal(x, runs[0][2])
