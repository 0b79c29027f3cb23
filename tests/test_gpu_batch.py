"""Batched solves: problems of uneven order and size advanced together.

Each problem of the batch must stop at its own iteration count and return
exactly what a solve of that problem alone returns (the batched launches run
the same per-problem arithmetic), and agree with the oracle like a single
solve does.  The mixed form (both the residual-replacement and the restarted
inner PCG) must meet the FP64 tolerance per problem."""
import numpy as np
import pytest

from conftest import rank_spread, rng_unit_vector

pytestmark = pytest.mark.gpu

CASES = [  # (lx1, kx, ky, kz, periodic, h2)
    (6, 2, 3, 2, (False, False, False), 0.0),
    (8, 3, 2, 2, (False, True, True), 10.0),
    (10, 2, 2, 2, (False, False, False), 1500.0),
    (7, 3, 3, 2, (False, False, False), 0.0),  # 18 elements: a ragged block of 4
    (9, 2, 2, 2, (False, False, False), 1.0),
    (8, 2, 2, 2, (False, False, False), 0.0),  # zero right-hand side
]


@pytest.fixture(scope="module")
def problems(oracle):
    out = []
    for q, (nx1, kx, ky, kz, per, h2) in enumerate(CASES):
        P = oracle.box_problem(nx1, kx, ky, kz, periodic=per, v=rng_unit_vector(30 + q))
        n = P["n"]
        rng = np.random.default_rng(30 + q)
        f = P["ops"].dssum(P["bm1"] * (P["ops"].dssum(rng.standard_normal(n)) * P["mult"]))
        f = f * P["mask"]
        if q == len(CASES) - 1:
            f[:] = 0.0
        P["f"] = f
        P["h1v"] = np.ones(n)
        P["h2v"] = np.full(n, h2)
        out.append(P)
    return out


def _dev(torch, a):
    return torch.tensor(a, device="cuda")


def test_batch_fp64_equals_single_solves(gpu_lib, oracle, problems):
    torch = pytest.importorskip("torch")
    from nek5000_gb300 import NekGpuBatch
    B = NekGpuBatch(0)
    for P in problems:
        B.add(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    xs = [torch.zeros(P["n"], dtype=torch.float64, device="cuda") for P in problems]
    col = lambda k: [_dev(torch, P[k]) for P in problems]
    res = B.solve(xs, col("f"), col("h1v"), col("h2v"), col("mask"), col("mult"), col("binv"),
                  tin=-1e-10)
    assert res["status"] == [0] * len(problems)
    for q, P in enumerate(problems):
        lib = gpu_lib(0)
        lib.setup(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
        x1 = torch.zeros(P["n"], dtype=torch.float64, device="cuda")
        it, r0, r2, rc = lib.cggo(x1, _dev(torch, P["f"]), _dev(torch, P["h1v"]),
                                  _dev(torch, P["h2v"]), _dev(torch, P["mask"]),
                                  _dev(torch, P["mult"]), 1, -1e-10, 10 ** 6, 1,
                                  _dev(torch, P["binv"]), maxcg=10 ** 6)
        assert res["niter"][q] == it
        assert torch.equal(xs[q], x1), q
        if it:
            x_ref, it_ref, _, _ = P["ops"].cggo(P["f"], P["h1v"], P["h2v"], P["mask"], P["mult"],
                                               P["binv"], -1e-10, maxcg=10 ** 6)
            assert abs(it - it_ref) <= 1
            _, spread = rank_spread(oracle, P, lambda ops: ops.cggo(
                P["f"], P["h1v"], P["h2v"], P["mask"], P["mult"], P["binv"], -1e-10,
                maxcg=10 ** 6)[0])
            err = np.linalg.norm(x1.cpu().numpy() - x_ref) / np.linalg.norm(x_ref)
            assert err <= max(1e-12, 2 * spread), (q, err, spread)
    assert res["niter"][-1] == 0 and float(xs[-1].abs().max()) == 0.0
    # uneven orders really stop at different counts
    assert len(set(res["niter"][:-1])) > 1


@pytest.mark.parametrize("mixed", [1, 2])  # 1: residual replacement (default), 2: restarted
def test_batch_mixed_meets_fp64_tolerance(gpu_lib, oracle, problems, mixed):
    torch = pytest.importorskip("torch")
    from nek5000_gb300 import NekGpuBatch
    B = NekGpuBatch(0)
    for P in problems:
        B.add(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    xs = [torch.zeros(P["n"], dtype=torch.float64, device="cuda") for P in problems]
    col = lambda k: [_dev(torch, P[k]) for P in problems]
    res = B.solve(xs, col("f"), col("h1v"), col("h2v"), col("mask"), col("mult"), col("binv"),
                  tin=-1e-10, mixed=mixed)
    assert res["status"] == [0] * len(problems)
    for q, P in enumerate(problems[:-1]):
        x = xs[q].cpu().numpy()
        ops = P["ops"]
        w = ops.dssum(ops.axhelm(x, P["h1v"], P["h2v"])) * P["mask"]
        r = P["f"] - w
        rn = np.sqrt(np.sum(P["mult"] * P["binv"] * r * r) / np.sum(P["bm1"]))
        assert rn <= 1.05e-10 * res["rbn0"][q], (q, rn / res["rbn0"][q])
        assert 2 <= res["nouter"][q] <= (12 if mixed == 1 else 8)


def test_batch_block_sizes_give_identical_solves(problems):
    """The batched operator's block size (tuned or pinned) changes speed only."""
    torch = pytest.importorskip("torch")
    from nek5000_gb300 import NekGpuBatch
    col = lambda k: [_dev(torch, P[k]) for P in problems]
    out = {}
    for threads in (0, 128, 256):
        B = NekGpuBatch(0)
        B.set_persistent(False)  # the block size is tuned for the three-launch form
        for P in problems:
            B.add(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
        if threads:
            B.set_shape(0, threads)
        xs = [torch.zeros(P["n"], dtype=torch.float64, device="cuda") for P in problems]
        res = B.solve(xs, col("f"), col("h1v"), col("h2v"), col("mask"), col("mult"), col("binv"),
                      tin=-1e-10)
        assert res["status"] == [0] * len(problems)
        used, ms = B.shape(0)
        assert used in (128, 256)
        if threads:
            assert used == threads
        else:
            assert ms > 0  # tuned: both sizes were timed
        out[threads] = (res["niter"], [x.cpu().numpy() for x in xs])
        B.close()
    for threads in (128, 256):
        assert out[threads][0] == out[0][0]
        for a, b in zip(out[threads][1], out[0][1]):
            assert np.array_equal(a, b)


@pytest.mark.parametrize("mixed", [0, 1])
def test_persistent_launch_equals_graph_launches(gpu_lib, oracle, problems, mixed):
    """The persistent cooperative form (nekgpu_batch_set_persistent 1) and
    the graph-replayed launches (the default) run the same per-problem
    arithmetic: identical iteration counts, norms and solutions, bit for
    bit, FP64 and mixed."""
    torch = pytest.importorskip("torch")
    from nek5000_gb300 import NekGpuBatch
    col = lambda k: [_dev(torch, P[k]) for P in problems]
    out = {}
    for persistent in (True, False):
        B = NekGpuBatch(0)
        B.set_persistent(persistent)
        for P in problems:
            B.add(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
        xs = [torch.zeros(P["n"], dtype=torch.float64, device="cuda") for P in problems]
        res = B.solve(xs, col("f"), col("h1v"), col("h2v"), col("mask"), col("mult"),
                      col("binv"), tin=-1e-10, mixed=mixed)
        assert res["status"] == [0] * len(problems), B.last_error()
        out[persistent] = (res, [x.cpu().numpy() for x in xs])
        B.close()
    (ra, xa), (rb, xb) = out[True], out[False]
    assert ra["niter"] == rb["niter"] and ra["rbn2"] == rb["rbn2"]
    for a, b in zip(xa, xb):
        assert np.array_equal(a, b)


def test_batch_mixed_problem_independent_of_the_others(gpu_lib, oracle, problems):
    """Residual replacement runs per problem as soon as its FP32 PCG stops,
    while the others go on, and the launch tables drop converged problems
    now and then: a problem's solve must not depend on that schedule.  Each
    problem solved in a batch of its own gives the batched result bit for
    bit (outer steps, inner iterations, norms, x)."""
    torch = pytest.importorskip("torch")
    from nek5000_gb300 import NekGpuBatch
    col = lambda ps, k: [_dev(torch, P[k]) for P in ps]

    def run(ps):
        B = NekGpuBatch(0)
        for P in ps:
            B.add(P["nx1"], P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
        xs = [torch.zeros(P["n"], dtype=torch.float64, device="cuda") for P in ps]
        res = B.solve(xs, col(ps, "f"), col(ps, "h1v"), col(ps, "h2v"), col(ps, "mask"),
                      col(ps, "mult"), col(ps, "binv"), tin=-1e-10, mixed=1)
        B.close()
        return res, [x.cpu().numpy() for x in xs]

    res, xs = run(problems)
    assert res["status"] == [0] * len(problems)
    for q, P in enumerate(problems):
        r1, x1 = run([P])
        for key in ("status", "niter", "nouter", "rbn0", "rbn2"):
            assert r1[key][0] == res[key][q], (q, key, r1[key][0], res[key][q])
        assert np.array_equal(x1[0], xs[q]), q
