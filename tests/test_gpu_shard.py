"""The solve split over element shards on the device: two DeviceShards
(two library handles on disjoint element slabs) in one process, their
interface sums exchanged in shard order (LocalExchange; no kernel waits on
another shard's), against the oracle's cggo (core/hmholtz.f:611-846) and the
library's single-domain cggo on the same problem: iterations to +-1,
solutions to 1e-9 relative."""
import numpy as np
import pytest

from conftest import rng_unit_vector

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["dirichlet", "null"])
def test_two_device_shards_match_the_single_domain(gpu_lib, oracle, case):
    torch = pytest.importorskip("torch")
    from nek5000_gb300.shard import DeviceShard, LocalExchange, ShardedCggo, slab_partition
    if case == "dirichlet":
        P = oracle.box_problem(6, 4, 3, 2, v=rng_unit_vector(131))
    else:
        P = oracle.box_problem(5, 4, 2, 2, dirichlet=(False,) * 6, v=rng_unit_vector(132))
    n, nx1 = P["n"], P["nx1"]
    h1, h2 = np.ones(n), np.zeros(n)
    f = P["ops"].dssum(P["bm1"] * np.random.default_rng(133).standard_normal(n)) * P["mask"]
    dev = lambda a: torch.tensor(np.ascontiguousarray(a), device="cuda")
    full = gpu_lib(0)
    full.setup(nx1, P["nel"], P["D"], P["g"], P["bm1"], P["glo_num"])
    xf = torch.zeros(n, dtype=torch.float64, device="cuda")
    itf, r0f, _ = full.cggo(xf, dev(f), dev(h1), dev(h2), dev(P["mask"]), dev(P["mult"]), 1,
                            -1e-10, 10 ** 5, 1, dev(P["binv"]), maxcg=10 ** 5)[:3]
    nxyz = nx1 ** 3
    shards, idxs = [], []
    for els in slab_partition(P["x"], nx1, 2):
        idx = (els[:, None] * nxyz + np.arange(nxyz)).reshape(-1)
        lib = gpu_lib(0)
        g = np.asarray(P["g"]).reshape(6, -1)[:, idx]
        lib.setup(nx1, len(els), P["D"], g, P["bm1"][idx], P["glo_num"][idx])
        shards.append(DeviceShard(lib, P["glo_num"][idx], P["bm1"][idx]))
        idxs.append(idx)
    cg = ShardedCggo(shards, LocalExchange())
    sl = lambda a: [dev(np.asarray(a)[i]) for i in idxs]
    x, it, r0, r2 = cg.solve(sl(f), sl(h1), sl(h2), sl(P["mask"]), sl(P["mult"]),
                             sl(P["binv"]), -1e-10, 10 ** 5, maxcg=10 ** 5)
    xs = np.zeros(n)
    for i, xi in zip(idxs, x):
        xs[i] = xi.cpu().numpy()
    xh = xf.cpu().numpy()
    x_ref, it_ref, _, _ = P["ops"].cggo(f, h1, h2, P["mask"], P["mult"], P["binv"], -1e-10,
                                        maxcg=10 ** 5)
    assert abs(it - it_ref) <= 1, (it, it_ref)
    assert np.linalg.norm(xs - x_ref) <= 1e-9 * np.linalg.norm(x_ref)
    assert abs(it - itf) <= 1, (it, itf)
    assert np.linalg.norm(xs - xh) <= 1e-9 * np.linalg.norm(xh)
