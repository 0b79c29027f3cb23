"""The solve split over element shards (nek5000_gb300/shard.py) against the
oracle's single-domain cggo: the host logic (slab partition, interface maps,
the exchange of interface sums, the global scalar sums and the restated
cggo loop) runs with shards whose local work is the oracle's (a test-side
implementation of the shard protocol), in one process (LocalExchange) and
as two gloo ranks (DistExchange).  Iteration counts must agree to +-1 and
the solution to 1e-10 relative (sums are formed shard by shard)."""
import os
import socket
import sys

import numpy as np
import pytest

from conftest import rng_unit_vector

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


class HostShard:
    """The shard protocol on the host, local work by the oracle."""

    def __init__(self, oracle, P, els):
        import torch
        self.torch = torch
        nxyz = P["nx1"] ** 3
        idx = (np.asarray(els)[:, None] * nxyz + np.arange(nxyz)).reshape(-1)
        self.idx = idx
        g = np.asarray(P["g"]).reshape(6, -1)[:, idx]
        self.glo = np.asarray(P["glo_num"])[idx]
        self.bm1 = np.asarray(P["bm1"])[idx]
        self.n = idx.size
        self.ops = oracle.Ops(P["nx1"], len(els), P["D"], g, self.bm1, self.glo)

    def zeros(self):
        return np.zeros(self.n)

    def ones(self):
        return np.ones(self.n)

    def union_zeros(self, m):
        return self.torch.zeros(m, dtype=self.torch.float64)

    def index(self, a):
        return self.torch.tensor(np.asarray(a, dtype=np.int64))

    def copy(self, dst, src):
        dst[:] = src

    def fill0(self, a):
        a[:] = 0.0

    def dssum(self, u):
        u[:] = self.ops.dssum(u)

    def axhelm(self, w, p, h1, h2):
        w[:] = self.ops.axhelm(p, h1, h2)

    def setprec_local(self, d, h1, h2):
        d[:] = self.ops.setprec_local(h1, h2)

    def col2(self, a, b):
        a *= b

    def col3(self, a, b, c):
        a[:] = b * c

    def add2s1(self, a, b, c1):
        a[:] = c1 * a + b

    def add2s2(self, a, b, c2):
        a[:] = a + c2 * b

    def invcol1(self, a):
        a[:] = 1.0 / a

    def vlsc3(self, a, b, c):
        return float(np.sum(a * b * c))

    def vlsc32(self, a, b, c):
        return float(np.sum(b * c * a * a))

    def vlmax(self, a, mode):
        return float(np.max(np.abs(a)) if mode == 0 else (np.max(a) if mode == 1 else np.min(a)))

    def iface_setup(self, f):
        self.f = f

    def iface_gather(self, u):
        return self.torch.tensor(u[self.f.pos[self.f.start[:-1]]])

    def iface_scatter(self, u, buf):
        b = np.asarray(buf)
        u[self.f.pos] = np.repeat(b, np.diff(self.f.start))


def _problem(oracle, case):
    if case == "dirichlet":
        P = oracle.box_problem(6, 4, 3, 2, v=rng_unit_vector(121))
        h2v = 0.0
    elif case == "periodic":
        P = oracle.box_problem(5, 4, 3, 3, periodic=(False, True, True), v=rng_unit_vector(122))
        h2v = 10.0
    else:  # no Dirichlet point, h2 = 0: cggo's null-space correction
        P = oracle.box_problem(5, 4, 2, 2, dirichlet=(False,) * 6, v=rng_unit_vector(123))
        h2v = 0.0
    n = P["n"]
    h1, h2 = np.ones(n), np.full(n, h2v)
    f = P["ops"].dssum(P["bm1"] * np.random.default_rng(124).standard_normal(n)) * P["mask"]
    return P, h1, h2, f


def _sharded(oracle, P, h1, h2, f, shards_els, exchange):
    from nek5000_gb300.shard import ShardedCggo
    sh = [HostShard(oracle, P, els) for els in shards_els]
    cg = ShardedCggo(sh, exchange)
    sl = lambda a: [np.asarray(a)[s.idx].copy() for s in sh]
    x, it, r0, r2 = cg.solve(sl(f), sl(h1), sl(h2), sl(P["mask"]), sl(P["mult"]), sl(P["binv"]),
                             -1e-10, 10 ** 5, maxcg=10 ** 5)
    return sh, x, it, r0, r2


@pytest.mark.parametrize("case", ["dirichlet", "periodic", "null"])
@pytest.mark.parametrize("nshards", [1, 2, 3])
def test_sharded_cggo_matches_the_single_domain(oracle, case, nshards):
    pytest.importorskip("torch")
    from nek5000_gb300.shard import LocalExchange, slab_partition
    P, h1, h2, f = _problem(oracle, case)
    xr, itr, r0r, r2r = _oracle_cggo(oracle, P, h1, h2, f)
    parts = slab_partition(P["x"], P["nx1"], nshards)
    assert sorted(np.concatenate(parts).tolist()) == list(range(P["nel"]))
    sh, x, it, r0, r2 = _sharded(oracle, P, h1, h2, f, parts, LocalExchange())
    xs = np.zeros(P["n"])
    for s, xi in zip(sh, x):
        xs[s.idx] = xi
    assert abs(it - itr) <= 1, (it, itr)
    assert abs(r0 - r0r) <= 1e-12 * r0r
    assert np.linalg.norm(xs - xr) <= 1e-10 * np.linalg.norm(xr)


def _oracle_cggo(oracle, P, h1, h2, f):
    out = P["ops"].cggo(f, h1, h2, P["mask"], P["mult"], P["binv"], -1e-10, maxit=10 ** 5,
                        maxcg=10 ** 5)
    return out


def test_interface_maps():
    """Every id shared by two shards is an interface point of both, with all
    its local copies listed; ids held by one shard are not."""
    from nek5000_gb300.shard import Interface
    a = np.array([0, 5, 7, 7, 9, 0, 11])
    b = np.array([7, 3, 11, 11, 0])
    fa, fb = Interface(a, [a, b]), Interface(b, [a, b])
    assert fa.ids.tolist() == [7, 11] and fb.ids.tolist() == [7, 11]
    assert fa.nunion == 2 and fa.slot.tolist() == [0, 1] and fb.slot.tolist() == [0, 1]
    assert fa.pos[fa.start[0]:fa.start[1]].tolist() == [2, 3]
    assert fb.pos[fb.start[1]:fb.start[2]].tolist() == [2, 3]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, case, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import nekref
    from nek5000_gb300.shard import DistExchange, slab_partition
    P, h1, h2, f = _problem(nekref, case)
    parts = slab_partition(P["x"], P["nx1"], world)
    sh, x, it, r0, r2 = _sharded(nekref, P, h1, h2, f, [parts[rank]], DistExchange())
    out.put((rank, sh[0].idx, x[0], it, r0))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("case", ["dirichlet", "null"])
def test_two_gloo_ranks(oracle, case):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    P, h1, h2, f = _problem(oracle, case)
    xr, itr, r0r, r2r = _oracle_cggo(oracle, P, h1, h2, f)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, case, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    xs = np.zeros(P["n"])
    its = set()
    for rank, idx, x, it, r0 in res:
        xs[idx] = x
        its.add(it)
    assert len(its) == 1 and abs(its.pop() - itr) <= 1
    assert np.linalg.norm(xs - xr) <= 1e-10 * np.linalg.norm(xr)
