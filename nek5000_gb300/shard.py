"""A Helmholtz solve split over element shards: the reference's own domain
decomposition (each MPI rank owns a set of elements; gs_op sums the copies
of shared points across ranks; gop adds the ranks' local dot products,
core/comm_mpi.f:216).

One shard = one library handle on its own elements (the global numbering
restricted to them, so the handle's dssum sums the shard's own copies).  A
global dssum is then: local dssum on every shard, gather of the interface
points (the ids that other shards also hold), a sum of the interface
buffers over all shards, scatter back.  The exchange object does the sums:

  DistExchange   -- one shard per process, torch.distributed all-reduce
                    (NCCL on GPUs, gloo on the host)
  LocalExchange  -- several shards in one process (one GPU), summed in
                    shard order; no kernel of one shard waits on another's

ShardedCggo restates cggo (core/hmholtz.f:611-846: Jacobi PCG with the
null-space correction, the tin < 0 relative tolerance and the maxcg cap) on
top of per-shard operations, so with one shard it is cggo itself and with
several it is the reference's parallel cggo.  The per-shard operations are
a small protocol (DeviceShard implements it with the library's device entry
points; a test may implement it on the host).
"""
from __future__ import annotations

import math

import numpy as np


def slab_partition(x, nx1: int, nshards: int):
    """Element lists of nshards contiguous slabs along x: elements sorted by
    the x of their centroid (ties by element number), cut into nearly equal
    counts.  x: the GLL x coordinates, nx1^3 per element."""
    xe = np.asarray(x, dtype=np.float64).reshape(-1, nx1 ** 3).mean(axis=1)
    order = np.lexsort((np.arange(xe.size), xe))
    return [np.sort(a) for a in np.array_split(order, nshards)]


class Interface:
    """Interface points of one shard: the non-zero ids of its numbering that
    at least one other shard holds.  k-th interface point = the k-th of those
    ids ascending; start/pos list its local copies (ascending positions);
    slot[k] = its place in the buffer of all shards' interface ids (the
    union, ascending), the same on every shard."""

    def __init__(self, glo_local, all_ids):
        glo = np.asarray(glo_local, dtype=np.int64).reshape(-1)
        mine = np.unique(glo[glo != 0])
        counts = {}
        for ids in all_ids:
            for v in np.unique(np.asarray(ids, dtype=np.int64)):
                if v != 0:  # element interiors (id 0) are never shared
                    counts[int(v)] = counts.get(int(v), 0) + 1
        union = np.array(sorted(v for v, c in counts.items() if c > 1), dtype=np.int64)
        self.nunion = int(union.size)
        ids = mine[np.isin(mine, union)]
        self.ids = ids
        self.nk = int(ids.size)
        self.slot = np.searchsorted(union, ids).astype(np.int64)
        order = np.argsort(glo, kind="stable")
        g = glo[order]
        lo = np.searchsorted(g, ids, side="left")
        hi = np.searchsorted(g, ids, side="right")
        self.start = np.zeros(self.nk + 1, dtype=np.int64)
        self.start[1:] = np.cumsum(hi - lo)
        self.pos = np.concatenate([np.sort(order[a:b]) for a, b in zip(lo, hi)]).astype(np.int64) \
            if self.nk else np.zeros(0, dtype=np.int64)


class LocalExchange:
    """Several shards in this process: interface buffers and scalars summed
    over the shards in shard order."""

    def all_ids(self, id_lists):
        return list(id_lists)

    def sum_interface(self, ifaces, bufs, full):
        """bufs[s]: shard s's interface values; returns the summed values per
        shard.  full: a zeroed buffer factory of the union size."""
        tot = full()
        for f, b in zip(ifaces, bufs):
            tot[f.slot] += b
        return [tot[f.slot] for f in ifaces]

    def sum_scalars(self, vals):
        t = 0.0
        for v in vals:
            t += v
        return t

    def max_scalars(self, vals):
        return max(vals)

    def min_scalars(self, vals):
        return min(vals)


class DistExchange:
    """One shard per process; sums over the process group (torch.distributed).
    Interface buffers travel as tensors of the shard's device."""

    def __init__(self, group=None):
        import torch.distributed as dist
        self.dist = dist
        self.group = group

    def all_ids(self, id_lists):
        (ids,) = id_lists
        out = [None] * self.dist.get_world_size(self.group)
        self.dist.all_gather_object(out, [int(v) for v in ids], group=self.group)
        return out

    def sum_interface(self, ifaces, bufs, full):
        (f,), (b,) = ifaces, bufs
        tot = full()
        tot[f.slot] = b
        self.dist.all_reduce(tot, group=self.group)
        return [tot[f.slot]]

    def _reduce(self, v, op):
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        if self.dist.get_backend(self.group) == "nccl":
            t = t.cuda()
        self.dist.all_reduce(t, op=op, group=self.group)
        return float(t.item())

    def sum_scalars(self, vals):
        (v,) = vals
        return self._reduce(v, self.dist.ReduceOp.SUM)

    def max_scalars(self, vals):
        (v,) = vals
        return self._reduce(v, self.dist.ReduceOp.MAX)

    def min_scalars(self, vals):
        (v,) = vals
        return self._reduce(v, self.dist.ReduceOp.MIN)


class ShardedCggo:
    """cggo (core/hmholtz.f:611-846) over shards.  shards: the shards this
    process owns (objects with the per-shard protocol: glo, dssum, axhelm,
    setprec_local, col2, col3, add2s1, add2s2, invcol1, vlsc3, vlsc32,
    vlmax, zeros, copy, iface_setup, iface_gather, iface_scatter, union_zeros,
    index); exchange: LocalExchange or DistExchange."""

    def __init__(self, shards, exchange):
        self.S = list(shards)
        self.X = exchange
        ids = [np.unique(np.asarray(s.glo)[np.asarray(s.glo) != 0]) for s in self.S]
        all_ids = self.X.all_ids(ids)
        self.iface = [Interface(s.glo, all_ids) for s in self.S]
        self.nunion = self.iface[0].nunion
        for s, f in zip(self.S, self.iface):
            s.iface_setup(f)
            f.slot_t = s.index(f.slot)

    # ---- global operations (gop / gs_op across shards)
    def gsum(self, vals):
        return self.X.sum_scalars(vals)

    def dssum(self, us):
        for s, u in zip(self.S, us):
            s.dssum(u)
        bufs = [s.iface_gather(u) for s, u in zip(self.S, us)]
        sums = self.X.sum_interface([_Slot(f) for f in self.iface], bufs,
                                    lambda: self.S[0].union_zeros(self.nunion))
        for s, u, b in zip(self.S, us, sums):
            s.iface_scatter(u, b)

    def setprec(self, h1, h2):
        """d = 1 / dssum(diag) over all shards (setprec, core/hmholtz.f:380)."""
        d = [s.zeros() for s in self.S]
        for s, di, a, b in zip(self.S, d, h1, h2):
            s.setprec_local(di, a, b)
        self.dssum(d)
        for s, di in zip(self.S, d):
            s.invcol1(di)
        return d

    def solve(self, f, h1, h2, mask, mult, binv, tin, maxit, maxcg=900, istep=0):
        """x (per shard), niter, rbn0, rbn2 -- cggo's outputs."""
        S = self.S
        ones = [s.ones() for s in S]
        vol = self.gsum([s.vlsc3(s.bm1, o, o) for s, o in zip(S, ones)])
        tol = abs(tin)
        niter = min(maxit, maxcg)
        d = self.setprec(h1, h2)
        r = [s.zeros() for s in S]
        for s, ri, fi in zip(S, r, f):
            s.copy(ri, fi)
        x = [s.zeros() for s in S]
        p = [s.zeros() for s in S]
        w = [s.zeros() for s in S]
        z = [s.zeros() for s in S]
        fmax = self.X.max_scalars([s.vlmax(fi, 0) for s, fi in zip(S, f)])
        if fmax == 0.0:
            return x, 0, 0.0, 0.0
        h2max = self.X.max_scalars([s.vlmax(b, 1) for s, b in zip(S, h2)])
        skmin = self.X.min_scalars([s.vlmax(m, 2) for s, m in zip(S, mask)])
        ifmcor = skmin > 0.0 and h2max == 0.0
        smean = 0.0
        if ifmcor:
            sb = self.gsum([s.vlsc3(s.bm1, o, o) for s, o in zip(S, ones)])
            smean = -1.0 / sb
            sr = self.gsum([s.vlsc3(ri, mi, o) for s, ri, mi, o in zip(S, r, mult, ones)])
            rmean = smean * sr
            for s, xi in zip(S, x):
                s.copy(xi, s.bm1)
            self.dssum(x)
            for s, ri, xi in zip(S, r, x):
                s.add2s2(ri, xi, rmean)
            for s, xi in zip(S, x):
                s.fill0(xi)
        rtz1, rbn0, rbn2 = 1.0, 0.0, 0.0
        it = 1
        done = False
        while it <= niter:
            for s, zi, ri, di in zip(S, z, r, d):
                s.col3(zi, ri, di)
            if ifmcor:
                sz = self.gsum([s.vlsc3(zi, s.bm1, o) for s, zi, o in zip(S, z, ones)])
                rmean = smean * sz
                for s, zi, o in zip(S, z, ones):
                    s.add2s2(zi, o, rmean)
            rtz2 = rtz1
            s1 = self.gsum([s.vlsc3(zi, ri, mi) for s, zi, ri, mi in zip(S, z, r, mult)])
            s2 = self.gsum([s.vlsc32(ri, mi, bi) for s, ri, mi, bi in zip(S, r, mult, binv)])
            rtz1 = s1
            rbn2 = math.sqrt(s2 / vol)
            if it == 1:
                rbn0 = rbn2
            if tin < 0:
                tol = abs(tin) * rbn0
            if rbn2 <= tol and (it > 1 or istep <= 5):
                done = True
                break
            beta = 0.0 if it == 1 else rtz1 / rtz2
            for s, pi, zi in zip(S, p, z):
                s.add2s1(pi, zi, beta)
            for s, wi, pi, a, b in zip(S, w, p, h1, h2):
                s.axhelm(wi, pi, a, b)
            self.dssum(w)
            for s, wi, mi in zip(S, w, mask):
                s.col2(wi, mi)
            rho = self.gsum([s.vlsc3(wi, pi, mi) for s, wi, pi, mi in zip(S, w, p, mult)])
            alpha = rtz1 / rho
            for s, xi, pi in zip(S, x, p):
                s.add2s2(xi, pi, alpha)
            for s, ri, wi in zip(S, r, w):
                s.add2s2(ri, wi, -alpha)
            it += 1
        niter = it - 1
        return x, niter, rbn0, rbn2


class _Slot:
    """the interface's buffer slots in the shard's index form"""

    def __init__(self, f):
        self.slot = f.slot_t


class DeviceShard:
    """One shard on the device: a library handle set up with the shard's
    elements (operator data and the global numbering restricted to them),
    driven through the device entry points of nekgpu.h."""

    def __init__(self, lib, glo, bm1):
        import torch
        self.torch = torch
        self.lib = lib
        self.glo = np.asarray(glo, dtype=np.int64).reshape(-1)
        self.n = self.glo.size
        self.dev = torch.device("cuda", torch.cuda.current_device())
        self.bm1 = torch.tensor(np.asarray(bm1, dtype=np.float64).reshape(-1), device=self.dev)

    # ---- plumbing
    def _c(self, fn, *args):
        import ctypes as C
        from .solver import _ptr
        conv = [C.byref(C.c_double(a)) if isinstance(a, float) else
                (C.byref(a) if isinstance(a, (C.c_double, C.c_int)) else _ptr(a)) for a in args]
        self.lib._check(getattr(self.lib._L, fn)(C.byref(self.lib._h), *conv))

    def zeros(self):
        return self.torch.zeros(self.n, dtype=self.torch.float64, device=self.dev)

    def ones(self):
        return self.torch.ones(self.n, dtype=self.torch.float64, device=self.dev)

    def union_zeros(self, m):
        return self.torch.zeros(m, dtype=self.torch.float64, device=self.dev)

    def index(self, a):
        return self.torch.tensor(np.asarray(a, dtype=np.int64), device=self.dev)

    def copy(self, dst, src):
        dst.copy_(src)

    def fill0(self, a):
        a.zero_()

    # ---- the library's local operations
    def dssum(self, u):
        self._c("nekgpu_dssum_dev", u)

    def axhelm(self, w, p, h1, h2):
        import ctypes as C
        self._c("nekgpu_axhelm_dev", w, p, h1, h2, C.c_int(1), C.c_int(1))

    def setprec_local(self, d, h1, h2):
        self._c("nekgpu_setprec_local_dev", d, h1, h2)

    def col2(self, a, b):
        self._c("nekgpu_col2_dev", a, b)

    def col3(self, a, b, c):
        self._c("nekgpu_col3_dev", a, b, c)

    def add2s1(self, a, b, c1):
        self._c("nekgpu_add2s1_dev", a, b, float(c1))

    def add2s2(self, a, b, c2):
        self._c("nekgpu_add2s2_dev", a, b, float(c2))

    def invcol1(self, a):
        self._c("nekgpu_invcol1_dev", a)

    def vlsc3(self, a, b, c):
        import ctypes as C
        out = C.c_double(0.0)
        self._c("nekgpu_vlsc3_dev", a, b, c, out)
        return out.value

    def vlsc32(self, a, b, c):
        import ctypes as C
        out = C.c_double(0.0)
        self._c("nekgpu_vlsc32_dev", a, b, c, out)
        return out.value

    def vlmax(self, a, mode):
        import ctypes as C
        out = C.c_double(0.0)
        self._c("nekgpu_vlmax_dev", a, C.c_int(mode), out)
        return out.value

    def iface_setup(self, f):
        import ctypes as C
        nk = C.c_int64(f.nk)
        start = np.ascontiguousarray(f.start, dtype=np.int64)
        pos = np.ascontiguousarray(f.pos, dtype=np.int64)
        self.lib._check(self.lib._L.nekgpu_iface_setup(
            C.byref(self.lib._h), C.byref(nk), C.c_void_p(start.ctypes.data),
            C.c_void_p(pos.ctypes.data) if pos.size else None))
        self._nk = f.nk

    def iface_gather(self, u):
        buf = self.torch.zeros(max(self._nk, 1), dtype=self.torch.float64, device=self.dev)
        self._c("nekgpu_iface_gather_dev", buf, u)
        return buf[:self._nk]

    def iface_scatter(self, u, buf):
        b = buf.contiguous()
        if self._nk:
            self._c("nekgpu_iface_scatter_dev", u, b)
