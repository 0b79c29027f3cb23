"""Regenerates tests/golden/oracle_golden.npz from the oracle (serial order,
nthreads = 1).

These fixtures pin the oracle against itself over time: tests/test_oracle.py
recomputes every entry and requires bit-identical results, so a change to
the restatement that moves any output is caught.  They are not reference
outputs -- the reference Fortran cannot be built or run here -- and the
oracle stays "parity unpinned" with respect to the reference.

Contents (all FP64 unless stated):
  gll_z_<np>, gll_w_<np>, dgll_<np>      GLL nodes, weights, D for np = 2..12
  small_*                                 lx1 = 5, 2x2x3 deformed box (seed vector 21):
                                          glo_num (int64), G checksums, axhelm,
                                          dssum, setprec, cggo (x, niter, norms)
  cfg1_*                                  E = 4^3 N = 7 Poisson (the CPU-runnable
                                          configuration): hmholtz niter, norms, |u|,
                                          every 64th entry of u
  proj_*                                  hsolve with projection, 6 steps on a
                                          lx1 = 6, 2x2x2 box: niter, m, |u|

Run from the repository root:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from conftest import rng_unit_vector  # noqa: E402
from oracle import nekref  # noqa: E402


def compute():
    out = {}
    for np_ in range(2, 13):
        z, w = nekref.zwgll(np_)
        D, _ = nekref.dgll(z)
        out[f"gll_z_{np_}"], out[f"gll_w_{np_}"], out[f"dgll_{np_}"] = z, w, D
    # small deformed box
    P = nekref.box_problem(5, 2, 2, 3, v=rng_unit_vector(21))
    ops, n = P["ops"], P["n"]
    rng = np.random.default_rng(21)
    u = rng.standard_normal(n)
    h1 = np.exp(0.2 * rng.standard_normal(n))
    h2 = rng.uniform(0.0, 3.0, n)
    out["small_glo_num"] = P["glo_num"].astype(np.int64)
    out["small_g_sum"] = P["g"].reshape(6, n).sum(axis=1)
    out["small_g_sumsq"] = (P["g"].reshape(6, n) ** 2).sum(axis=1)
    out["small_bm1"] = P["bm1"]
    out["small_axhelm"] = ops.axhelm(u, h1, h2)
    out["small_dssum"] = ops.dssum(u)
    out["small_setprec"] = ops.setprec(h1, h2)
    f = ops.dssum(P["bm1"] * (ops.dssum(rng.standard_normal(n)) * P["mult"])) * P["mask"]
    x, it, r0, r2 = ops.cggo(f, h1, h2, P["mask"], P["mult"], P["binv"], -1e-10, maxcg=10 ** 6)
    out["small_cggo_x"] = x
    out["small_cggo_stats"] = np.array([it, r0, r2])
    # configuration 1: E = 4^3, N = 7 Poisson, uniform [-1, 1] per global node (seed 0)
    P1 = nekref.box_problem(8, 4, 4, 4, v=rng_unit_vector(0))
    n1 = P1["n"]
    ng = int(P1["glo_num"].max()) + 1
    fg = np.random.default_rng(0).uniform(-1.0, 1.0, ng)[P1["glo_num"]]
    rhs = P1["bm1"] * fg
    u1, _, it1, r01, r21 = P1["ops"].hmholtz(rhs, np.ones(n1), np.zeros(n1), P1["mask"],
                                             P1["mult"], P1["binv"], -1e-10, maxcg=10 ** 6)
    out["cfg1_stats"] = np.array([it1, r01, r21, np.linalg.norm(u1)])
    out["cfg1_u_sample"] = u1[::64]
    # projection sequence
    P2 = nekref.box_problem(6, 2, 2, 2, v=rng_unit_vector(22))
    n2 = P2["n"]
    proj = nekref.Projection(P2["ops"], 4)
    r2g = np.random.default_rng(22)
    f0, f1 = r2g.standard_normal(n2), r2g.standard_normal(n2)
    stats = []
    for t in range(6):
        rr = P2["bm1"] * P2["ops"].dssum((f0 + np.sin(0.4 * t) * f1) * P2["mult"])
        uu, _, itp, _, _ = proj.hsolve(rr, np.ones(n2), np.full(n2, 30.0), P2["mask"],
                                       P2["mult"], P2["binv"], 1e-10, maxcg=10 ** 6)
        stats.append([itp, proj.m, np.linalg.norm(uu)])
    out["proj_stats"] = np.array(stats)
    return out


if __name__ == "__main__":
    nekref.build()
    np.savez_compressed(os.path.join(HERE, "oracle_golden.npz"), **compute())
    print("wrote", os.path.join(HERE, "oracle_golden.npz"))
