"""Oracle of the algebraic multigrid coarse solve: the reference's V-cycle
amg_exec (core/crs_amg.c:129-186) and crs_solve's null-space step (:186-203),
restated with numpy / scipy.sparse on a hierarchy given as arrays.  Test
infrastructure only: the GPU path never calls it.

A hierarchy is a list of levels, level l holding its F points at
[off[l], off[l+1]) of the plan's order; each level a dict with nf, nc, m
(Chebyshev steps), rho, dff (nf) and the scipy CSR matrices W (nf x nc),
WT (nc x nf), AFP (nf x nc: Aff W + A_FC, the F rows of A P, P = [W; I]) and
AFF (nf x nf).  The last level has one unknown.
"""
from __future__ import annotations

import numpy as np


def amg_exec(levels, off, b):
    """One V-cycle; b in the plan's order (copied, not modified).  Returns x."""
    b = np.array(b, dtype=np.float64, copy=True)
    x = np.zeros_like(b)
    nl = len(levels)
    for lvl in range(nl - 1):  # restrict down all levels: b_{l+1} += W^T b_l
        L = levels[lvl]
        bl = b[off[lvl]:off[lvl + 1]]
        b[off[lvl + 1]:] += L["WT"] @ bl
    i = off[nl - 1]  # bottom equation (1 dof)
    if off[nl] - i:
        x[i] = levels[nl - 1]["dff"][0] * b[i]
    for lvl in range(nl - 2, -1, -1):
        L = levels[lvl]
        s, e = off[lvl], off[lvl + 1]
        bl = b[s:e]
        xc = x[e:]
        d = L["dff"]
        m = L["m"]
        x[s:e] = L["W"] @ xc                   # x_l = W x_{l+1}
        bl -= L["AFP"] @ xc                    # b_l -= AfP x_{l+1}
        c = d * bl                             # c_1 = Dff b_l
        c_old = np.zeros_like(c)
        alpha = beta = gamma = 0.0
        if m > 1:
            alpha = (L["rho"] / 2.0) ** 2
            gamma = 2.0 * alpha / (1.0 - 2.0 * alpha)
            beta = 1.0 + gamma
            r = bl - L["AFF"] @ c              # r_1 = b_l - Aff c_1
            c, c_old = c_old, c
            c = beta * (c_old + d * r)         # c_2 = (1+gamma)(c_1 + Dff r_1)
        for _ci in range(3, m + 1):
            gamma = alpha * beta
            gamma = gamma / (1.0 - gamma)
            beta = 1.0 + gamma
            r = bl - L["AFF"] @ c              # r_i = b_l - Aff c_i
            c, c_old = c_old, c
            c = beta * (c_old + d * r) - gamma * c  # c_{i+1}
        x[s:e] += c
    return x


def crs_solve(levels, off, perm, v, n, null_space):
    """crs_amg_solve on the unknowns' order: v has n values; with the null
    space the last unknown is left out of the cycle (pinned to 0) and the
    mean of the result removed."""
    m = n - 1 if null_space else n
    b = np.asarray(v, dtype=np.float64)[np.asarray(perm[:m])]
    xp = amg_exec(levels, off, b)
    x = np.zeros(n)
    x[np.asarray(perm[:m])] = xp
    if null_space:
        x[n - 1] = 0.0
        x -= np.sum(x) / n
    return x
