"""Oracle of the PN-PN splitting step (plan4, core/plan4.f:2-97): the
reference's step restated over the oracle's own routines (oracle/nekref.c and
oracle/gradops.c through nekref.py), in the reference's order.  Test
infrastructure only: the GPU path never calls it.

  plan4(1)  makef (core/navier1.f:1425-1461): makeuf (bf = f bm1, :1463),
            advab (:1516), makeabf (:1597), makebdf (:1548); sumab for the
            extrapolated velocity (core/plan4.f:45-49, :525)
  plan4(2)  lagvel (core/navier1.f:1929); bcdirvc (homogeneous walls: v =
            mask v); crespsp (core/plan4.f:99); h1 = 1/vtrans, h2 = 0;
            ctolspl (core/navier1.f:193); hsolve('PRES') with projection
            (core/navier4.f:562); pr += dpr; ortho (core/navier1.f:223);
            cresvsp (core/plan4.f:264, h1 = vdiff, h2 = vtrans bd(1)/dt from
            sethlm, core/subs1.f:1013); ophinv (core/induct.f:1022: hmholtz
            per component); v += dv
  stress    the stress formulation's branch (core/plan4.f:84-86):
            cresvsp_weak (:308) and hmhzsf (core/induct.f:1057-1061,
            core/subs1.f:1093) for the three components together

Coefficients: the same constant-step BDF / extrapolation pairs as the device
driver (setbd / setabbd, core/navier1.f:1662-1800, with setordbd's ramp).
"""
from __future__ import annotations

import numpy as np

from . import nekref

_BD = {1: [1.0, 1.0], 2: [1.5, 2.0, -0.5], 3: [11.0 / 6.0, 3.0, -1.5, 1.0 / 3.0]}
_AB = {1: [1.0, 0.0, 0.0], 2: [2.0, -1.0, 0.0], 3: [3.0, -3.0, 1.0]}


class SplittingStepOracle:
    def __init__(self, P, vmask, pmask, vtrans, vdiff, qtl, dt, tolhv=1e-10, tolpdf=1e-10,
                 order=3, null_space=True, nmxv=1000, nmxp=1000, mmx=8, convection=True,
                 tolps=1e-8, prelax=1e-3, stress=False):
        self.P = P
        self.ops = P["ops"]
        self.nx1, self.nel, self.n = P["nx1"], P["nel"], P["n"]
        self.rst, self.jac = nekref.geom_rst(self.nx1, self.nel, P["x"], P["y"], P["z"])
        self.bm1, self.binv, self.mult = P["bm1"], P["binv"], P["mult"]
        self.vmask, self.pmask = np.asarray(vmask, float), np.asarray(pmask, float)
        self.vtrans, self.vdiff, self.qtl = (np.asarray(a, float) for a in (vtrans, vdiff, qtl))
        self.dt, self.tolhv, self.tolpdf, self.order = float(dt), tolhv, tolpdf, order
        self.null_space, self.nmxv, self.nmxp = null_space, nmxv, nmxp
        self.convection, self.tolps, self.prelax = convection, tolps, prelax
        self.stress = stress
        self.proj = nekref.Projection(self.ops, mmx)
        n = self.n
        self.v = [np.zeros(n) for _ in range(3)]
        self.pr = np.zeros(n)
        self.vlag = [[np.zeros(n), np.zeros(n)] for _ in range(3)]
        self.abx1 = [np.zeros(n) for _ in range(3)]
        self.abx2 = [np.zeros(n) for _ in range(3)]
        self.volvm1 = float(np.sum(self.bm1))
        self.istep = 0

    def step(self, forcing=None):
        n, dt = self.n, self.dt
        self.istep += 1
        nbd = min(self.istep, self.order)
        bd, ab = np.array(_BD[nbd]), np.array(_AB[nbd])
        nab = nbd
        # makef
        bf = [np.zeros(n) if forcing is None else forcing[c] * self.bm1 for c in range(3)]
        if self.convection:
            bf = nekref.advab(self.nx1, self.nel, bf, self.v, self.bm1, self.rst, self.jac)
        for c in range(3):
            bf[c], self.abx1[c], self.abx2[c] = nekref.makeabf(bf[c], self.abx1[c], self.abx2[c],
                                                               self.vtrans, ab)
            bf[c] = nekref.makebdf(bf[c], self.v[c], self.vlag[c][:nbd - 1], self.bm1,
                                   self.vtrans, bd, nbd, dt)
        ve = [self.v[c].copy() if nab == 1 else
              nekref.sumab(self.v[c], self.vlag[c][:nab - 1], ab, nab) for c in range(3)]
        # lagvel, bcdirvc
        for c in range(3):
            self.vlag[c] = [self.v[c].copy(), self.vlag[c][0]]
            self.v[c] = self.v[c] * self.vmask
        dtbd = bd[0] / dt
        respr = nekref.crespsp(self.ops, ve, self.pr, self.qtl, self.vdiff, self.vtrans, bf,
                               self.bm1, self.binv, dtbd, self.null_space, self.rst, self.jac)
        rinit = np.sqrt(np.sum(respr / self.bm1 * respr) / self.volvm1)
        tolspl = self.tolpdf if self.tolpdf > 0 else max(self.tolps / dt, rinit * self.prelax)
        h1p, h2p = 1.0 / self.vtrans, np.zeros(n)
        dpr, _, itp, _, _ = self.proj.hsolve(respr, h1p, h2p, self.pmask, self.mult, self.binv,
                                             tolspl, maxit=self.nmxp, maxcg=self.nmxp)
        self.pr = self.pr + dpr
        if self.null_space:
            self.pr = self.pr - np.sum(self.pr) / n
        h1v, h2v = self.vdiff.copy(), self.vtrans * dtbd
        if self.stress:
            res = nekref.cresvsp_weak(self.ops, self.v, h1v, h2v, self.vdiff, self.qtl, self.pr,
                                      bf, self.rst, self.jac, self.bm1, stress=True)
            dv, _, it, _, _ = nekref.hmhzsf(self.ops, res, h1v, h2v, [self.vmask] * 3, self.mult,
                                            self.binv, self.rst, self.jac, self.bm1,
                                            self.volvm1, self.tolhv)
            for c in range(3):
                self.v[c] = self.v[c] + dv[c]
            return itp, [it]
        res = nekref.cresvsp(self.ops, self.v, h1v, h2v, self.vdiff, self.qtl, self.pr, bf,
                             self.rst)
        itv = []
        for c in range(3):
            dv, _, it, _, _ = self.ops.hmholtz(res[c], h1v, h2v, self.vmask, self.mult,
                                               self.binv, self.tolhv, maxit=self.nmxv,
                                               maxcg=self.nmxv)
            itv.append(it)
            self.v[c] = self.v[c] + dv
        return itp, itv
