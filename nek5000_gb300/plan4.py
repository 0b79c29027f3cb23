"""The PN-PN splitting step (plan4, core/plan4.f:2-97) on the device.

One time step strings the library's device entry points together in the
reference's order, each a call through the C ABI on device arrays:

  plan4(igeom=1)  makef (core/navier1.f:1425): makeuf (bf = bm1 f), advab
                  (bf -= bm1 (v.grad) v), makeabf, makebdf; sumab for the
                  extrapolated velocity v_e (core/plan4.f:45-49)
  plan4(igeom=2)  lagvel; bcdirvc (v = mask v); crespsp; h1 = 1/vtrans,
                  h2 = 0; ctolspl; hsolve('PRES') with projection; pr += dpr;
                  ortho(pr); cresvsp; ophinv (one hmholtz per component,
                  core/induct.f:1063-1073); v += dv
  stress=True     the stress formulation's branch (core/plan4.f:84-86):
                  cresvsp_weak, then ophinv's coupled hmhzsf
                  (core/induct.f:1057-1061); walls need no bcneutr terms

The coefficients of the BDF/extrapolation pair follow setbd / setabbd
(core/navier1.f:1662, :1735) for a constant time step, ramping the order up
over the first steps as setordbd does.  Velocity walls are homogeneous
Dirichlet (bcdirvc then multiplies by the mask); the pressure is the
all-Neumann one of a closed box when `null_space` (ortho removes its mean and
the pressure solve applies cggo's null-space correction).  Not covered:
traction boundaries of the stress formulation (bcneutr), moving geometry,
variable density and characteristics (the `ifchar` branches of makef).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

# BDF (bd, nbd + 1 values) and matching extrapolation (ab, 3 values, setab3)
# coefficients for a constant time step: what setbd / setabbd give for
# dtlag(k) = dt.
_BD = {1: [1.0, 1.0], 2: [1.5, 2.0, -0.5], 3: [11.0 / 6.0, 3.0, -1.5, 1.0 / 3.0]}
_AB = {1: [1.0, 0.0, 0.0], 2: [2.0, -1.0, 0.0], 3: [3.0, -3.0, 1.0]}


def coefficients(istep: int, order: int = 3):
    """(nbd, bd, ab) of time step istep (1-based): the order ramps up as
    min(istep, order) (setordbd, core/navier1.f:2002)."""
    nbd = min(istep, order)
    return nbd, list(_BD[nbd]), list(_AB[nbd])


class SplittingStep:
    """The state and one-step driver of the splitting scheme on one handle
    (NekGpu set up from coordinates: the gradient operators need the metric
    terms).  Arrays are torch float64 CUDA tensors of n points; v and pr are
    the solution, updated in place by step()."""

    def __init__(self, lib, bm1, binvm1, vmask, pmask, vmult, vtrans, vdiff, qtl, dt,
                 tolhv=1e-10, tolpdf=1e-10, order=3, null_space=True, nmxv=1000,
                 nmxp=1000, proj_space=0, mmx=8, convection=True, tolps=1e-8, prelax=1e-3,
                 stress=False):
        import torch
        self.torch, self.lib = torch, lib
        t = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64),
                                      device="cuda").clone()
        self.bm1, self.binvm1 = t(bm1), t(binvm1)
        self.vmask, self.pmask, self.vmult = t(vmask), t(pmask), t(vmult)
        self.vtrans, self.vdiff, self.qtl = t(vtrans), t(vdiff), t(qtl)
        self.n = self.bm1.numel()
        self.dt, self.tolhv, self.tolpdf, self.order = float(dt), tolhv, tolpdf, order
        self.null_space, self.nmxv, self.nmxp = null_space, nmxv, nmxp
        self.space, self.convection, self.stress = proj_space, convection, stress
        self.tolps, self.prelax = tolps, prelax  # param(21) and 0.1 tolrel (drive2.f:238)
        z = lambda: torch.zeros(self.n, dtype=torch.float64, device="cuda")
        self.ones = z() + 1.0
        # 1/bm1 (ctolspl's invcol3) and h1 = 1/vtrans of the pressure solve
        self.ibm1 = self.bm1.clone()
        self._c("nekgpu_invcol1_dev", self.ibm1)
        self.h1p = self.vtrans.clone()
        self._c("nekgpu_invcol1_dev", self.h1p)
        self.h2p = z()
        self.volvm1 = self._glsum(self.bm1)
        self.v = [z() for _ in range(3)]
        self.pr = z()
        self.vlag = [torch.zeros(2 * self.n, dtype=torch.float64, device="cuda")
                     for _ in range(3)]
        self.abx1 = [z() for _ in range(3)]
        self.abx2 = [z() for _ in range(3)]
        self.bf = [z() for _ in range(3)]
        self.ve = [z() for _ in range(3)]
        self.res = [z() for _ in range(3)]
        self.dv = [z() for _ in range(3)]
        self.respr, self.dpr = z(), z()
        self.h1v, self.h2v = z(), z()
        self.istep = 0
        self.stats = []
        lib.proj_setup(proj_space, mmx)

    # ---- plumbing: one library call per vector operation
    def _c(self, fn, *args):
        conv = []
        for a in args:
            if isinstance(a, float):
                conv.append(C.byref(C.c_double(a)))
            elif isinstance(a, int):
                conv.append(C.byref(C.c_int(a)))
            else:
                conv.append(C.c_void_p(a.data_ptr()))
        self.lib._check(getattr(self.lib._L, fn)(C.byref(self.lib._h), *conv))

    def _glsum(self, a):
        out = C.c_double(0.0)
        self.lib._check(self.lib._L.nekgpu_vlsc3_dev(C.byref(self.lib._h),
                                                     C.c_void_p(a.data_ptr()),
                                                     C.c_void_p(self.ones.data_ptr()),
                                                     C.c_void_p(self.ones.data_ptr()),
                                                     C.byref(out)))
        return out.value

    def set_velocity(self, vx, vy, vz):
        for c, a in enumerate((vx, vy, vz)):
            self.v[c].copy_(self.torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64),
                                                 device="cuda"))

    # ---- one time step
    def step(self, forcing=None):
        """Advance one step.  forcing: None or 3 device arrays of the user
        force per unit mass (makeuf multiplies by bm1).  Returns the
        iteration counts of the pressure and the three velocity solves."""
        lib, n = self.lib, self.n
        self.istep += 1
        nbd, bd, ab = coefficients(self.istep, self.order)
        nab = nbd
        dt = self.dt
        # plan4(igeom = 1): makef
        for c in range(3):  # makeuf: bf = f bm1
            if forcing is None:
                self.bf[c].zero_()
            else:
                self.bf[c].copy_(forcing[c])
                self._c("nekgpu_col2_dev", self.bf[c], self.bm1)
        if self.convection:
            lib.advab(self.bf, self.v)
        for c in range(3):
            lib.makeabf(self.bf[c], self.abx1[c], self.abx2[c], self.vtrans, ab)
            lib.makebdf(self.bf[c], self.v[c], self.vlag[c], self.vtrans, bd, nbd, dt)
        for c in range(3):  # extrapolated velocity
            if nab == 1:
                self.ve[c].copy_(self.v[c])
            else:
                lib.sumab(self.ve[c], self.v[c], self.vlag[c], ab, nab)
        # plan4(igeom = 2)
        for c in range(3):  # lagvel
            self.vlag[c][n:].copy_(self.vlag[c][:n])
            self.vlag[c][:n].copy_(self.v[c])
            self._c("nekgpu_col2_dev", self.v[c], self.vmask)  # bcdirvc, walls
        dtbd = bd[0] / dt
        lib.crespsp(self.respr, self.ve, self.pr, self.qtl, self.vdiff, self.vtrans, self.bf,
                    self.binvm1, dtbd, null_space=self.null_space)
        # ctolspl (core/navier1.f:193)
        w = self.respr.clone()
        self._c("nekgpu_col2_dev", w, self.ibm1)
        rinit = np.sqrt(self._vdot(w, self.respr) / self.volvm1)
        # tolpdf > 0: that tolerance; else tolps / dt, relaxed to rinit prelax
        tolspl = self.tolpdf if self.tolpdf > 0 else max(self.tolps / dt, rinit * self.prelax)
        itp = lib.hsolve("PRES", self.dpr, self.respr, self.h1p, self.h2p, self.pmask,
                         self.vmult, 1, tolspl, self.nmxp, 1, self.binvm1, space=self.space,
                         maxcg=self.nmxp)[0]
        self._c("nekgpu_add2s2_dev", self.pr, self.dpr, 1.0)
        if self.null_space:  # ortho (core/navier1.f:223)
            rlam = self._glsum(self.pr) / n
            self._c("nekgpu_add2s2_dev", self.pr, self.ones, -rlam)
        # cresvsp: sethlm(h1, h2, -1) -> h1 = vdiff, h2 = vtrans bd(1) / dt
        self.h1v.copy_(self.vdiff)
        self.h2v.zero_()
        self._c("nekgpu_add2s2_dev", self.h2v, self.vtrans, dtbd)
        itv = []
        if self.stress:  # cresvsp_weak; ophinv -> hmhzsf, the components coupled
            lib.cresvsp_weak(self.res, self.v, self.h1v, self.h2v, self.vdiff, self.qtl, self.pr,
                             self.bf, stress=True)
            it = lib.hmhzsf(self.dv, self.res, self.h1v, self.h2v, [self.vmask] * 3, self.vmult,
                            self.binvm1, self.tolhv)[0]
            for c in range(3):
                self._c("nekgpu_add2s2_dev", self.v[c], self.dv[c], 1.0)
            self.stats.append((itp, [it]))
            return itp, [it]
        lib.cresvsp(self.res, self.v, self.h1v, self.h2v, self.vdiff, self.qtl, self.pr, self.bf)
        for c in range(3):  # ophinv: hmholtz per component
            itv.append(lib.hmholtz("VEL", self.dv[c], self.res[c], self.h1v, self.h2v,
                                   self.vmask, self.vmult, 1, self.tolhv, self.nmxv, c + 1,
                                   self.binvm1, maxcg=self.nmxv)[0])
            self._c("nekgpu_add2s2_dev", self.v[c], self.dv[c], 1.0)
        self.stats.append((itp, itv))
        return itp, itv

    def _vdot(self, a, b):
        out = C.c_double(0.0)
        self.lib._check(self.lib._L.nekgpu_vlsc3_dev(C.byref(self.lib._h),
                                                     C.c_void_p(a.data_ptr()),
                                                     C.c_void_p(b.data_ptr()),
                                                     C.c_void_p(self.ones.data_ptr()),
                                                     C.byref(out)))
        return out.value
