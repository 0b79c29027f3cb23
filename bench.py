#!/usr/bin/env python
"""Benchmark of the Helmholtz Jacobi-PCG solve path on one GB300 (or N replicas).

Workload (the Helmholtz configuration on one GPU): a 32x32x32 = 32768-element
deformed box, N = 7 (lx1 = 8, 16.8 M element-local points), deformation
x -> x + 0.05 sin(pi x) sin(pi y) sin(pi z) v with a unit vector v from seed 1,
Dirichlet on the x faces and periodic in y and z, h1 = 1, h2 = 10, right-hand
side B f with f standard normal per global node (seed 1), Jacobi-PCG to a
relative residual of 1e-10 (the reference's cggo norm and stopping rule, the
900-iteration cap lifted).

A step is one complete solve.  `value` is the mixed-precision solve (FP32
inner Jacobi-PCG in FP64 defect correction) as time-to-solution
DOF-iterations/s: n * (iteration count of the plain FP64 solve) / mixed solve
time, over the K timed steps, every input resident in HBM (device entry
points).  The plain FP64 solve (nekgpu_cggo_dev) is reported beside it under
"fp64".  `e2e` is the same metric through the host entry point
nekgpu_hmholtz_mixed: rhs, h1, h2, mask, mult and binv copied in from pinned
host memory and u, rhs copied out inside each timed call.

--impl reference times the CPU restatement of the reference (the oracle, all
host threads) on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DOF-iters/s, E=32^3 N=7 PCG to 1e-10: mixed vs FP64; axhelm HBM GB/s"
FALLBACK_HBM_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--k", type=int, default=32, help="elements per direction")
    ap.add_argument("--N", type=int, default=7, help="polynomial order")
    ap.add_argument("--tol", type=float, default=1e-10)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--split", action="store_true",
                    help="mixed solve: FP32 vectors in the assembled-boundary layout "
                         "(NEKGPU_OPT_SPLIT 1) instead of element-local ones")
    ap.add_argument("--no-df", action="store_true",
                    help="skip the FP64 solve with the double-float operator")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the oracle's full solve (the FP64 and mixed solutions' error "
                         "against the CPU restatement of the reference at the bench's size)")
    ap.add_argument("--cpu-iters", type=int, default=0, help="oracle PCG iterations per sample")
    ap.add_argument("--inner-tol", type=float, default=None,
                    help="mixed: inner FP32 tolerance (default: the library's for the mode)")
    ap.add_argument("--only-mixed", action="store_true", help="skip the plain FP64 solve")
    ap.add_argument("--mixed-mode", type=int, default=1, choices=[0, 1],
                    help="mixed: 1 residual replacement keeping the search direction, "
                         "0 restarted FP32 PCG per outer step")
    ap.add_argument("--workload", default="helmholtz",
                    choices=["helmholtz", "poisson-n9", "batch", "axhelm-sweep", "hsolve",
                             "adjoint", "velocity3", "ingest", "pressure"],
                    help="helmholtz: E=32^3 N=7 (default); poisson-n9: E=24^3 N=9 Poisson; "
                         "batch: 3 velocity solves + 61 uneven Poisson problems in one batch; "
                         "axhelm-sweep: in-solve operator bandwidth at N=5..9, E=32^3; "
                         "hsolve: a sequence of solves with projection onto previous solutions; "
                         "adjoint: dJ/dh1 through the adjoint solve, E=16^3 N=7; "
                         "velocity3: 3 velocity components in one fused mixed solve; "
                         "ingest: .re2 mesh ingestion on the host; "
                         "pressure: the pressure solve's GMRES")
    ap.add_argument("--batch-problems", type=int, default=61)
    ap.add_argument("--persistent-batch", action="store_true",
                    help="batch: one persistent cooperative launch per segment instead of "
                         "three graph-replayed launches per iteration")
    ap.add_argument("--fp64-shape", default=None,
                    help="pin the FP64 operator launch shape 'kind,epb' instead of autotuning")
    ap.add_argument("--gs-shape", default=None,
                    help="pin the FP32 boundary-group kernel shape 'threads,gshift'")
    ap.add_argument("--fp32-shape", default=None,
                    help="pin the FP32 operator launch shape 'kind,epb' instead of autotuning "
                         "(kind 0 plain, 1 TMA; see nekgpu_ax_candidates)")
    args = ap.parse_args()
    if args.workload == "poisson-n9":
        if args.k == 32:
            args.k = 24
        if args.N == 7:
            args.N = 9
    if args.workload == "pressure" and args.k == 32:
        args.k = 16  # restarted GMRES needs several times cggo's iterations
    if args.inner_tol is None:  # the library's defaults for the mode
        args.inner_tol = 1e-2 if args.mixed_mode == 1 else 1e-5
    return args


def workload(k, N, kind="helmholtz", keep_xyz=False):
    """helmholtz: deformed box (seed 1), Dirichlet on the x-faces, periodic in
    y and z, h1 = 1, h2 = 10, standard-normal right-hand side per global node.
    poisson: deformed box (seed 0), Dirichlet on every face, h1 = 1, h2 = 0,
    uniform [-1, 1] right-hand side per global node (seed 0).  Both
    mass-weighted: rhs = bm1 * f."""
    from nek5000_gb300 import mesh
    if kind == "poisson":
        M = mesh.box_mesh(N, k, k, k, seed=0)
        rng = np.random.default_rng(0)
        nglob = int(M["lattice"].max()) + 1
        f = rng.uniform(-1.0, 1.0, nglob)[M["lattice"]]
        h2 = 0.0
    else:
        M = mesh.box_mesh(N, k, k, k, periodic=(False, True, True),
                          dirichlet=(True, True, False, False, False, False), seed=1)
        rng = np.random.default_rng(1)
        nglob = int(M["lattice"].max()) + 1
        f = rng.standard_normal(nglob)[M["lattice"]]
        h2 = 10.0
    M["rhs"] = M["bm1"] * f
    # assembled, masked right-hand side (what hmholtz hands to cggo)
    M["f"] = mesh.dssum_host(M["lattice"], M["rhs"], nglob) * M["mask"]
    M["h1"] = np.ones(M["n"])
    M["h2"] = np.full(M["n"], h2)
    if not keep_xyz:
        for c in ("x", "y", "z"):
            M.pop(c, None)
    return M


def workload_name(args):
    if args.workload == "poisson-n9":
        return f"poisson E={args.k}^3 N={args.N} h1=1 h2=0 dirichlet-all"
    return f"helmholtz E={args.k}^3 N={args.N} h1=1 h2=10 dirichlet-x periodic-yz"


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "of measured"
    except Exception:
        return FALLBACK_HBM_GBS, "of fallback"


def ncu_summary(kernel_key):
    """Figures from the committed ncu capture of a kernel (profiles/ncu_summary.json)."""
    p = os.path.join(ROOT, "profiles", "ncu_summary.json")
    try:
        return json.load(open(p)).get(kernel_key)
    except Exception:
        return None


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None
        self.out = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.out.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.out:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(n_gpus):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        pg = dist
    return ws, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allmax(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([float(v)])
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def allsum(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([float(v)])
    pg.all_reduce(t)
    return float(t.item())


# ---------------------------------------------------------------------------
def cpu_model():
    """The host CPU's model name as lscpu reports it (aarch64 hosts have no
    'model name' line in /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.strip().lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    import platform
    return platform.processor() or platform.machine()


def cpu_sample(M, nthreads, iters):
    """Oracle (CPU restatement of the reference) PCG iterations on the full problem."""
    from oracle import nekref
    ops = nekref.Ops(M["lx1"], M["nel"], M["D"], M["g"], M["bm1"], M["glo_num"], nthreads)
    t0 = time.perf_counter()
    x, it, r0, r2 = ops.cggo(M["f"], M["h1"], M["h2"], M["mask"], M["mult"], M["binv"], -1e-30,
                             maxcg=iters)
    dt = time.perf_counter() - t0
    return M["n"] * it / dt, it, dt


def run_reference(args):
    ws, rank, local, pg = dist_setup(args.gpus)
    if rank != 0:
        return
    M = workload(args.k, args.N, "poisson" if args.workload == "poisson-n9" else "helmholtz")
    nth = os.cpu_count() or 1
    iters = args.cpu_iters or 100
    for _ in range(args.warmup):
        cpu_sample(M, nth, max(2, iters // 10))
    vals, times = [], []
    for _ in range(args.steps):
        v, it, dt = cpu_sample(M, nth, iters)
        vals.append(v)
        times.append(dt)
    value = M["n"] * iters * len(times) / sum(times)
    sample = (f"{iters} Jacobi-PCG iterations (cggo restated in C, FP64) on the full "
              f"E={args.k}^3 N={args.N} problem per step")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "DOF-iters/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": workload_name(args), "n_points": M["n"]},
            "cpu_baseline": {"value": value, "unit": "DOF-iters/s", "cores": nth, "kind": "port",
                             "sample": sample},
            "e2e": {"value": value, "unit": "DOF-iters/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def boundary_nodes(glo_num, lx1):
    """Global nodes on element boundaries: the distinct ids of the
    element-boundary points (the boundary groups of the gather-scatter)."""
    g = np.asarray(glo_num).reshape(-1, lx1, lx1, lx1)
    inner = np.zeros((lx1, lx1, lx1), dtype=bool)
    inner[1:-1, 1:-1, 1:-1] = True
    return int(np.unique(g[:, ~inner]).size)


def oracle_parity(M, x64, xmx, it64, tol, nthreads, xdf=None):
    """The oracle's own FP64 Jacobi-PCG on the same full problem, to the same
    relative tolerance: its iteration count and the relative 2-norm error of
    the GPU's FP64 and mixed solutions against its solution.  The oracle sums
    its dot products over `nthreads` element ranges, as that many ranks of
    the reference would."""
    from oracle import nekref
    ops = nekref.Ops(M["lx1"], M["nel"], M["D"], M["g"], M["bm1"], M["glo_num"], nthreads)
    t0 = time.perf_counter()
    xr, it, r0, r2 = ops.cggo(M["f"], M["h1"], M["h2"], M["mask"], M["mult"], M["binv"], -tol,
                              maxcg=10 ** 6)
    dt = time.perf_counter() - t0
    nr = float(np.linalg.norm(xr))
    return {"oracle_iterations": int(it), "fp64_iterations": int(it64),
            "rel_error_fp64_vs_oracle": float(np.linalg.norm(x64 - xr)) / nr,
            "rel_error_mixed_vs_oracle": float(np.linalg.norm(xmx - xr)) / nr,
            "rel_error_fp64_df_vs_oracle": (None if xdf is None
                                            else float(np.linalg.norm(xdf - xr)) / nr),
            "oracle_rbn2_over_rbn0": r2 / r0 if r0 else None,
            "oracle_threads": nthreads, "oracle_seconds": dt,
            "note": "oracle = C restatement of cggo (core/hmholtz.f:611-846), FP64, "
                    "summation over element ranges as that many ranks would"}


def run_gpu(args):
    import torch
    ws, rank, local, pg = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    from nek5000_gb300 import NekGpu
    from nek5000_gb300 import build as nb
    nb.build()
    M = workload(args.k, args.N, "poisson" if args.workload == "poisson-n9" else "helmholtz")
    n = M["n"]
    lib = NekGpu(local)
    lib.setup(M["lx1"], M["nel"], M["D"], M["g"], M["bm1"], M["glo_num"])
    dev = lambda a: torch.tensor(a, device=f"cuda:{local}")
    f, h1, h2 = dev(M["f"]), dev(M["h1"]), dev(M["h2"])
    mask, mult, binv = dev(M["mask"]), dev(M["mult"]), dev(M["binv"])
    x = torch.zeros(n, dtype=torch.float64, device=f"cuda:{local}")
    big = 10 ** 6
    lib.set_option(7, args.mixed_mode)
    lib.set_option(9, 1 if args.split else 0)
    for prec, spec in ((0, args.fp64_shape), (1, args.fp32_shape)):
        if spec:
            kind, epb = (int(v) for v in spec.split(","))
            lib.set_ax_shape(prec, kind, epb)
    if args.gs_shape:
        threads, gshift = (int(v) for v in args.gs_shape.split(","))
        lib.set_gs_shape(threads, gshift)

    def fp64():
        it, r0, r2, rc = lib.cggo(x, f, h1, h2, mask, mult, 1, -args.tol, big, 1, binv, maxcg=big)
        return it, rc

    def mixed():
        no, ni, r0, r2, rc = lib.cggo_mixed(x, f, h1, h2, mask, mult, 1, -args.tol, big, 1, binv,
                                            inner_tol=args.inner_tol)
        return (no, ni), rc

    def timed(solve):
        """Warm-up, then the timed steps with the library's per-kernel timing
        off (the PCG chunks replay as CUDA graphs): CUDA events on the calling
        stream around each call (every call waits for that stream's earlier
        work and returns with its own finished).  Then two more solves outside
        the timed region with per-kernel timing on (direct launches bracketed
        by events) for the kernel breakdown."""
        lib.set_option(2, 0)
        for _ in range(args.warmup):
            solve()
        barrier(pg)
        torch.cuda.synchronize()
        l0 = lib.launch_count()
        its, ms_tot = [], 0.0
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        with Clocks(local) as ck:
            for q in range(args.steps):
                ev[q][0].record()
                it, rc = solve()
                ev[q][1].record()
                if rc != 0:
                    raise RuntimeError(f"solve did not converge: {lib.last_error()}")
                its.append(it)
            torch.cuda.synchronize()
        launches = lib.launch_count() - l0
        ms_tot = sum(a.elapsed_time(b) for a, b in ev)
        barrier(pg)
        lib.set_option(2, 1)  # breakdown runs (not timed)
        ms_ax = ms_gs = ms_up = 0.0
        n_ax = 0
        for _ in range(2):
            solve()
            _, t_ax, k_ax = lib.last_timing()
            _, t_gs, t_up, _ = lib.last_kernel_times()
            ms_ax += t_ax
            n_ax += k_ax
            ms_gs += t_gs
            ms_up += t_up
        lib.set_option(2, 0)
        k = max(n_ax, 1)
        return dict(iters=its, T=allmax(pg, ms_tot / 1e3), ms_ax=ms_ax / k, n_ax=n_ax,
                    per_iter_ms={"operator": ms_ax / k, "boundary_groups": ms_gs / k,
                                 "update": ms_up / k},
                    launches=launches, clocks=ck.summary())

    peak, peak_src = peaks()
    flops_pt = 12 * M["lx1"] + 25
    # ---- end to end through the host entry points ---------------------------------
    # Each solver is timed on device arrays and then, right after, through its
    # host entry point (pinned host arrays, the copies inside the timed region):
    # the mixed solve first, then the FP64 ones.
    per_call = {}
    if not args.no_e2e:
        pin = lambda a: torch.tensor(a).pin_memory().numpy()
        rhs0 = pin(M["rhs"])
        hb = {k: pin(M[k]) for k in ("h1", "h2", "mask", "mult", "binv")}
        rhs = pin(M["rhs"])
        u = pin(np.zeros(n))

    def e2e(call, name):
        np.copyto(rhs, rhs0)
        call()  # warm the staging buffers
        tot, ms = 0.0, []
        barrier(pg)
        for _ in range(args.steps):
            np.copyto(rhs, rhs0)
            t0 = time.perf_counter()
            call()
            dt = time.perf_counter() - t0
            tot += dt
            ms.append(round(1e3 * dt, 2))
        barrier(pg)
        per_call[name] = ms
        return allmax(pg, tot)

    rmx = timed(mixed)
    x_mx = x.clone()
    if not args.no_e2e:
        tm = e2e(lambda: lib.hmholtz_mixed("TEMP", u, rhs, hb["h1"], hb["h2"], hb["mask"],
                                           hb["mult"], 1, -args.tol, big, 1, hb["binv"],
                                           inner_tol=args.inner_tol), "mixed")
    if args.only_mixed:  # profiling runs: iteration count of the FP64 solve not measured
        r64 = dict(iters=[0], T=1.0, ms_ax=float("nan"), launches=0, clocks=None)
    else:
        r64 = timed(fp64)
    it64 = r64["iters"][0]
    v64 = allsum(pg, n * sum(r64["iters"])) / r64["T"] if not args.only_mixed else float("nan")
    b64 = 8 * 12  # fused operator: r, d, p_old, G1..G6, bm1 in; p, w out (FP64 words)
    ns64 = ncu_summary("axhelm_fused_f64_n7")
    fp64_block = {
        "value": v64, "unit": "DOF-iters/s", "iterations": r64["iters"],
        "ms_per_solve": 1e3 * r64["T"] / args.steps,
        "axhelm": {"kernel": f"axhelm_kernel<{M['lx1']},double,fused>",
                   "avg_launch_ms": r64["ms_ax"],
                   "GB/s": b64 * n / (r64["ms_ax"] * 1e-3) / 1e9, "bytes_per_point": b64,
                   "fp64_tflops": flops_pt * n / (r64["ms_ax"] * 1e-3) / 1e12,
                   "ncu_fp64_pipe_active_pct": (ns64 or {}).get("fp64_pipe_active_pct"),
                   "ncu_source": (f"{ns64['source']}: committed ncu capture at E=20^3 "
                                  "(not measured in this run)") if ns64 else None},
        "per_iteration_ms": r64.get("per_iter_ms"),
        "gpu_launches": r64["launches"], "clocks": r64["clocks"]}
    x64 = x.clone() if not args.only_mixed else None
    # the same FP64 solve with the double-float operator (NEKGPU_OPT_DF)
    df_block = None
    if not args.only_mixed and not args.no_df:
        lib.set_option(10, 1)
        rdf = timed(fp64)
        lib.set_option(10, 0)
        vdf = allsum(pg, n * sum(rdf["iters"])) / rdf["T"]
        nsdf = ncu_summary("axhelm_df_f64_n7")
        df_block = {
            "value": vdf, "unit": "DOF-iters/s", "iterations": rdf["iters"],
            "ms_per_solve": 1e3 * rdf["T"] / args.steps,
            "axhelm": {"kernel": f"axhelm_df_kernel<{M['lx1']},fused> (double-float contractions "
                                 "on the FP32 pipe, FP64 in/out)",
                       "avg_launch_ms": rdf["ms_ax"],
                       "GB/s": b64 * n / (rdf["ms_ax"] * 1e-3) / 1e9, "bytes_per_point": b64,
                       "frac_of_hbm_peak": b64 * n / (rdf["ms_ax"] * 1e-3) / 1e9 / peak,
                       "speedup_vs_fp64_operator": r64["ms_ax"] / rdf["ms_ax"],
                       "ncu_fp64_pipe_active_pct": (nsdf or {}).get("fp64_pipe_active_pct"),
                       "ncu_fma_pipe_active_pct": (nsdf or {}).get("fma_pipe_active_pct"),
                       "ncu_source": (f"{nsdf['source']}: committed ncu capture at E=20^3 "
                                      "(not measured in this run)") if nsdf else None},
            "per_iteration_ms": rdf.get("per_iter_ms"),
            "rel_error_vs_fp64_operator_solution":
                float(torch.linalg.norm(x - x64) / torch.linalg.norm(x64)),
            "gpu_launches": rdf["launches"], "clocks": rdf["clocks"]}
        x_df = x.clone()
    err64 = (float(torch.linalg.norm(x_mx - x64) / torch.linalg.norm(x64))
             if x64 is not None else None)
    outer = [o for o, i in rmx["iters"]]
    inner = [i for o, i in rmx["iters"]]
    # time to solution, counted with the FP64 solve's iteration count
    vmx = allsum(pg, n * (it64 or sum(inner) // len(inner)) * args.steps) / rmx["T"]
    # The FP32 operator of the inner solve.  Element-local form: r, d, p_old,
    # G1..G6, bm1 in, p and w out (12 words per point).  Assembled-boundary
    # form (even lx1, mixed mode 1): G1..G6 and bm1 per point, r, d, p_old once
    # per global node (interior per element, boundary per node), the 4-byte
    # group index of every element-boundary point, w out once per point.
    lx1 = M["lx1"]
    split = (args.split and args.mixed_mode == 1 and lx1 % 2 == 0 and lx1 >= 4)
    if split:
        ni = (lx1 - 2) ** 3
        nb_nodes = boundary_nodes(M["glo_num"], lx1)
        b32 = (4 * (6 + (1 if M["h2"][0] != 0 else 0) + 1)
               + 12.0 * (ni * M["nel"] + nb_nodes) / n + 4.0 * (lx1 ** 3 - ni) / lx1 ** 3)
        kname = f"split_ax_kernel<{lx1},1> (fp32 operator, assembled-boundary layout)"
    else:
        b32 = 4 * 12
        kname = f"fused fp32 operator lx1={lx1} (inner solve)"
    ax_gbs = b32 * n / (rmx["ms_ax"] * 1e-3) / 1e9
    ns32 = ncu_summary("split_ax_f32_n7" if split else "axhelm_fused_f32_n7")
    line = {"metric": METRIC, "value": vmx, "unit": "DOF-iters/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * rmx["T"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 inner / f64 outer",
            "data": "synthetic",
            "config": {"workload": workload_name(args), "n_points": n,
                       "solver": "mixed: fp32 jacobi-pcg (inner tol "
                                 f"{args.inner_tol:g}) in fp64 defect correction, " +
                                 ("fp64 residual replacement, search direction kept"
                                  if args.mixed_mode == 1 else "restarted per outer step"),
                       "value_definition": "n * (FP64 PCG iteration count) / mixed solve time",
                       "tol": args.tol, "outer_steps": outer, "inner_iterations": inner,
                       "inner_rate_dof_iters_per_s": allsum(pg, n * sum(inner)) / rmx["T"],
                       "rel_error_vs_fp64_solution": err64,
                       "gs_shape_fp32": lib.gs_shape(1)[:2],
                       "operator_shape": {"fp64": lib.ax_shape(0)[:2], "fp32": lib.ax_shape(1)[:2],
                                          "note": "(kind 0 plain / 1 TMA, elements per block), "
                                                  "autotuned on the first solve"},
                       "l2": "inputs larger than L2", "parallelism": f"replicas{ws}"},
            "fp64": fp64_block,
            "fp64_df": df_block,
            "speedup_mixed_vs_fp64": vmx / v64 if v64 > 0 else None,
            "roofline": {"kernel": kname,
                         "bound": "hbm",
                         "achieved": ax_gbs, "peak": peak, "unit": "GB/s", "frac": ax_gbs / peak,
                         "peak_source": peak_src, "bytes_per_point": b32,
                         "avg_launch_ms": rmx["ms_ax"], "launches_timed": rmx["n_ax"],
                         "inner_iteration_ms": rmx["per_iter_ms"],
                         "traffic": ns32["dram_bytes_per_point"] * n if ns32 else None,
                         "traffic_source": (f"{ns32['source']}: DRAM bytes per point of a "
                                            "committed ncu capture at E=20^3, times this n "
                                            "(not measured in this run)") if ns32 else None},
            "gpu_launches": rmx["launches"],
            "clocks": rmx["clocks"]}
    if not args.no_e2e:
        t6 = e2e(lambda: lib.hmholtz("TEMP", u, rhs, hb["h1"], hb["h2"], hb["mask"], hb["mult"], 1,
                                     -args.tol, big, 1, hb["binv"], maxcg=big), "fp64")
        line["e2e"] = {"value": allsum(pg, n * it64 * args.steps) / tm, "unit": "DOF-iters/s",
                       "h2d_bytes_per_step": 6 * 8 * n, "d2h_bytes_per_step": 2 * 8 * n,
                       "api": "nekgpu_hmholtz_mixed (host arrays, pinned)",
                       "ms_per_call": per_call["mixed"],
                       "measured": "right after the device-timed mixed solve, before the FP64 "
                                   "solves"}
        fp64_block["e2e"] = {"value": allsum(pg, n * it64 * args.steps) / t6,
                             "unit": "DOF-iters/s", "api": "nekgpu_hmholtz (host arrays, pinned)"}
    # ---- CPU baseline (oracle) on rank 0, N=1 only ------------------------------
    if rank == 0 and ws == 1 and not args.no_cpu:
        nth = os.cpu_count() or 1
        iters_cpu = args.cpu_iters or 200
        v, it, dt = cpu_sample(M, nth, iters_cpu)
        v1, it1, dt1 = cpu_sample(M, 1, max(2, iters_cpu // 10))
        line["cpu_baseline"] = {"value": v, "unit": "DOF-iters/s", "cores": nth, "kind": "port",
                                "cpu_model": cpu_model(),
                                "sample": f"{it} Jacobi-PCG iterations of the full problem "
                                          f"({dt:.1f} s), C restatement of the reference, FP64",
                                "one_core": {"value": v1, "unit": "DOF-iters/s", "cores": 1,
                                             "sample": f"{it1} iterations ({dt1:.1f} s)"}}
    # ---- parity against the oracle at this size (outside every timed region) ----
    if rank == 0 and ws == 1 and not args.no_parity and x64 is not None:
        line["parity"] = oracle_parity(M, x64.cpu().numpy(), x_mx.cpu().numpy(), it64,
                                       args.tol, os.cpu_count() or 1,
                                       None if df_block is None else x_df.cpu().numpy())
    if rank == 0:
        print(json.dumps(line), flush=True)
    lib.close()


def batch_workload(nprob, seed=4):
    """Three velocity-component Helmholtz problems (E=16^3, N=7, h1=1,
    h2=1.5/dt with dt=1e-3) plus nprob Poisson problems with E log-uniform in
    [64, 8192] (near-cubic kx*ky*kz) and N uniform in 5..9; every problem a
    seeded deformed box with a standard-normal right-hand side."""
    from nek5000_gb300 import mesh
    rng = np.random.default_rng(seed)
    specs = [(7, (16, 16, 16), 1500.0, 100 + c) for c in range(3)]
    for q in range(nprob):
        E = int(round(np.exp(rng.uniform(np.log(64), np.log(8192)))))
        kx = max(2, int(round(E ** (1 / 3))))
        ky = max(2, int(round((E / kx) ** 0.5)))
        kz = max(2, int(round(E / (kx * ky))))
        specs.append((int(rng.integers(5, 10)), (kx, ky, kz), 0.0, 200 + q))
    probs = []
    for N, (kx, ky, kz), h2, sd in specs:
        M = mesh.box_mesh(N, kx, ky, kz, seed=sd)
        r = np.random.default_rng(sd)
        nglob = int(M["lattice"].max()) + 1
        fg = r.standard_normal(nglob)[M["lattice"]]
        M["f"] = mesh.dssum_host(M["lattice"], M["bm1"] * fg, nglob) * M["mask"]
        M["h1"] = np.ones(M["n"])
        M["h2"] = np.full(M["n"], h2)
        M["spec"] = (N, kx, ky, kz, h2)
        for k in ("x", "y", "z"):
            M.pop(k, None)
        probs.append(M)
    return probs


def run_batch(args):
    import torch
    ws, rank, local, pg = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    from nek5000_gb300 import NekGpuBatch
    from nek5000_gb300 import build as nb
    nb.build()
    probs = batch_workload(args.batch_problems)
    B = NekGpuBatch(local)
    B.set_persistent(args.persistent_batch)
    for M in probs:
        B.add(M["lx1"], M["nel"], M["D"], M["g"], M["bm1"], M["glo_num"])
        M.pop("g")
    dev = lambda a: torch.tensor(a, device=f"cuda:{local}")
    cols = {k: [dev(M[k]) for M in probs] for k in ("f", "h1", "h2", "mask", "mult", "binv")}
    xs = [torch.zeros(M["n"], dtype=torch.float64, device=f"cuda:{local}") for M in probs]
    ns = np.array([M["n"] for M in probs], dtype=np.float64)

    def solve(mixed):
        return B.solve(xs, cols["f"], cols["h1"], cols["h2"], cols["mask"], cols["mult"],
                       cols["binv"], tin=-args.tol,
                       mixed=(1 if args.mixed_mode == 1 else 2) if mixed else 0,
                       inner_tol=args.inner_tol)

    out = {}
    # --only-mixed (profiling runs): the FP64 leg is skipped, and the value is
    # counted with the mixed solve's inner iterations
    for mixed in ((True,) if args.only_mixed else (False, True)):
        for _ in range(args.warmup):
            solve(mixed)
        barrier(pg)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with Clocks(local) as ck:
            for _ in range(args.steps):
                res = solve(mixed)
            torch.cuda.synchronize()
        T = allmax(pg, time.perf_counter() - t0)
        if any(s != 0 for s in res["status"]):
            raise RuntimeError(f"batch: status {res['status']}: {B.last_error()}")
        out[mixed] = dict(res=res, T=T, clocks=ck.summary())
    if args.only_mixed:
        out[False] = dict(res=out[True]["res"], T=float("nan"), clocks=None)
    it64 = np.array(out[False]["res"]["niter"], dtype=np.float64)
    v64 = allsum(pg, float((ns * it64).sum()) * args.steps) / out[False]["T"]
    vmx = allsum(pg, float((ns * it64).sum()) * args.steps) / out[True]["T"]
    line = {"metric": METRIC + " (batched workload)", "value": vmx, "unit": "DOF-iters/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * out[True]["T"] / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 inner / f64 outer",
            "data": "synthetic",
            "config": {"workload": f"batch: 3 x helmholtz E=16^3 N=7 h2=1500 + "
                                   f"{args.batch_problems} poisson E in [64,8192] log-uniform, "
                                   "N in 5..9", "problems": len(probs),
                       "n_points_total": int(ns.sum()),
                       "value_definition": "sum_p n_p * (FP64 iterations of p) / batch solve time",
                       "orders": [M["spec"][0] for M in probs],
                       "elements": [M["nel"] for M in probs],
                       "fp64_iterations": out[False]["res"]["niter"],
                       "mixed_inner_iterations": out[True]["res"]["niter"],
                       "mixed_outer_steps": out[True]["res"]["nouter"],
                       "solver": "mixed: fp32 jacobi-pcg (inner tol "
                                 f"{args.inner_tol:g}) in fp64 defect correction, " +
                                 ("fp64 residual replacement, search direction kept"
                                  if args.mixed_mode == 1 else "restarted per outer step"),
                       "operator_block_threads": {"fp64": B.shape(0)[0], "fp32": B.shape(1)[0],
                                                  "note": "plain operator body, autotuned on "
                                                          "the first solve (graph form); 256 "
                                                          "in the persistent form"},
                       "fp32_operator_form_by_lx1": {str(k): ("tma" if v else "plain")
                                                     for k, v in B.operator_forms().items()},
                       "launch_form": ("one persistent cooperative launch per segment"
                                       if args.persistent_batch else
                                       "per iteration one operator launch per order (FP32: "
                                       "TMA-staged or plain body, tuned per order) + "
                                       "boundary-group + update, graph-replayed"),
                       "parallelism": f"replicas{ws}"},
            "fp64": {"value": v64, "unit": "DOF-iters/s",
                     "ms_per_step": 1e3 * out[False]["T"] / args.steps},
            "speedup_mixed_vs_fp64": vmx / v64,
            "clocks": out[True]["clocks"]}
    if rank == 0:
        print(json.dumps(line), flush=True)
    B.close()


def run_sweep(args):
    """In-solve fused operator at N = 5...9 on the E=32^3 Helmholtz box:
    60 PCG iterations per precision, every operator launch timed with CUDA
    events; bytes per point are the fused operator's algorithmic 12 words."""
    import torch
    ws, rank, local, pg = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    from nek5000_gb300 import NekGpu
    from nek5000_gb300 import build as nb
    nb.build()
    peak, peak_src = peaks()
    rows = []
    l0 = None
    for N in (5, 6, 7, 8, 9):
        M = workload(args.k, N)
        n = M["n"]
        lib = NekGpu(local)
        lib.setup(M["lx1"], M["nel"], M["D"], M["g"], M["bm1"], M["glo_num"])
        lib.set_option(2, 1)
        dev = lambda a: torch.tensor(a, device=f"cuda:{local}")
        a = [dev(M[c]) for c in ("f", "h1", "h2", "mask", "mult")]
        binv = dev(M["binv"])
        x = torch.zeros(n, dtype=torch.float64, device=f"cuda:{local}")
        row = {"N": N, "n_points": n}
        if l0 is None:
            l0 = lib.launch_count()
        for prec, w in ((0, 8), (1, 4)):
            for rep in range(2):  # the first call also tunes the launch shape
                if prec == 0:
                    lib.cggo(x, *a, 1, -1e-30, 60, 1, binv, maxcg=60)
                else:
                    lib.cggo_mixed(x, *a, 1, -1e-30, 60, 1, binv)
            t_tot, t_ax, k_ax = lib.last_timing()
            ms = t_ax / max(k_ax, 1)
            gbs = 12 * w * n / (ms * 1e-3) / 1e9
            row["fp64" if prec == 0 else "fp32"] = {
                "avg_launch_ms": ms, "launches": k_ax, "GB/s": gbs, "frac": gbs / peak,
                "shape": lib.ax_shape(prec)[:2]}
        rows.append(row)
        lib.close()
        del a, binv, x, M
        torch.cuda.empty_cache()
    if rank == 0:
        print(json.dumps({"metric": "fused operator HBM GB/s in the PCG, N=5..9",
                          "unit": "GB/s", "peak": peak, "peak_source": peak_src,
                          "workload": f"helmholtz E={args.k}^3 h1=1 h2=10, 60 iterations",
                          "bytes_per_point": {"fp64": 96, "fp32": 48},
                          "sweep": rows}), flush=True)


def run_hsolve(args):
    """Time stepping with projection (hsolve, navier4.f:562): a sequence of
    FP64 Helmholtz solves (E=k^3, N, h1 = 1, h2 = 1500 as for a velocity step
    with dt = 1e-3) whose right-hand sides vary smoothly, each to the absolute
    tolerance tol * rinit of the first, once through nekgpu_hsolve_dev
    (projection space of 8) and once through plain cggo."""
    import torch
    ws, rank, local, pg = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    from nek5000_gb300 import NekGpu, mesh
    from nek5000_gb300 import build as nb
    nb.build()
    M = mesh.box_mesh(args.N, args.k, args.k, args.k, seed=3)
    n = M["n"]
    nglob = int(M["lattice"].max()) + 1
    lib = NekGpu(local)
    lib.setup(M["lx1"], M["nel"], M["D"], M["g"], M["bm1"], M["glo_num"])
    dev = lambda a: torch.tensor(a, device=f"cuda:{local}")
    h1, h2 = dev(np.ones(n)), dev(np.full(n, 1500.0))
    mask, mult, binv = dev(M["mask"]), dev(M["mult"]), dev(M["binv"])
    rng = np.random.default_rng(3)
    fs = [rng.standard_normal(nglob)[M["lattice"]] for _ in range(3)]
    bm1 = dev(M["bm1"])
    steps = max(args.steps, 1) * 10

    def rhs(t):  # local (unassembled) right-hand side, as hsolve takes it
        f = fs[0] + np.sin(0.05 * t) * fs[1] + 1e-3 * t * fs[2]
        return dev(M["bm1"] * f)

    rinit = None
    out = {}
    for mode in ("projection", "plain"):
        lib.proj_setup(0, 8)
        its, ms = [], []
        for t in range(steps + args.warmup):
            r = rhs(t)
            if rinit is None:
                ra = lib.dssum(r.clone()) * mask
                rinit = float(torch.sqrt(torch.sum(mult * binv * ra * ra) / torch.sum(bm1)))
            tol = args.tol * rinit
            u = torch.zeros(n, dtype=torch.float64, device=f"cuda:{local}")
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if mode == "projection":
                it, r0, r2, m, rc = lib.hsolve("VELX", u, r, h1, h2, mask, mult, 1, tol, 10 ** 6,
                                               1, binv, space=0, maxcg=10 ** 6)
            else:  # hmholtz's right-hand side: dssum, then mask
                r = lib.dssum(r) * mask
                it, r0, r2, rc = lib.cggo(u, r, h1, h2, mask, mult, 1, tol, 10 ** 6, 1, binv,
                                          maxcg=10 ** 6)
            torch.cuda.synchronize()
            if t >= args.warmup:
                its.append(it)
                ms.append(1e3 * (time.perf_counter() - t0))
        out[mode] = {"iterations": its, "ms_per_solve": sum(ms) / len(ms),
                     "total_s": sum(ms) / 1e3}
    if rank == 0:
        sp = out["plain"]["total_s"] / out["projection"]["total_s"]
        print(json.dumps({"metric": "time-stepping Helmholtz solves with projection onto "
                                    "previous solutions (hsolve)",
                          "value": out["projection"]["ms_per_solve"], "unit": "ms/solve",
                          "higher_is_better": False, "steps": steps, "warmup": args.warmup,
                          "n_gpus": ws, "dtype": "f64", "data": "synthetic",
                          "config": {"workload": f"helmholtz E={args.k}^3 N={args.N} h1=1 "
                                                 "h2=1500 dirichlet-all, rhs f0 + sin(0.05t) f1 "
                                                 "+ 1e-3 t f2", "n_points": n,
                                     "tol": f"{args.tol:g} * rinit (absolute)",
                                     "projection_space": 8},
                          "projection": out["projection"], "plain_cggo": out["plain"],
                          "speedup_projection_vs_plain": sp}), flush=True)
    lib.close()


def run_adjoint(args):
    """Gradient of J = 0.5 |u - u*|_B^2 with respect to the per-point viscosity
    h1 on E=16^3, N=7 (h1 = exp(0.3 g), g a seeded smooth random field of
    correlation length 0.2; h2 = 0; all-Dirichlet box): forward FP64 solve,
    adjoint solve (the operator is symmetric) and the axhelm adjoint kernel,
    every step on the device."""
    import torch
    ws, rank, local, pg = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    from nek5000_gb300 import NekGpu, mesh
    from nek5000_gb300 import build as nb
    nb.build()
    k = 16 if args.k == 32 else args.k
    M = mesh.box_mesh(args.N, k, k, k, seed=5)
    n = M["n"]
    x, y, z = M["x"], M["y"], M["z"]
    r = np.random.default_rng(5)
    kv = r.standard_normal((64, 3)) / 0.2
    ph = r.uniform(0, 2 * np.pi, 64)
    am = r.standard_normal(64) * np.sqrt(2.0 / 64)
    g = np.zeros(n)
    for q in range(64):  # the Gaussian random field, mode by mode
        g += am[q] * np.cos(x * kv[q, 0] + y * kv[q, 1] + z * kv[q, 2] + ph[q])
    h1v = np.exp(0.3 * g)
    lib = NekGpu(local)
    lib.setup(M["lx1"], M["nel"], M["D"], M["g"], M["bm1"], M["glo_num"])
    dev = lambda a: torch.tensor(a, device=f"cuda:{local}")
    h1, h2 = dev(h1v), torch.zeros(n, dtype=torch.float64, device=f"cuda:{local}")
    mask, mult, binv, bm1 = dev(M["mask"]), dev(M["mult"]), dev(M["binv"]), dev(M["bm1"])
    nglob = int(M["lattice"].max()) + 1
    f = dev(M["bm1"] * np.random.default_rng(6).standard_normal(nglob)[M["lattice"]])
    lib.dssum(f)
    f = f * mask
    ustar = torch.zeros(n, dtype=torch.float64, device=f"cuda:{local}")
    lib.cggo(ustar, f, dev(h1v * 1.1), h2, mask, mult, 1, -1e-10, 10 ** 6, 1, binv, maxcg=10 ** 6)

    def gradient():
        u = torch.zeros_like(ustar)
        it1, _, _, _ = lib.cggo(u, f, h1, h2, mask, mult, 1, -1e-10, 10 ** 6, 1, binv,
                                maxcg=10 ** 6)
        gsrc = bm1 * (u - ustar)
        lib.dssum(gsrc)
        gsrc = gsrc * mask
        lam = torch.zeros_like(u)
        it2, _, _, _ = lib.cggo_adjoint(lam, gsrc, h1, h2, mask, mult, 1, -1e-10, 10 ** 6, 1,
                                        binv, maxcg=10 ** 6)
        gh1 = torch.zeros_like(u)
        lib.axhelm_adjoint_h1(gh1, lam, u)
        return it1, it2, -gh1

    for _ in range(args.warmup):
        gradient()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        it1, it2, grad = gradient()
    torch.cuda.synchronize()
    T = (time.perf_counter() - t0) / args.steps
    if rank == 0:
        print(json.dumps({"metric": "adjoint gradient dJ/dh1 (forward solve + adjoint solve + "
                                    "axhelm adjoint)", "value": 1e3 * T, "unit": "ms/gradient",
                          "higher_is_better": False, "steps": args.steps, "warmup": args.warmup,
                          "n_gpus": ws, "dtype": "f64", "data": "synthetic",
                          "config": {"workload": f"E={k}^3 N={args.N} h1=exp(0.3 g) h2=0 "
                                                 "dirichlet-all", "n_points": n,
                                     "forward_iterations": it1, "adjoint_iterations": it2,
                                     "grad_norm": float(torch.linalg.norm(grad))}}), flush=True)
    lib.close()


VELOCITY_FACES = ((True, True, True, True, True, True),      # u: every wall
                  (True, True, False, False, False, False),  # v: x walls only
                  (True, True, True, True, True, False))     # w: outflow at z+


def run_velocity3(args):
    """The three velocity components of one time step (ophinv,
    core/induct.f:1064-1071): one deformed box E=k^3, N (seed 4), h1 = 1,
    h2 = 1500 (1.5/dt, dt = 1e-3), a mask per component (every wall; the x
    walls only; every wall but the z+ outflow), standard-normal right-hand
    sides per global node (seeds 40, 41, 42), each solved to tol * its rbn0.
    Timed three ways: the fused multi-field mixed solve
    (nekgpu_cggo_mixed_multi_dev), three single-field mixed solves, three FP64
    solves."""
    import torch
    ws, rank, local, pg = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    from nek5000_gb300 import NekGpu, mesh
    from nek5000_gb300 import build as nb
    nb.build()
    M = mesh.box_mesh(args.N, args.k, args.k, args.k, seed=4)
    n = M["n"]
    nglob = int(M["lattice"].max()) + 1
    dev = lambda a: torch.tensor(a, device=f"cuda:{local}")
    masks, fs = [], []
    for c, faces in enumerate(VELOCITY_FACES):
        mk = mesh.face_mask(M, faces)
        g = np.random.default_rng(40 + c).standard_normal(nglob)[M["lattice"]]
        masks.append(dev(mk))
        fs.append(dev(mesh.dssum_host(M["lattice"], M["bm1"] * g, nglob) * mk))
    lib = NekGpu(local)
    lib.setup(M["lx1"], M["nel"], M["D"], M["g"], M["bm1"], M["glo_num"])
    h1, h2 = dev(np.ones(n)), dev(np.full(n, 1500.0))
    mult, binv = dev(M["mult"]), dev(M["binv"])
    del M
    xs = [torch.zeros(n, dtype=torch.float64, device=f"cuda:{local}") for _ in range(3)]
    big = 10 ** 6
    lib.set_option(2, 1)  # timing: solve-total and per-kernel events
    kt = [0.0, 0.0, 0.0, 0]  # operator, boundary groups, update ms; iterations

    def kernel_times():
        t_ax, t_gs, t_up, it = lib.last_kernel_times()
        for q, v in enumerate((t_ax, t_gs, t_up, it)):
            kt[q] += v

    def multi():
        r = lib.cggo_mixed_multi(xs, fs, h1, h2, masks, mult, 1, -args.tol, big, 1, binv,
                                 inner_tol=args.inner_tol)
        if any(r["status"]):
            raise RuntimeError(f"multi-field solve: {r} {lib.last_error()}")
        kernel_times()
        return r["ninner"]

    def mixed():
        its = []
        for c in range(3):
            no, ni, r0, r2, rc = lib.cggo_mixed(xs[c], fs[c], h1, h2, masks[c], mult, 1,
                                                -args.tol, big, 1, binv, inner_tol=args.inner_tol)
            if rc:
                raise RuntimeError(lib.last_error())
            kernel_times()
            its.append(ni)
        return its

    def fp64():
        its = []
        for c in range(3):
            it, r0, r2, rc = lib.cggo(xs[c], fs[c], h1, h2, masks[c], mult, 1, -args.tol, big, 1,
                                      binv, maxcg=big)
            if rc:
                raise RuntimeError(lib.last_error())
            its.append(it)
        return its

    def timed(solve):
        for _ in range(args.warmup):
            solve()
        barrier(pg)
        torch.cuda.synchronize()
        l0 = lib.launch_count()
        t = 0.0
        kt[:] = [0.0, 0.0, 0.0, 0]
        with Clocks(local) as ck:
            for _ in range(args.steps):
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                its = solve()
                torch.cuda.synchronize()
                t += time.perf_counter() - t0
        barrier(pg)
        k = max(kt[3], 1)
        return dict(its=its, T=allmax(pg, t), launches=lib.launch_count() - l0,
                    clocks=ck.summary(),
                    per_iter_ms={"operator": kt[0] / k, "boundary_groups": kt[1] / k,
                                 "update": kt[2] / k, "iterations_timed": kt[3]})

    out = {}
    if not args.only_mixed:
        out["fp64"] = timed(fp64)
        ref = [x.clone() for x in xs]
        out["mixed_single"] = timed(mixed)
    out["mixed_multi"] = timed(multi)
    err = (max(float(torch.linalg.norm(xs[c] - ref[c]) / torch.linalg.norm(ref[c]))
               for c in range(3)) if not args.only_mixed else None)
    it64 = out["fp64"]["its"] if "fp64" in out else out["mixed_multi"]["its"]
    rate = {k: allsum(pg, n * sum(it64) * args.steps) / v["T"] for k, v in out.items()}
    # the fused operator's algorithmic bytes: G (6), d, bm1 once; p, r in and
    # p, w out per field (FP32 words)
    b_op = 4 * (8 + 4 * 3)
    op_ms = out["mixed_multi"]["per_iter_ms"]["operator"]
    gbs = b_op * n / (op_ms * 1e-3) / 1e9 if op_ms > 0 else None
    peak, peak_src = peaks()
    if rank == 0:
        ms = {k: 1e3 * v["T"] / args.steps for k, v in out.items()}
        single = out.get("mixed_single")
        print(json.dumps({
            "metric": "DOF-iters/s, 3 velocity components E=32^3 N=7 to 1e-10 (fused "
                      "multi-field mixed solve)",
            "value": rate["mixed_multi"], "unit": "DOF-iters/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms["mixed_multi"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32 inner / f64 outer", "data": "synthetic",
            "config": {"workload": f"velocity E={args.k}^3 N={args.N} h1=1 h2=1500, 3 fields "
                                   "(masks: all walls / x walls / all but z+)",
                       "n_points": n, "tol": args.tol, "inner_tol": args.inner_tol,
                       "value_definition": "n * (sum of the 3 FP64 PCG iteration counts) / time "
                                           "of the 3-field solve",
                       "fp64_iterations": it64 if "fp64" in out else None,
                       "inner_iterations_single": single["its"] if single else None,
                       "inner_iterations_multi": out["mixed_multi"]["its"],
                       "rel_error_vs_fp64_solution": err,
                       "l2": "inputs larger than L2", "parallelism": f"replicas{ws}"},
            "ms_per_3_field_solve": ms, "dof_iters_per_s": rate,
            "inner_iteration_ms": {k: v["per_iter_ms"] for k, v in out.items()},
            "speedup_multi_vs_single_mixed": (single["T"] / out["mixed_multi"]["T"]
                                              if single else None),
            "speedup_multi_vs_fp64": (out["fp64"]["T"] / out["mixed_multi"]["T"]
                                      if "fp64" in out else None),
            "roofline": {"kernel": f"fused 3-field fp32 operator lx1={args.N + 1}",
                         "bound": "hbm", "achieved": gbs, "peak": peak, "unit": "GB/s",
                         "frac": gbs / peak if gbs else None, "peak_source": peak_src,
                         "bytes_per_point": b_op, "avg_launch_ms": op_ms, "traffic": None},
            "gpu_launches": out["mixed_multi"]["launches"],
            "clocks": out["mixed_multi"]["clocks"]}), flush=True)
    lib.close()


def run_pressure(args):
    """The pressure solve's Krylov method (hmh_gmres, restart 30) on the
    E=k^3, N Poisson problem (all-Dirichlet box, h1 = 1, h2 = 0, seed 0), to
    1e-10 of the initial residual norm, beside FP64 Jacobi-PCG (cggo) and the
    flexible CG (hmh_flex_cg) on the same system; all with the Jacobi
    preconditioner."""
    import torch
    ws, rank, local, pg = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    from nek5000_gb300 import NekGpu
    from nek5000_gb300 import build as nb
    nb.build()
    M = workload(args.k, args.N, "poisson", keep_xyz=True)
    n = M["n"]
    lib = NekGpu(local)
    lib.setup(M["lx1"], M["nel"], M["D"], M["g"], M["bm1"], M["glo_num"])
    dev = lambda a: torch.tensor(a, device=f"cuda:{local}")
    f, h1, h2 = dev(M["f"]), dev(M["h1"]), dev(M["h2"])
    mask, mult, binv = dev(M["mask"]), dev(M["mult"]), dev(M["binv"])

    def gmres():
        x = f.clone()
        return lib.hmh_gmres(x, h1, h2, mult, mask, -args.tol, maxit=10 ** 5, kmax=30)

    def cg():
        x = torch.zeros(n, dtype=torch.float64, device=f"cuda:{local}")
        return lib.cggo(x, f, h1, h2, mask, mult, 1, -args.tol, 10 ** 6, 1, binv, maxcg=10 ** 6)

    def flex():
        x = f.clone()
        return lib.hmh_flex_cg(x, h1, h2, mult, mask, -args.tol, maxit=10 ** 6)

    out = {}

    def timed(name, fn):
        for _ in range(args.warmup):
            r = fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with Clocks(local) as ck:
            for _ in range(args.steps):
                r = fn()
            torch.cuda.synchronize()
        T = (time.perf_counter() - t0) / args.steps
        out[name] = dict(iterations=r[0], ms_per_solve=1e3 * T,
                         dof_iters_per_s=n * r[0] / T, clocks=ck.summary())

    for name, fn in (("gmres", gmres), ("cggo", cg), ("flex_cg", flex)):
        timed(name, fn)
    # the reference's own preconditioner for these solves: h1mg_solve
    h1mg = {}
    try:
        t0 = time.perf_counter()
        lib.h1mg_setup(M["x"], M["y"], M["z"], M["glo_num"], mask=M["mask"])
        h1mg["setup_s"] = time.perf_counter() - t0
        timed("gmres_h1mg", gmres)
        timed("flex_cg_h1mg", flex)
        h1mg.update(gmres=out["gmres_h1mg"], flex_cg=out["flex_cg_h1mg"])
        lib.h1mg_free()
    except Exception as exc:  # reported in the line, the Jacobi rows stand
        h1mg["error"] = str(exc)
    # the same with the coarse solve by algebraic multigrid (param(40) = 1)
    h1amg = {}
    try:
        lib.set_option(12, 1)
        t0 = time.perf_counter()
        lib.h1mg_setup(M["x"], M["y"], M["z"], M["glo_num"], mask=M["mask"])
        h1amg["setup_s"] = time.perf_counter() - t0
        timed("gmres_h1mg_amg", gmres)
        timed("flex_cg_h1mg_amg", flex)
        h1amg.update(gmres=out["gmres_h1mg_amg"], flex_cg=out["flex_cg_h1mg_amg"])
        lib.h1mg_free()
        lib.set_option(12, 0)
    except Exception as exc:
        h1amg["error"] = str(exc)
    line = {"metric": f"pressure-solve GMRES (hmh_gmres, restart 30, Jacobi) DOF-iters/s, "
                      f"E={args.k}^3 N={args.N} Poisson",
            "value": out["gmres"]["dof_iters_per_s"], "unit": "DOF-iters/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": out["gmres"]["ms_per_solve"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": {"workload": workload_name(argparse.Namespace(workload="poisson-n9", k=args.k,
                                                                    N=args.N)),
                       "n_points": n, "tol": f"{args.tol:g} x initial rnorm"},
            "gmres": out["gmres"], "cggo_same_system": out["cggo"],
            "flex_cg_same_system": out["flex_cg"], "h1mg_preconditioned": h1mg,
            "h1mg_amg_coarse_preconditioned": h1amg,
            "clocks": out["gmres"]["clocks"]}
    if rank == 0 and ws == 1 and not args.no_cpu:
        from oracle import nekref
        nth = os.cpu_count() or 1
        ops = nekref.Ops(M["lx1"], M["nel"], M["D"], M["g"], M["bm1"], M["glo_num"], nth)
        t0 = time.perf_counter()
        _, itc, _, _ = ops.gmres(M["f"], M["h1"], M["h2"], M["mult"], M["mask"], -args.tol,
                                 maxit=20, m=30)
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": n * itc / dt, "unit": "DOF-iters/s", "cores": nth,
                                "kind": "port",
                                "sample": f"{itc} GMRES iterations of the full problem ({dt:.1f} s),"
                                          " the oracle's hmh_gmres restatement"}
    if rank == 0:
        print(json.dumps(line), flush=True)
    lib.close()


def write_box_re2(path, k, jitter=0.2, seed=6):
    """A #v002 .re2 file of a k^3 box of straight-sided hexahedra on the unit
    cube (interior vertices moved by up to jitter * h, elements in a seeded
    random order), walls on every outside face."""
    rng = np.random.default_rng(seed)
    nv = k + 1
    g = np.stack(np.meshgrid(*(np.arange(nv) / k,) * 3, indexing="ij"), -1)
    inner = np.zeros((nv,) * 3, dtype=bool)
    inner[1:-1, 1:-1, 1:-1] = True
    g[inner] += jitter / k * rng.uniform(-1, 1, (int(inner.sum()), 3))
    nel = k ** 3
    order = rng.permutation(nel)
    ex, ey, ez = order % k, (order // k) % k, order // (k * k)
    pre = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 0, 1), (1, 0, 1), (1, 1, 1), (0, 1, 1)]
    rec = np.zeros((nel, 25))
    for c, (i, j, l) in enumerate(pre):
        for d in range(3):
            rec[:, 1 + 8 * d + c] = g[ex + i, ey + j, ez + l, d]
    faces = []  # preprocessor faces: 1 y-, 2 x+, 3 y+, 4 x-, 5 z-, 6 z+
    for f, on in ((1, ey == 0), (2, ex == k - 1), (3, ey == k - 1), (4, ex == 0),
                  (5, ez == 0), (6, ez == k - 1)):
        q = np.nonzero(on)[0]
        b = np.zeros((len(q), 8))
        b[:, 0], b[:, 1] = q + 1, f
        faces.append(b)
    bcr = np.concatenate(faces)
    bcbytes = bcr.astype("<f8").tobytes()
    # the type occupies the 8th word of each record
    raw = bytearray(bcbytes)
    for r in range(len(bcr)):
        raw[64 * r + 56:64 * r + 64] = b"W       "
    with open(path, "wb") as fh:
        fh.write(f"#v002{nel:9d}{3:3d}{nel:9d} hdr".ljust(80).encode())
        fh.write(np.float32(6.54321).tobytes())
        fh.write(rec.astype("<f8").tobytes())
        fh.write(np.float64(0).tobytes())          # no curved sides
        fh.write(np.float64(len(bcr)).tobytes())   # one boundary section
        fh.write(bytes(raw))
    return nel


def run_ingest(args):
    """Mesh ingestion on the host: a k^3 box of perturbed straight-sided
    hexahedra in a .re2 file read, its vertex connectivity computed from the
    corners (the reference's gencon algorithm), its GLL points numbered
    (set_vert) and placed (xyzlin) at order N, and the mesh handed to the GPU,
    which forms the geometric factors itself (nekgpu_setup_xyz)."""
    import tempfile
    import torch
    from nek5000_gb300 import NekGpu, meshio
    from nek5000_gb300 import build as nb
    from nek5000_gb300.mesh import deriv_matrix, gll
    nb.build()
    k, nx = args.k, args.N + 1
    tmp = tempfile.mkdtemp()
    path = os.path.join(tmp, "box.re2")
    nel = write_box_re2(path, k)
    D = None
    T = {"read_re2": 0.0, "connect": 0.0, "setvert3d": 0.0, "xyzlin": 0.0,
         "gpu_setup_xyz": 0.0}
    steps = max(args.steps, 1)
    for it in range(args.warmup + steps):
        t = [time.perf_counter()]
        R = meshio.read_re2(path)
        t.append(time.perf_counter())
        vertex, nvert = meshio.connect(R["xc"], R["yc"], R["zc"], *R["bcs"][0])
        t.append(time.perf_counter())
        glo, ngv = meshio.setvert3d(nx, vertex)
        t.append(time.perf_counter())
        zg, wg = gll(nx)
        x, y, z = meshio.xyzlin(nx, zg, R["xc"], R["yc"], R["zc"])
        t.append(time.perf_counter())
        D = deriv_matrix(zg)
        lib = NekGpu(0)
        lib.setup_xyz(nx, nel, D, wg, x, y, z, glo)  # geometry formed on the GPU
        torch.cuda.synchronize()
        t.append(time.perf_counter())
        lib.close()
        del x, y, z
        if it >= args.warmup:
            for key, a, b in zip(T, t[:-1], t[1:]):
                T[key] += (b - a) / steps
    native = T["read_re2"] + T["connect"] + T["setvert3d"] + T["xyzlin"]
    line = {"metric": f"mesh ingestion elements/s (.re2 read, connectivity, set_vert, xyzlin; "
                      f"E={k}^3 N={args.N})",
            "value": nel / native, "unit": "elements/s", "n_gpus": 1, "steps": steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * native, "higher_is_better": True,
            "scaling": "none", "vs_baseline": None, "dtype": "f64 / int64", "data": "synthetic",
            "config": {"workload": f"perturbed box E={k}^3 (seeded element order), N={args.N}",
                       "elements": nel, "vertices": int(nvert), "glo_ids": int(ngv),
                       "file_bytes": os.path.getsize(path)},
            "ms": {kk: 1e3 * v for kk, v in T.items()},
            "end_to_end_ms_incl_gpu_setup": 1e3 * sum(T.values())}
    if not args.no_cpu:
        from oracle import nekref
        t0 = time.perf_counter()
        glo_ref, ngv_ref = nekref.setvert3d(nx, nel, vertex.reshape(-1))
        dt = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": nel / dt, "unit": "elements/s (set_vert only)",
                                "cores": 1, "kind": "port",
                                "sample": "the oracle's restatement of set_vert on the same "
                                          "vertex ids (gencon is Fortran: no compiler here)",
                                "identical_glo_num": bool(np.array_equal(glo, glo_ref))}
    print(json.dumps(line), flush=True)
    os.remove(path)
    os.rmdir(tmp)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "axhelm-sweep":
        run_sweep(args)
    elif args.workload == "hsolve":
        run_hsolve(args)
    elif args.workload == "adjoint":
        run_adjoint(args)
    elif args.workload == "velocity3":
        run_velocity3(args)
    elif args.workload == "ingest":
        run_ingest(args)
    elif args.workload == "pressure":
        run_pressure(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
