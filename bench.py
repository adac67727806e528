"""Benchmark: 3D Helmholtz solves/s and FWI gradients/s at a 1e-6 true relative residual on one
GB300, mixed precision (complex64 inner solves under FP64 refinement) against plain FP64.

Headline workload (one "step" = one complete solve): the 201 x 201 x 101 grid (20-point PML,
h = 20 m, 6 Hz, 8 seeded layers 1500->4000 m/s with +-40 m relief and a +-5% random field,
point source at the surface centre), solved by CGMN with the Kaczmarz preconditioner to
||b - H u||_2 / ||b||_2 <= 1e-6 in FP64.

Reported (one JSON line on rank 0):
  value      solves/s with wn and b already in HBM (CUDA events on the launching stream)
  e2e        solves/s through the C ABI with host buffers (h3d_solve_host: the host->device
             copies of wn and b and the device->host copy of u are timed)
  roofline   the dominant kernel (the complex64 BLOCK8 sweep): algorithmic bytes of the timed
             double sweeps (x read and written per right-hand side, the wavenumber read once)
             over their device time, sampled live inside the timed solves by event nodes in the
             solver's CUDA graph
  fp64       the same solve in plain FP64 (mixed-versus-FP64 speed-up, wavefield difference, and
             its algorithmic FP64 flop rate against the nominal FP64 peak: that path is bound by
             GB300's FP64 throughput, not by HBM)
  error_vs_fp64_oracle  both wavefields against the C oracle's FP64 solution of the same
             problem to a true residual of 1.1e-9 (tests/golden/config1_solve.npz)
  mlgmres    the same problem by FGMRES + the three-level ML_GMRES multigrid (the reference
             applications' default solver; h3d_mlgmres_solve): mixed and FP64 seconds per solve,
             outer iterations, the mixed wavefield against the oracle's
  batched    the 256-right-hand-side batch (64 surface sources x 3/4/5/6 Hz, Ricker weights)
             as one batched mixed solve with its sweep's live roofline, beside plain FP64 solves
             of a sample of it (speed-up per solve, wavefield difference on the sample), and
             the same right-hand sides one at a time by FGMRES + ML_GMRES (batched.mlgmres)
  fwi        the FWI gradient of the 161 x 161 x 81 workload (32 sources x 3 frequencies, 400
             receivers) in mixed precision, beside a plain-FP64 gradient of a sample of its
             (source, frequency) pairs, the same gradient with every solve by FGMRES + ML_GMRES
             (fwi.mlgmres, and its difference to the CGMN gradient), and the error of the mixed
             gradient against the FP64 oracle's gradient on the reduced problem of
             tests/golden/config3_grad.npz
  cpu_baseline  the CPU oracle port of the reference algorithm (lexicographic Kaczmarz sweep,
             single-threaded per right-hand side as the reference) timed on a bounded sample of
             CGMN iterations and extrapolated with the reference-order iteration count

--impl reference prints the same line for the CPU reference path alone: each step is a bounded
sample (a few CGMN iterations) of the headline solve, and the run adds one complete, measured
CPU solve of the 61^3 workload.  With torchrun (N > 1) every rank solves its own copy of the
problem (replicas: the (source, frequency) axis shards without any data-path collective); the max
over ranks of the elapsed time is reported and value counts every rank's solves.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "slim-release-apps_gb300"))

METRIC = "3D Helmholtz solves/s & FWI grads/s at 1e-6 resid: mixed batched vs FP64"
WORKLOAD = "config1: 201x201x101 incl. 20-pt PML, h=20 m, 6 Hz, single surface source, 1e-6 true residual"
# Algorithmic flops per grid point: a Kaczmarz double sweep (two passes of 27 complex
# multiply-adds for the projection, 27 for the update and the row norm) and the CGMN vector work
# of one iteration (two inner products and three updates in complex arithmetic).
SWEEP_FLOP_PER_PT = 1040
CG_FLOP_PER_PT = 40
FP64_NOMINAL_TFLOPS = 1.25   # GB300 FP64 (nominal; the FP64 path is bound by it, not by HBM)

# CGMN iterations the reference ordering (lexicographic Kaczmarz double sweep,
# linearsolve.m:148-156 + CGMN.m) needs on the headline workload to reach a true relative
# residual of 1e-6 (true residual 5.08e-7 at stop), measured on a GB300 with the library's LEX
# path, whose arithmetic is the reference sweep's (h3d_solve, order LEX, precision FP64, stop on
# the true residual); `bench.py --derive-ref-iters` measures it again in the same run.
REF_ITERS_CONFIG1 = 1481

# Row order of the timed solves (the solver's tuner then picks the kernel configuration).
DEFAULT_ORDER = "block8"

# DRAM bytes (read + write) per launch of the dominant kernel from one ncu capture of the
# complex64 config-1 solve, keyed by (order, tuned variant).
TRAFFIC_PER_LAUNCH = {("block8", 0): 112.6e6}


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _roofline(sweep_bytes, sweep_seconds, samples, launches_per_ds, kernel, traffic=None):
    """Roofline of the BLOCK8 sweep from the solver's live samples: algorithmic bytes of the
    timed double sweeps over their device time; a launch is a fifteenth of a double sweep."""
    peak, kind = _peaks()
    if not sweep_seconds or not samples:
        return None
    achieved = sweep_bytes / sweep_seconds / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": traffic, "kernel": kernel, "alg_bytes_per_launch": sweep_bytes / samples / launches_per_ds,
            "avg_launch_us": 1e6 * sweep_seconds / samples / launches_per_ds, "samples": samples,
            "peak_source": kind}


def _cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    return platform.processor() or platform.machine()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int = 0):
        self.idx = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(5)
        except Exception:
            self.proc.kill()
        if self.t:
            self.t.join(2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


def _dist_init():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if os.environ.get("H3D_BENCH_GLOO") is None else "gloo")
    return world, rank


def _max_over_ranks(x: float, world: int, dev) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


# ---- the CPU reference: oracle port of linearsolve + CGMN with the lexicographic sweep -----------
class CpuCgmn:
    """The reference algorithm on the host: b~ = DSWP(0, b) with the lexicographic Kaczmarz
    double sweep (the C oracle, equal to the compiled Helm3d_kacz_sweep_mex bit for bit; one
    thread, as the reference runs one right-hand side per thread, Helm3dkaczswp_mex.c:90), then
    CGMN iterations (CGMN.m:48-90) in numpy, timed step by step."""

    def __init__(self, model):
        import numpy as np

        from oracle import h3d_oracle as O

        self.O, self.np = O, np
        self.g = O.make_grid(model.n_total, model.h, model.npml6)
        self.wn = model.wavenumber()
        self.b = model.point_source()
        O.lib()
        t0 = time.perf_counter()
        bt = O.sweep(self.g, self.wn, 1.5, np.zeros_like(self.b), self.b, order=O.ORDER_LEX, nthreads=1)
        self.t_setup = time.perf_counter() - t0
        self.normb = np.linalg.norm(bt)
        self.x = np.zeros_like(bt)
        self.r = bt.copy()
        self.p = self.r.copy()
        self.rr = np.vdot(self.r, self.r).real
        self.iters = 0

    def iterate(self, k: int) -> float:
        """k CGMN iterations; returns their wall time."""
        O, np = self.O, self.np
        t0 = time.perf_counter()
        for _ in range(k):
            y = O.sweep(self.g, self.wn, 1.5, self.p, None, order=O.ORDER_LEX, nthreads=1)
            Ap = self.p - y
            alpha = self.rr / np.vdot(self.p, Ap)
            self.x += alpha * self.p
            self.r -= alpha * Ap
            rn = np.vdot(self.r, self.r).real
            self.p = self.r + (rn / self.rr) * self.p
            self.rr = rn
            self.iters += 1
        return time.perf_counter() - t0

    def ratio(self) -> float:
        return float(self.np.sqrt(self.rr) / self.normb)


def cpu_full_solve(model, tol=1e-6, maxit=2000):
    """One complete reference-order CPU solve (preconditioned stop, CGMN.m:79)."""
    c = CpuCgmn(model)
    t = c.t_setup
    while c.iters < maxit and c.ratio() > tol:
        t += c.iterate(1)
    return {"seconds": t, "iters": c.iters, "rel_res_prec": c.ratio()}


def cpu_sample(model, iters: int, ref_iters: int):
    c = CpuCgmn(model)
    t_iter = c.iterate(iters) / iters
    return {"t_iter_s": t_iter, "t_setup_s": c.t_setup, "value": 1.0 / (c.t_setup + ref_iters * t_iter)}


def run_reference_arm(args, world, rank):
    from h3d import models

    if rank != 0:
        return
    m = models.config1()
    ref_iters = args.ref_iters or REF_ITERS_CONFIG1
    c = CpuCgmn(m)
    for _ in range(args.warmup):
        c.iterate(1)
    step_times = [c.iterate(args.ref_sample_iters) for _ in range(max(1, args.steps))]
    n_it = args.ref_sample_iters * len(step_times)
    t_iter = sum(step_times) / n_it
    v = 1.0 / (c.t_setup + ref_iters * t_iter)
    cpu = {"value": v, "unit": "solves/s", "cores": 1, "kind": "port", "cpu_model": _cpu_model(),
           "sample": f"each step: {args.ref_sample_iters} CGMN iterations of the headline solve (LEX-ordered "
                     f"oracle port, one thread); pooled over {n_it} iterations: {t_iter:.3f} s per iteration "
                     f"(MEASURED); value EXTRAPOLATED to a full solve as the setup sweep ({c.t_setup:.2f} s) + "
                     f"{ref_iters} reference-order iterations (REF_ITERS_CONFIG1, measured on a GB300 with the "
                     f"bit-compatible LEX path)",
           "measured": {"t_iter_s": t_iter, "iters_timed": n_it, "t_setup_s": c.t_setup}}
    if not args.skip_config0:
        s0 = cpu_full_solve(models.config0())
        cpu["full_solve_config0"] = {
            "workload": "config0: 61^3 incl. 10-pt PML, h=25 m, 4 Hz, point source, reference stop 1e-6",
            "seconds": s0["seconds"], "iters": s0["iters"], "rel_res_prec": s0["rel_res_prec"], "cores": 1,
            "measured": True, "solves_per_s": 1.0 / s0["seconds"]}
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "solves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        # one timed step is the bounded sample (ref_sample_iters iterations), not a full solve
        "ms_per_step": 1e3 * sum(step_times) / len(step_times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
        "data": "synthetic (seeded config-1 model)",
        "config": {"workload": WORKLOAD, "path": "oracle port of the reference CGMN (LEX sweep)",
                   "step": f"{args.ref_sample_iters} CGMN iterations of the solve (a bounded sample)",
                   "value": "extrapolated from the pooled per-iteration time"},
        "cpu_baseline": cpu,
        "e2e": {"value": v, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---- the GPU arm ----------------------------------------------------------------------------------
KERNEL = "sweep_b8_kernel<float> (batched BLOCK8 parity phase)"


def run_batched(args):
    """Config 2: the whole batch in one mixed solve; plain FP64 solves of a sample of it."""
    import torch

    from h3d import workloads as W

    mixed, us = W.config2(precision="mixed", nsrc=args.batch_nsrc)
    out = {"workload": f"config2: config-1 model, {mixed['nsrc']} surface sources x 3/4/5/6 Hz (Ricker 8 Hz) = "
                       f"{mixed['solves']} right-hand sides in one batched solve", "mixed": mixed,
           "roofline": _roofline(mixed["sweep_bytes_total"], mixed["sweep_seconds_total"], mixed["sweep_samples"],
                                 15, KERNEL)}
    if args.batch_fp64_nsrc:
        # plain FP64 of source 0 .. n-1 at 6 Hz (the quickest frequency to converge, so the
        # FP64 time per solve of the whole batch is at least this; the speed-up a lower bound)
        f64, u64 = W.config2(precision="fp64", nsrc=args.batch_fp64_nsrc, freqs=[6.0])
        k6 = len(us) - 1
        a = us[k6][:args.batch_fp64_nsrc]
        d = (a - u64[0]).reshape(a.shape[0], -1)
        out["fp64_sample"] = {"what": f"sources 0-{args.batch_fp64_nsrc - 1} at 6 Hz, plain FP64 batched solve",
                              **f64}
        out["mixed_speedup_per_solve_lower_bound"] = mixed["solves_per_s"] / f64["solves_per_s"]
        out["wavefield_rel_diff_mixed_vs_fp64_sample_max"] = float(
            (d.norm(dim=1) / u64[0].reshape(d.shape).norm(dim=1)).max())
        del u64
    del us
    torch.cuda.empty_cache()
    if not args.skip_batch_mlgmres:
        # the same 256 right-hand sides one at a time by FGMRES + ML_GMRES
        out["mlgmres"] = W.config2_mlgmres(precision="mixed", nsrc=args.batch_nsrc)
        torch.cuda.empty_cache()
    return out


def run_fwi(args):
    """Config 3: the full gradient (mixed); a plain-FP64 gradient of a sample of its pairs; the error
    of both precisions against the FP64 oracle's gradient on the reduced problem."""
    import numpy as np
    import torch

    from h3d import workloads as W

    mixed, g_cgmn = W.config3(precision="mixed", return_grad=True)
    out = {"workload": "config3: 161x161x81 incl. 15-pt PML, 32 sources x 3/4.5/6 Hz, 400 receivers, gradient "
                       "w.r.t. squared slowness at the background model", "mixed": mixed,
           "roofline": _roofline(mixed["sweep_bytes_total"], mixed["sweep_seconds_total"],
                                 mixed["sweep_samples_total"], 15, KERNEL)}
    if args.fwi_fp64_nsrc:
        # plain FP64 gradient of sources 0 .. n-1 at 6 Hz (observed data zero: the solves cost the
        # same; 6 Hz converges quickest, so the speed-up is a lower bound)
        f64 = W.config3(precision="fp64", nsrc=args.fwi_fp64_nsrc, freqs=[6.0], dobs_zero=True)
        out["fp64_sample"] = {"what": f"sources 0-{args.fwi_fp64_nsrc - 1} at 6 Hz, plain FP64", **f64}
        out["mixed_speedup_pairs_per_s_lower_bound"] = mixed["pairs_per_s"] / f64["pairs_per_s"]
    if not args.skip_fwi_mlgmres:
        # the same gradient with every forward and adjoint solve by FGMRES + ML_GMRES (one source
        # at a time, levels built per frequency inside the timed region)
        ml, g_ml = W.config3(precision="mixed", solver="mlgmres", return_grad=True)
        ml["grad_rel_diff_vs_cgmn"] = float((g_ml - g_cgmn).norm() / g_cgmn.norm())
        out["mlgmres"] = ml
    del g_cgmn
    path = os.path.join(ROOT, "tests", "golden", "config3_grad.npz")
    if os.path.exists(path):
        d = dict(np.load(path))
        errs = {}
        for prec in ("mixed",):   # (plain FP64 against the same golden: tests/test_configs_gpu.py)
            prob, _, m0 = W.config3_problem(precision=prec, nsrc=2, freqs=[6.0])
            D0 = torch.zeros(prob.nrec, prob.nsrc, dtype=torch.complex128, device=prob.dev)
            f, g = prob.objective(m0, D0)
            gv = g.permute(2, 1, 0).reshape(-1).cpu().numpy()
            idx = d["g/idx"]
            errs[prec] = {"f_rel_err": abs(f - float(d["f"])) / abs(float(d["f"])),
                          "g_rel_err_samples": float(np.linalg.norm(gv[idx] - d["g/samples"]) /
                                                     np.linalg.norm(d["g/samples"])),
                          "g_rel_err_norm": abs(float(np.linalg.norm(gv)) - float(d["g/norm"])) / float(d["g/norm"])}
        out["error_vs_fp64_oracle_reduced"] = {
            "problem": "161x161x81, sources 0-1, 6 Hz, observed data 0; oracle: PDEfunc restatement over the C "
                       "oracle (LEX sweep, CGMN to the preconditioned tolerance 1e-6, as the reference)", **errs}
    torch.cuda.empty_cache()
    return out


def run_mlgmres(args):
    """Config 1 by FGMRES + ML_GMRES (the reference applications' default solver): mixed (complex64
    V-cycle under complex128 FGMRES) and plain FP64, and the mixed wavefield against the oracle's."""
    import numpy as np
    import torch

    from h3d import workloads as W

    mixed, u = W.config1_mlgmres(precision="mixed", reps=args.mlgmres_reps, return_u=True)
    out = {"workload": "config1 (201x201x101, 6 Hz, one source) by FGMRES (restart 5, tol 1e-6) preconditioned "
                       "by the three-level ML_GMRES V-cycle", "mixed": mixed}
    gpath = os.path.join(ROOT, "tests", "golden", "config1_solve.npz")
    if os.path.exists(gpath):
        d = dict(np.load(gpath))
        v = u.reshape(-1).cpu().numpy()
        out["mixed"]["error_vs_fp64_oracle_samples"] = float(
            np.linalg.norm(v[d["exact/idx"]] - d["exact/samples"]) / np.linalg.norm(d["exact/samples"]))
    del u
    if not args.skip_fp64:
        out["fp64"] = W.config1_mlgmres(precision="fp64", reps=1)
        out["mixed_speedup"] = out["fp64"]["seconds_per_solve"] / mixed["seconds_per_solve"]
    torch.cuda.empty_cache()
    return out


def run_gpu_arm(args, world, rank):
    import ctypes as C

    import torch

    from h3d import _lib as L
    from h3d import build, models, solver

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(dev)
    # one build per node: local rank 0 compiles (the build is also locked and renames its
    # outputs into place), the other ranks wait at the barrier and then load the library
    if int(os.environ.get("LOCAL_RANK", "0")) == 0:
        build.build_lib()
    _barrier(world)
    L.load()
    m = models.config1()
    grid = L.make_grid(m.n_total, m.h, m.npml6)
    N = m.N
    wn = torch.as_tensor(m.wavenumber(), device=dev)
    b = torch.as_tensor(m.point_source(), device=dev)
    opts = solver.make_opts(tol=1e-6, precision="mixed", order=args.order, inner_tol=args.inner_tol,
                            check_every=args.check_every, block=args.block)

    def step():
        return solver.solve(grid, wn, b, opts=opts)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    clk = ClockSampler(dev.index or 0)
    clk.start()
    _barrier(world)
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    infos = []
    for _ in range(args.steps):
        u, info = step()
        infos.append(info)
    e1.record(st)
    torch.cuda.synchronize()
    _barrier(world)
    clocks = clk.stop()
    elapsed = e0.elapsed_time(e1) / 1e3
    elapsed = _max_over_ranks(elapsed, world, dev)
    value = args.steps * world / elapsed

    # end to end through the C ABI with host buffers
    wn_h = torch.as_tensor(m.wavenumber()).pin_memory()
    b_h = torch.as_tensor(m.point_source()).pin_memory()
    u_h = torch.empty_like(b_h).pin_memory()
    lib = L.load()
    _barrier(world)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        inf = L.SolveInfo()
        rc = lib.h3d_solve_host(C.byref(grid), C.c_void_p(wn_h.data_ptr()), C.c_void_p(),
                                C.c_void_p(b_h.data_ptr()), C.c_void_p(u_h.data_ptr()), 1, 1,
                                C.byref(opts), C.byref(inf))
        L.check(rc, "h3d_solve_host")
    t_e2e = _max_over_ranks(time.perf_counter() - t0, world, dev)
    e2e = args.steps * world / t_e2e

    if rank != 0:
        return
    # FP64 solve of the same problem (speed-up and wavefield difference)
    fp64 = None
    if not args.skip_fp64:
        e0.record(st)
        u64, info64 = solver.solve(grid, wn, b, tol=1e-6, precision="fp64", order=args.order,
                                   check_every=args.check_every)
        e1.record(st)
        torch.cuda.synchronize()
        t64 = e0.elapsed_time(e1) / 1e3
        diff = float(((u.to(torch.complex128) - u64).norm() / u64.norm()).item())
        fp64 = {"solves_per_s": 1.0 / t64, "ms_per_solve": 1e3 * t64, "iters": info64["iters"],
                "mixed_speedup": (1.0 / (elapsed / args.steps)) / (1.0 / t64),
                "wavefield_rel_diff_mixed_vs_fp64": diff, "rel_res_true": info64["rel_res_true"]}
        tf = info64["iters"] * (SWEEP_FLOP_PER_PT + CG_FLOP_PER_PT) * N / t64 / 1e12
        fp64["fp64_flop_rate"] = {"achieved_tflops": tf, "peak_tflops": FP64_NOMINAL_TFLOPS,
                                  "frac": tf / FP64_NOMINAL_TFLOPS, "peak_source": "nominal",
                                  "flop_per_pt_iter": SWEEP_FLOP_PER_PT + CG_FLOP_PER_PT}
    else:
        u64 = None
    # error of the wavefields against the FP64 oracle's solution of the same problem (true
    # residual 1.1e-9, tests/golden/config1_solve.npz)
    oracle_err = None
    gpath = os.path.join(ROOT, "tests", "golden", "config1_solve.npz")
    if os.path.exists(gpath):
        import numpy as np

        d = dict(np.load(gpath))
        idx = d["exact/idx"]
        ref = d["exact/samples"]
        oracle_err = {"oracle": "C oracle, COLOUR27 order, true residual %.1e" % float(d["rel_res_true"])}
        for tag, uu in (("mixed", u), ("fp64", u64 if fp64 is not None else None)):
            if uu is None:
                continue
            v = uu.reshape(-1).to(torch.complex128).cpu().numpy()
            oracle_err[tag] = {"samples": float(np.linalg.norm(v[idx] - ref) / np.linalg.norm(ref)),
                               "norm": abs(float(np.linalg.norm(v)) - float(d["exact/norm"])) / float(d["exact/norm"])}
    # roofline of the dominant kernel: the complex64 sweep, sampled live
    sb = sum(i["sweep_bytes"] for i in infos)
    ss = sum(i["sweep_seconds"] for i in infos)
    sn = sum(i["sweep_samples"] for i in infos)
    roof = _roofline(sb, ss, sn, 15, "sweep_b8_kernel<float, 1, 3> (BLOCK8 parity phase, one right-hand side)",
                     args.traffic_per_launch if args.traffic_per_launch is not None
                     else TRAFFIC_PER_LAUNCH.get((args.order, infos[-1]["sweep_variant"])))
    cpu = None
    if not args.skip_cpu:
        ref_iters = args.ref_iters or REF_ITERS_CONFIG1
        c = cpu_sample(m, args.cpu_sample_iters, ref_iters)
        cpu = {"value": c["value"], "unit": "solves/s", "cores": 1, "kind": "port", "cpu_model": _cpu_model(),
               "sample": f"{args.cpu_sample_iters} CGMN iterations of the LEX-ordered oracle port (measured "
                         f"t_iter {c['t_iter_s']:.3f} s) x {ref_iters} reference-order iterations per solve: "
                         "EXTRAPOLATED (the --impl reference line adds a measured full CPU solve of config 0)"}
    launches = int(sum(i["kernel_launches"] for i in infos))
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "c64 inner / f64 refinement",
        "data": "synthetic (seeded config-1 velocity model)",
        "config": {"workload": WORKLOAD, "precision": "mixed", "order": args.order,
                   "inner_tol": args.inner_tol, "l2": "working set > L2 (>= 340 MB per solve)",
                   "parallelism": f"replicas x{world}", "iters": infos[-1]["iters"],
                   "outer": infos[-1]["outer"], "rel_res_true": infos[-1]["rel_res_true"]},
        "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": 24 * N, "d2h_bytes_per_step": 16 * N},
        "roofline": roof, "cpu_baseline": cpu, "gpu_launches": launches, "clocks": clocks, "fp64": fp64,
        "error_vs_fp64_oracle": oracle_err,
    }
    del u, u64
    torch.cuda.empty_cache()
    if not args.skip_mlgmres:
        line["mlgmres"] = run_mlgmres(args)
    if not args.skip_batched:
        line["batched"] = run_batched(args)
    if not args.skip_fwi:
        line["fwi"] = run_fwi(args)
    if args.derive_ref_iters:
        _, info_l = solver.solve(grid, wn, b, tol=1e-6, precision="fp64", order="lex", check_every=25)
        line["ref_iters_derived"] = {"iters": info_l["iters"], "seconds": info_l["seconds"],
                                     "rel_res_true": info_l["rel_res_true"]}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="h3d", choices=["h3d", "reference"])
    ap.add_argument("--inner-tol", type=float, default=1e-4)
    ap.add_argument("--order", default=DEFAULT_ORDER, choices=["colour27", "block8", "block", "lex"])
    ap.add_argument("--block", type=int, nargs=3, default=None,
                    help="fixed block size for BLOCK/BLOCK8 (skips the solver's measured tuning)")
    ap.add_argument("--check-every", type=int, default=25)
    ap.add_argument("--cpu-sample-iters", type=int, default=4)
    ap.add_argument("--ref-sample-iters", type=int, default=2,
                    help="CGMN iterations per timed step of the reference arm")
    ap.add_argument("--ref-iters", type=int, default=None)
    ap.add_argument("--traffic-per-launch", type=float, default=None)
    ap.add_argument("--batch-nsrc", type=int, default=64, help="sources of the config-2 batch (x 4 frequencies)")
    ap.add_argument("--batch-fp64-nsrc", type=int, default=1, help="sources of its FP64 sample (at 6 Hz)")
    ap.add_argument("--fwi-fp64-nsrc", type=int, default=1, help="sources of the FP64 FWI sample (at 6 Hz)")
    ap.add_argument("--skip-fp64", action="store_true")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--skip-batched", action="store_true")
    ap.add_argument("--skip-mlgmres", action="store_true")
    ap.add_argument("--skip-fwi-mlgmres", action="store_true", help="no config-3 gradient by the multigrid solver")
    ap.add_argument("--skip-batch-mlgmres", action="store_true", help="no config-2 solves by the multigrid solver")
    ap.add_argument("--mlgmres-reps", type=int, default=3, help="timed config-1 FGMRES + ML_GMRES solves")
    ap.add_argument("--skip-fwi", action="store_true")
    ap.add_argument("--skip-config0", action="store_true", help="reference arm: no full config-0 CPU solve")
    ap.add_argument("--derive-ref-iters", action="store_true",
                    help="also run the reference-order (LEX) FP64 solve of the headline workload")
    args = ap.parse_args()
    world, rank = _dist_init()
    if args.impl == "reference":
        run_reference_arm(args, world, rank)
    else:
        run_gpu_arm(args, world, rank)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
