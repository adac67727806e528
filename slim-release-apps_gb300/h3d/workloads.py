"""The batched and FWI benchmark workloads (seeded synthetic data).

    python -m h3d.workloads --config 2     # 64 sources x 4 frequencies, batched solves
    python -m h3d.workloads --config 3     # FWI gradient, 32 sources x 3 frequencies
    python -m h3d.workloads --config 4     # 48 uneven problems in one batched call
    python -m h3d.workloads --config 1 --solver mlgmres   # config 1 by FGMRES + ML_GMRES
    python -m h3d.workloads --config 2 --solver mlgmres   # the config-2 sources one at a time by it

Each prints one JSON line: throughput (solves/s or gradients/s) with CUDA-event timing on
the launching stream, iteration counts, the worst true residual, and the solver settings.
Config 1 (one source, the headline) by CGMN is bench.py's workload; here it runs by FGMRES with
the ML_GMRES multigrid preconditioner (the reference applications' default solver).
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import time

import numpy as np
import torch

from . import _lib as L
from . import fwi, models, solver
from . import solver as S


def _events():
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def _summary(infos, seconds):
    """Throughput figures of one batched solve: the live sweep roofline (algorithmic bytes of the
    timed double sweeps over their device time) and the iteration counts."""
    sb = sum(i["sweep_bytes"] for i in infos)          # a batch reports its timing in the first entry
    ss = sum(i["sweep_seconds"] for i in infos)
    return {"seconds": seconds, "iters": [i["iters"] for i in infos],
            "rel_res_true_max": max(i["rel_res_true"] for i in infos),
            "sweep_gbs": (sb / ss / 1e9) if ss > 0 else None,
            "sweep_samples": sum(i["sweep_samples"] for i in infos),
            "sweep_bytes_total": sb, "sweep_seconds_total": ss,
            "kernel_launches": int(sum(i["kernel_launches"] for i in infos))}


def config2_problems(freqs=None, nsrc=None, src0=0):
    """64 surface sources x {3,4,5,6} Hz on the config-1 model: one problem per frequency, its
    sources (Ricker-weighted unit impulses) as right-hand sides."""
    m = models.config2()
    dev = torch.device("cuda:0")
    fr = m.meta["freqs"] if freqs is None else np.asarray(freqs)
    wts = models.ricker_weight(fr, 8.0)
    srcs = m.sources[src0:] if nsrc is None else m.sources[src0:src0 + nsrc]
    nx, ny, _ = m.n_total
    probs = []
    for f, wgt in zip(fr, wts):
        wn = torch.as_tensor(m.wavenumber(float(f)), device=dev)
        b = torch.zeros(len(srcs), m.N, dtype=torch.complex128, device=dev)
        for s, (i, j, k) in enumerate(srcs):
            b[s, int(i) + nx * int(j) + nx * ny * int(k)] = complex(wgt)
        probs.append(solver.Problem((m.n_total, m.h, m.npml6), wn, b, 1))
    return m, probs, fr, srcs


def warm_up(probs, opts):
    """Set-up, tuning and graph capture of a batch shape, two iterations only (untimed)."""
    o = solver.make_opts()
    C.pointer(o)[0] = opts
    o.maxit = 2
    solver.solve_batch(probs, opts=o, raise_not_converged=False)
    torch.cuda.synchronize()


def timed_batch(probs, opts):
    e0, e1 = _events()
    e0.record()
    us, infos = solver.solve_batch(probs, opts=opts)
    e1.record()
    torch.cuda.synchronize()
    return us, infos, e0.elapsed_time(e1) / 1e3


def config2(order="block8", precision="mixed", freqs=None, nsrc=None, tol=1e-6, inner_tol=1e-4, warm=True):
    """The config-2 batch (by default all 64 sources x 4 frequencies = 256 right-hand sides) in
    one batched solve: all frequencies and sources iterate together."""
    m, probs, fr, srcs = config2_problems(freqs, nsrc)
    opts = solver.make_opts(tol=tol, precision=precision, order=order, inner_tol=inner_tol)
    if warm:
        warm_up(probs, opts)
    us, infos, t = timed_batch(probs, opts)
    nsolve = len(fr) * len(srcs)
    out = {"workload": "config2", "solves": nsolve, "solves_per_s": nsolve / t, "order": order,
           "precision": precision, "freqs": [float(f) for f in fr], "nsrc": len(srcs)}
    out.update(_summary(infos, t))
    return out, us


def config2_mlgmres(precision="mixed", freqs=None, nsrc=None, tol=1e-6):
    """The config-2 right-hand sides (64 surface sources x 3/4/5/6 Hz, Ricker-weighted) solved one
    at a time by FGMRES + ML_GMRES on the levels of each frequency (built inside the timed
    region).  True residuals against the config-2 operator of the batched CGMN solve."""
    from . import multigrid as MG
    from . import ops

    m = models.config2()
    dev = torch.device("cuda:0")
    fr = m.meta["freqs"] if freqs is None else np.asarray(freqs)
    wts = models.ricker_weight(fr, 8.0)
    srcs = m.sources if nsrc is None else m.sources[:nsrc]
    nx, ny, _ = m.n_total
    grid = (m.n_total, m.h, m.npml6)
    # untimed warm-up: one solve at the first frequency
    lv, R, P = MG.build_levels(m.v, m.h, m.npml6[0], float(fr[0]), "m/s", device=dev)
    b = torch.zeros(m.N, dtype=torch.complex128, device=dev)
    b[int(srcs[0][0]) + nx * int(srcs[0][1]) + nx * ny * int(srcs[0][2])] = 1.0
    MG.solve(lv, R, P, b, tol=tol, precision=precision)
    torch.cuda.synchronize()
    e0, e1 = _events()
    e0.record()
    iters, res = [], []
    for f, wgt in zip(fr, wts):
        lv, R, P = MG.build_levels(m.v, m.h, m.npml6[0], float(f), "m/s", device=dev)
        wn = torch.as_tensor(m.wavenumber(float(f)), device=dev)
        its = []
        for (i, j, k) in srcs:
            b = torch.zeros(m.N, dtype=torch.complex128, device=dev)
            b[int(i) + nx * int(j) + nx * ny * int(k)] = complex(wgt)
            u, info = MG.solve(lv, R, P, b, tol=tol, precision=precision)
            its.append(info["iters"])
            res.append(float((b - ops.mvp(grid, wn, u)).norm() / b.norm()))
        iters.append([min(its), max(its)])
    e1.record()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3
    n = len(srcs) * len(fr)
    return {"workload": "config2", "solver": "mlgmres", "precision": precision, "solves": n, "seconds": t,
            "solves_per_s": n / t, "freqs": [float(x) for x in fr], "nsrc": len(srcs),
            "outer_iters_min_max_per_freq": iters, "rel_res_true_max": max(res),
            "note": "one right-hand side per solve; levels built per frequency inside the timed region; the "
                    "true residuals (FP64 matvec per solve) are inside it too"}


def config3_problem(precision="mixed", order="block8", nsrc=None, freqs=None, solver="cgmn"):
    m = models.config3()
    meta = m.meta
    src = meta["src_xyz"] if nsrc is None else meta["src_xyz"][:nsrc]
    geom = fwi.Geometry(o=(0.0, 0.0, 0.0), d=m.h, n=m.n_phys, npml6=m.npml6, src_xyz=src,
                        rec_xyz=meta["rec_xyz"], freqs=meta["freqs"] if freqs is None else np.asarray(freqs),
                        f0=meta["f0"], t0=0.0, unit="s2/m2")
    prob = fwi.FWIProblem(geom, fwi.FWIConfig(tol=1e-6, precision=precision, order=order, solver=solver))
    m_true = torch.as_tensor(m.v ** -2.0, device=prob.dev)
    m0 = torch.as_tensor(meta["v0"] ** -2.0, device=prob.dev)
    return prob, m_true, m0


def config3(precision="mixed", order="block8", nsrc=None, freqs=None, solver="cgmn", return_grad=False,
            dobs_zero=False):
    """FWI gradient w.r.t. squared slowness: 32 jittered surface sources, 400 receivers,
    3 / 4.5 / 6 Hz on 161 x 161 x 81 (15-point PML); observed data modelled on the true
    model, gradient at the background model through the autograd function.  dobs_zero: observed
    data zero instead (no modelling run; the solves cost the same, the gradient differs)."""
    prob, m_true, m0 = config3_problem(precision, order, nsrc, freqs, solver)
    if dobs_zero:
        Dobs = torch.zeros(prob.nrec, prob.nsrc * len(prob.geom.freqs), dtype=torch.complex128, device=prob.dev)
    else:
        Dobs = prob.forward_model(m_true)
    if solver == "cgmn":   # the adjoint batch's set-up, tuning and capture, untimed
        gen = torch.Generator(device=prob.dev).manual_seed(5)
        jobs = [S.Problem(prob.g, prob._wavenumbers(m0, float(prob.geom.freqs[k]))[0],
                          torch.randn(len(srcs), prob.N, dtype=torch.complex128, device=prob.dev, generator=gen), 2)
                for k, srcs in prob._units()]
        warm_up(jobs, prob._opts())
    torch.cuda.synchronize()
    m = m0.clone().requires_grad_(True)
    prob.last_infos = []
    e0, e1 = _events()
    e0.record()
    f = fwi.fwi_objective(m, prob, Dobs)
    f.backward()
    e1.record()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3
    pairs = prob.nsrc * len(prob.geom.freqs)
    out = {"workload": "config3", "seconds": t, "grads_per_s": 1.0 / t, "pairs_per_s": pairs / t,
           "f": float(f.item()), "grad_norm": float(m.grad.norm().item()), "order": order,
           "precision": precision, "solver": solver, "nsrc": prob.nsrc, "freqs": [float(x) for x in prob.geom.freqs],
           "solves": len(prob.last_infos), "iters": [i["iters"] for i in prob.last_infos],
           "stored_wavefields": prob.wavefield_bytes() <= prob.cfg.hbm_budget_bytes}
    sw = [i for i in prob.last_infos if i.get("sweep_seconds")]
    ss, sb = sum(i["sweep_seconds"] for i in sw), sum(i["sweep_bytes"] for i in sw)
    out["sweep_gbs"] = sb / ss / 1e9 if ss > 0 else None
    out.update(sweep_bytes_total=sb, sweep_seconds_total=ss,
               sweep_samples_total=sum(i.get("sweep_samples", 0) for i in sw))
    return (out, m.grad.detach()) if return_grad else out


def config4_problems(nprob=48, first=0):
    probs_m = models.config4(nprob=first + nprob)[first:]
    dev = torch.device("cuda:0")
    probs = []
    for m in probs_m:
        nx, ny, _ = m.n_total
        wn = torch.as_tensor(m.wavenumber(), device=dev)
        b = torch.zeros(len(m.sources), m.N, dtype=torch.complex128, device=dev)
        for s, (i, j, k) in enumerate(m.sources):
            b[s, int(i) + nx * int(j) + nx * ny * int(k)] = 1.0
        probs.append(solver.Problem((m.n_total, m.h, m.npml6), wn, b, 1))
    return probs_m, probs


def config4(precision="mixed", order="block8", nprob=48, fp64_problems=None):
    """48 problems with seeded sizes in [64, 192] per axis, 12.5 Hz, 1-16 sources each: one
    batched solve of all of them, then (fp64_problems > 0) the first fp64_problems of them solved
    one by one in plain FP64, the comparison the workload asks for."""
    probs_m, probs = config4_problems(nprob)
    opts = solver.make_opts(tol=1e-6, precision=precision, order=order)
    warm_up(probs, opts)
    us, infos, t = timed_batch(probs, opts)
    nsolve = sum(len(m.sources) for m in probs_m)
    pts = sum(int(np.prod(m.n_total)) * len(m.sources) for m in probs_m)
    out = {"workload": "config4", "problems": len(probs), "solves": nsolve, "solves_per_s": nsolve / t,
           "grid_points_x_rhs": pts, "order": order, "precision": precision}
    out.update(_summary(infos, t))
    if fp64_problems:
        k = min(int(fp64_problems), len(probs))
        o64 = solver.make_opts(tol=1e-6, precision="fp64", order=order)
        t64, n64, pts64, errs = 0.0, 0, 0, []
        for q in range(k):
            e0, e1 = _events()
            e0.record()
            u64, info64 = solver.solve(probs[q].grid, probs[q].wn, probs[q].b, opts=o64)
            e1.record()
            torch.cuda.synchronize()
            t64 += e0.elapsed_time(e1) / 1e3
            n64 += probs[q].b.shape[0]
            pts64 += int(np.prod(probs_m[q].n_total)) * len(probs_m[q].sources)
            d = (us[q] - u64).reshape(probs[q].b.shape[0], -1)
            errs.append(float((d.norm(dim=1) / u64.reshape(d.shape).norm(dim=1)).max()))
        out["fp64_one_by_one"] = {"problems": k, "solves": n64, "grid_points_x_rhs": pts64, "seconds": t64,
                                  "solves_per_s": n64 / t64,
                                  "mixed_batched_speedup_points_per_s": (pts / t) / (pts64 / t64),
                                  "wavefield_rel_diff_mixed_vs_fp64_max": max(errs)}
    return out


def config1_mlgmres(precision="mixed", reps=3, tol=1e-6, return_u=False):
    """Config 1 (201 x 201 x 101 with a 20-point PML, 6 Hz, one surface source) by FGMRES +
    ML_GMRES: seconds per solve over `reps` solves after an untimed one (CUDA events on the
    launching stream), outer iterations, true residual, launches and host waits per solve."""
    from . import multigrid as MG
    from . import ops

    m = models.config1()
    dev = torch.device("cuda")
    t0 = time.time()
    lv, R, P = MG.build_levels(m.v, m.h, m.npml6[0], m.freq, "m/s", device=dev)
    t_build = time.time() - t0
    b = torch.as_tensor(m.point_source(), device=dev)
    MG.solve(lv, R, P, b, tol=tol, precision=precision)
    torch.cuda.synchronize()
    e0, e1 = _events()
    e0.record()
    infos = []
    for _ in range(reps):
        u, info = MG.solve(lv, R, P, b, tol=tol, precision=precision)
        infos.append(info)
    e1.record()
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) / 1e3 / reps
    r = b - ops.mvp(lv[0].grid, lv[0].wn, u)
    out = {"workload": "config1", "solver": "mlgmres", "precision": precision, "seconds_per_solve": sec,
            "solves_per_s": 1.0 / sec, "outer_iters": infos[-1]["iters"],
            "rel_res_true": float(r.norm() / b.norm()), "converged": infos[-1]["converged"],
            "kernel_launches": infos[-1]["kernel_launches"], "host_syncs": infos[-1]["host_syncs"],
            "levels": [list(l.nt) for l in lv], "level_build_s": t_build}
    return (out, u) if return_u else out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", type=int, choices=[1, 2, 3, 4], required=True)
    ap.add_argument("--order", default=None)
    ap.add_argument("--precision", default="mixed")
    ap.add_argument("--nsrc", type=int, default=None)
    ap.add_argument("--freqs", type=float, nargs="*", default=None)
    ap.add_argument("--nprob", type=int, default=48)
    ap.add_argument("--solver", default="cgmn", choices=["cgmn", "mlgmres"])
    ap.add_argument("--fp64-problems", type=int, default=0)
    ap.add_argument("--reps", type=int, default=3, help="config 1: timed solves after the untimed one")
    a = ap.parse_args(argv)
    t0 = time.time()
    if a.config == 1:
        if a.solver != "mlgmres":
            raise SystemExit("config 1 by CGMN is bench.py's workload; --config 1 takes --solver mlgmres")
        out = config1_mlgmres(precision=a.precision, reps=a.reps)
    elif a.config == 2 and a.solver == "mlgmres":
        out = config2_mlgmres(precision=a.precision, freqs=a.freqs, nsrc=a.nsrc)
    elif a.config == 2:
        out, _ = config2(order=a.order or "block8", precision=a.precision, freqs=a.freqs, nsrc=a.nsrc)
    elif a.config == 3:
        out = config3(precision=a.precision, order=a.order or "block8", nsrc=a.nsrc, freqs=a.freqs,
                      solver=a.solver)
    else:
        out = config4(precision=a.precision, order=a.order or "block8", nprob=a.nprob,
                      fp64_problems=a.fp64_problems)
    out["wall_s"] = time.time() - t0
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
