"""The batched and FWI benchmark workloads (seeded synthetic data).

    python -m h3d.workloads --config 2     # 64 sources x 4 frequencies, batched solves
    python -m h3d.workloads --config 3     # FWI gradient, 32 sources x 3 frequencies
    python -m h3d.workloads --config 4     # 48 uneven problems in one batched call

Each prints one JSON line: throughput (solves/s or gradients/s) with CUDA-event timing on
the launching stream, iteration counts, the worst true residual, and the solver settings.
Config 1 (one source, the headline) is bench.py's workload.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

from . import _lib as L
from . import fwi, models, solver


def _events():
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def config2(order="block8", precision="mixed", freqs=None, nsrc=None, tol=1e-6, inner_tol=1e-4):
    """64 surface sources x {3,4,5,6} Hz on the config-1 model: one problem per frequency,
    the sources of a frequency as right-hand sides of one batched solve."""
    m = models.config2()
    dev = torch.device("cuda:0")
    fr = m.meta["freqs"] if freqs is None else np.asarray(freqs)
    wts = models.ricker_weight(fr, 8.0)
    srcs = m.sources if nsrc is None else m.sources[:nsrc]
    nx, ny, _ = m.n_total
    probs = []
    for f, wgt in zip(fr, wts):
        wn = torch.as_tensor(m.wavenumber(float(f)), device=dev)
        b = torch.zeros(len(srcs), m.N, dtype=torch.complex128, device=dev)
        for s, (i, j, k) in enumerate(srcs):
            b[s, int(i) + nx * int(j) + nx * ny * int(k)] = complex(wgt)
        probs.append(solver.Problem((m.n_total, m.h, m.npml6), wn, b, 1))
    opts = solver.make_opts(tol=tol, precision=precision, order=order, inner_tol=inner_tol)
    solver.solve_batch(probs[:1], opts=opts)            # warm-up (autotuner, graphs)
    torch.cuda.synchronize()
    e0, e1 = _events()
    e0.record()
    us, infos = solver.solve_batch(probs, opts=opts)
    e1.record()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3
    nsolve = len(fr) * len(srcs)
    return {"workload": "config2", "solves": nsolve, "seconds": t, "solves_per_s": nsolve / t,
            "order": order, "precision": precision, "iters": [i["iters"] for i in infos],
            "rel_res_true_max": max(i["rel_res_true"] for i in infos), "freqs": [float(f) for f in fr],
            "nsrc": len(srcs)}


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


def config3(precision="mixed", order="block8", nsrc=None, freqs=None, solver="cgmn"):
    """FWI gradient w.r.t. squared slowness: 32 jittered surface sources, 400 receivers,
    3 / 4.5 / 6 Hz on 161 x 161 x 81 (15-point PML); observed data modelled on the true
    model, gradient at the background model through the autograd function."""
    prob, m_true, m0 = config3_problem(precision, order, nsrc, freqs, solver)
    Dobs = prob.forward_model(m_true)
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
    return {"workload": "config3", "seconds": t, "grads_per_s": 1.0 / t, "pairs_per_s": pairs / t,
            "f": float(f.item()), "grad_norm": float(m.grad.norm().item()), "order": order,
            "precision": precision, "solver": solver, "nsrc": prob.nsrc, "freqs": [float(x) for x in prob.geom.freqs],
            "solves": len(prob.last_infos), "iters": [i["iters"] for i in prob.last_infos],
            "stored_wavefields": prob.wavefield_bytes() <= prob.cfg.hbm_budget_bytes}


def config4(precision="mixed", order="block8", nprob=48):
    """48 problems with seeded sizes in [64, 192] per axis, 12.5 Hz, 1-16 sources each,
    solved in one batched call."""
    probs_m = models.config4(nprob=nprob)
    dev = torch.device("cuda:0")
    probs = []
    nsolve = 0
    for m in probs_m:
        nx, ny, _ = m.n_total
        wn = torch.as_tensor(m.wavenumber(), device=dev)
        b = torch.zeros(len(m.sources), m.N, dtype=torch.complex128, device=dev)
        for s, (i, j, k) in enumerate(m.sources):
            b[s, int(i) + nx * int(j) + nx * ny * int(k)] = 1.0
        probs.append(solver.Problem((m.n_total, m.h, m.npml6), wn, b, 1))
        nsolve += len(m.sources)
    opts = solver.make_opts(tol=1e-6, precision=precision, order=order)
    e0, e1 = _events()
    e0.record()
    us, infos = solver.solve_batch(probs, opts=opts)
    e1.record()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3
    pts = sum(int(np.prod(m.n_total)) * len(m.sources) for m in probs_m)
    return {"workload": "config4", "problems": nprob, "solves": nsolve, "seconds": t,
            "solves_per_s": nsolve / t, "grid_points_x_rhs": pts, "order": order, "precision": precision,
            "rel_res_true_max": max(i["rel_res_true"] for i in infos)}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--config", type=int, choices=[2, 3, 4], required=True)
    ap.add_argument("--order", default=None)
    ap.add_argument("--precision", default="mixed")
    ap.add_argument("--nsrc", type=int, default=None)
    ap.add_argument("--freqs", type=float, nargs="*", default=None)
    ap.add_argument("--nprob", type=int, default=48)
    ap.add_argument("--solver", default="cgmn", choices=["cgmn", "mlgmres"])
    a = ap.parse_args(argv)
    t0 = time.time()
    if a.config == 2:
        out = config2(order=a.order or "block8", precision=a.precision, freqs=a.freqs, nsrc=a.nsrc)
    elif a.config == 3:
        out = config3(precision=a.precision, order=a.order or "block8", nsrc=a.nsrc, freqs=a.freqs,
                      solver=a.solver)
    else:
        out = config4(precision=a.precision, order=a.order or "block8", nprob=a.nprob)
    out["wall_s"] = time.time() - t0
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
