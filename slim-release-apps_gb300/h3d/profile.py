"""Run one hot kernel on a benchmark workload, for timing and for profilers.

    python -m h3d.profile --kernel sweep --config 1 --dtype c64 --reps 3
    python -m h3d.profile --kernel mvp   --config 1 --dtype c64 --reps 10

Builds the operator of the chosen seeded workload (config 0: 61^3, config 1:
201 x 201 x 101), runs ``reps`` double sweeps (27-colour order by default) or matvecs
through the C ABI on the current stream, and prints the CUDA-event time per repetition
and the algorithmic bandwidth (matvec N (2 s_c + s_w) bytes, double sweep twice that).
"""
from __future__ import annotations

import argparse
import json

import torch

from . import _lib as L
from . import models, ops


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--kernel", choices=["sweep", "mvp", "mvp_adj", "cgmn"], default="sweep")
    ap.add_argument("--config", type=int, choices=[0, 1], default=1)
    ap.add_argument("--dtype", choices=["c64", "c128"], default="c64")
    ap.add_argument("--order", type=int, default=L.ORDER_COLOUR27)
    ap.add_argument("--block", type=int, nargs=3, default=None)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--nrhs", type=int, default=1)
    a = ap.parse_args(argv)
    m = models.config0() if a.config == 0 else models.config1()
    dev = torch.device("cuda:0")
    grid = (m.n_total, m.h, m.npml6)
    cdt, rdt = (torch.complex64, torch.float32) if a.dtype == "c64" else (torch.complex128, torch.float64)
    wn = torch.as_tensor(m.wavenumber(), device=dev).to(rdt)
    gen = torch.Generator(device=dev).manual_seed(0)
    x = torch.randn(a.nrhs, m.N, dtype=cdt, device=dev, generator=gen)
    if a.kernel == "cgmn":
        # a fixed number of CGMN iterations of the solver (sweeps with precomputed norms)
        from . import solver

        b = torch.as_tensor(m.point_source(), device=dev)
        opts = solver.make_opts(tol=1e-30, maxit=a.reps, precision="fp64" if a.dtype == "c128" else "mixed",
                                order=a.order, max_outer=1, inner_tol=1e-30, check_every=a.reps)
        fn = lambda: solver.solve(grid, wn.double(), b, opts=opts, raise_not_converged=False)
        bytes_per = a.reps * 2 * m.N * (2 * (8 if a.dtype == "c64" else 16) + (4 if a.dtype == "c64" else 8))
    elif a.kernel == "sweep":
        fn = lambda: ops.kacz_sweep(grid, wn, 1.5, x, None, 1, order=a.order, block=a.block)
        bytes_per = 2 * m.N * (2 * (8 if a.dtype == "c64" else 16) * a.nrhs + (4 if a.dtype == "c64" else 8))
    else:
        mode = 2 if a.kernel == "mvp_adj" else 1
        fn = lambda: ops.mvp(grid, wn, x, mode)
        bytes_per = m.N * (2 * (8 if a.dtype == "c64" else 16) * a.nrhs + (4 if a.dtype == "c64" else 8))
    fn()
    torch.cuda.synchronize()
    if a.kernel == "cgmn":
        a.reps = 1
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(a.reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3 / a.reps
    print(json.dumps({"kernel": a.kernel, "config": a.config, "dtype": a.dtype, "order": a.order,
                      "nrhs": a.nrhs, "N": m.N, "ms_per_rep": 1e3 * t, "alg_GBps": bytes_per / t / 1e9}))


if __name__ == "__main__":
    main()
