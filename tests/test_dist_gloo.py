"""Multi-rank (src,freq) sharding on CPU ranks with the gloo backend (world size 2).

Each rank owns a round-robin share of the pairs, computes its partial objective and
gradient, and one all-reduce sums them (PDEfunc_dist.m:212-215), then the 1/#pairs
scaling of misfit_setup.m:186,225-227 applies.  Two kinds of per-pair work, both on CPU:
a seeded stand-in function (the partition, the sum, the scaling, and a rank with no pairs),
and the real FWI wiring of h3d.dist (pairs grouped by frequency, PDEfunc OBJ per
(sources, frequency) subset) with the oracle's PDEfunc restatement as the evaluator, against
a serial evaluation of all pairs.
"""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _pair_fn_factory(shape):
    def fn(pairs):
        f = 0.0
        g = torch.zeros(shape, dtype=torch.float64)
        for p in pairs:
            rng = np.random.default_rng(100 + p)
            f += float(rng.random())
            g += torch.as_tensor(rng.standard_normal(shape))
        return f, g
    return fn


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, npairs, shape, out):
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, os.path.join(root, "slim-release-apps_gb300"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from h3d import dist as D

        f, g = D.distributed_objective(_pair_fn_factory(shape), npairs, shape)
        out[rank] = (f, g.numpy())
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("npairs", [5, 1])
def test_two_rank_sum_matches_serial(npairs):
    shape = (4, 3, 2)
    ctx = mp.get_context("spawn")      # no fork: earlier tests leave OpenMP threads running
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, npairs, shape, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    f_ser, g_ser = _pair_fn_factory(shape)(list(range(npairs)))
    for r in range(2):
        f, g = out[r]
        assert abs(f - f_ser / npairs) <= 1e-14
        np.testing.assert_allclose(g, g_ser.numpy() / npairs, rtol=0, atol=1e-14)


def _fwi_case():
    """A small FWI problem for the oracle's PDEfunc: 2 sources x 2 frequencies, 6 receivers."""
    n, d, npml = (10, 9, 8), (25.0, 25.0, 25.0), (3, 3, 3, 3, 3, 3)
    rng = np.random.default_rng(23)
    vel = 1500.0 + 1000.0 * rng.random(n)
    model = {"o": (0.0, 0.0, 0.0), "d": d, "n": n, "npml6": npml, "unit": "s2/m2", "f0": 8.0, "t0": 0.0}
    src = np.array([[95.0, 80.0, 40.0], [140.0, 130.0, 45.0]])
    rec = np.array([[x, y, 25.0] for x in (50.0, 110.0, 170.0) for y in (60.0, 150.0)])
    amp = np.array([1.0, 0.6 + 0.3j])
    freqs = np.array([4.0, 6.0])
    m = (vel ** -2).reshape(-1, order="F")
    D = rng.standard_normal((len(rec), 4)) * 1e-3 + 1j * rng.standard_normal((len(rec), 4)) * 1e-3
    return model, m, src, amp, rec, freqs, D


def _oracle_evaluate(k, srcs):
    from oracle import h3d_oracle as O
    from oracle import slim_ref

    model, m, src, amp, rec, freqs, D = _fwi_case()
    cols = [s + len(src) * k for s in srcs]
    f, g = slim_ref.pdefunc("obj", m, model, src[srcs], amp[srcs], rec, freqs[k:k + 1], Dobs=D[:, cols],
                            tol=1e-9, maxit=20000, order=O.ORDER_COLOUR27, nthreads=1)
    return f, torch.as_tensor(g.reshape(model["n"], order="F").copy())


def _fwi_worker(rank, world, port, out):
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "slim-release-apps_gb300")):
        sys.path.insert(0, p)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from h3d import dist as D

        model, m, src, amp, rec, freqs, Dobs = _fwi_case()
        fn = D.pair_objective(_oracle_evaluate, len(src), len(freqs))
        f, g = D.distributed_objective(fn, len(src) * len(freqs), model["n"])
        out[rank] = (f, g.numpy())
    finally:
        dist.destroy_process_group()


def test_two_rank_fwi_objective_with_oracle_pairs():
    """h3d.dist's FWI wiring on two gloo ranks, the oracle's PDEfunc OBJ per (sources,
    frequency) subset: equal to (1/#pairs) PDEfunc OBJ over all pairs in one process."""
    from oracle import h3d_oracle as O
    from oracle import slim_ref

    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_fwi_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(300)
        assert p.exitcode == 0
    model, m, src, amp, rec, freqs, D = _fwi_case()
    f_ser, g_ser = slim_ref.pdefunc("obj", m, model, src, amp, rec, freqs, Dobs=D, tol=1e-9, maxit=20000,
                                    order=O.ORDER_COLOUR27, nthreads=1)
    npairs = len(src) * len(freqs)
    g_ser = g_ser.reshape(model["n"], order="F") / npairs
    for r in range(2):
        f, g = out[r]
        assert abs(f - f_ser / npairs) <= 1e-12 * abs(f_ser)
        np.testing.assert_allclose(g, g_ser, rtol=0, atol=1e-12 * np.max(np.abs(g_ser)))


def test_pairs_group_by_frequency():
    from h3d import dist as D

    pairs = D.pairs_of(3, 2)
    assert D.by_frequency([pairs[i] for i in (5, 0, 2, 3)]) == [(0, [0, 2]), (1, [0, 2])]


def test_partition_covers_pairs_once():
    from h3d import dist as D

    for world in (1, 2, 3, 8):
        got = sorted(sum((D.partition(96, world, r) for r in range(world)), []))
        assert got == list(range(96))
    assert D.pairs_of(2, 3)[:3] == [(0, 0), (1, 0), (0, 1)]
