"""Multi-rank (src,freq) sharding on CPU ranks with the gloo backend (world size 2).

Each rank owns a round-robin share of the pairs, computes its partial objective and
gradient, and one all-reduce sums them (PDEfunc_dist.m:212-215), then the 1/#pairs
scaling of misfit_setup.m:186,225-227 applies.  The per-pair work here is a seeded
stand-in function, so the test needs no GPU; it checks the partition, the sum and the
scaling against a single-process evaluation, and that a rank with no pairs still joins.
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


def test_partition_covers_pairs_once():
    from h3d import dist as D

    for world in (1, 2, 3, 8):
        got = sorted(sum((D.partition(96, world, r) for r in range(world)), []))
        assert got == list(range(96))
    assert D.pairs_of(2, 3)[:3] == [(0, 0), (1, 0), (0, 1)]
