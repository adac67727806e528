"""Data-parallel FWI over (source, frequency) pairs: replicas plus one sum.

The reference distributes the independent (src,freq) solves over MATLAB workers and sums
the objective and gradient with ``pSPOT.utils.global_sum`` (PDEfunc_dist.m:188-232); the
objective handle of misfit_setup then scales both by ``c = 1/#pairs``
(misfit_setup.m:186,225-227).  Here every rank owns a round-robin share of the pairs,
computes its partial (f, g) on its own GPU, and one all-reduce (gloo or NCCL through
torch.distributed) forms the sums.  There is no other exchange: the path shards
without a data-path collective inside the solves.
"""
from __future__ import annotations

from typing import Callable, Sequence

import torch
import torch.distributed as dist


def partition(npairs: int, world: int, rank: int) -> list[int]:
    """Round-robin share of the pair indices 0..npairs-1 owned by ``rank``."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad world/rank")
    return list(range(rank, npairs, world))


def pairs_of(nsrc: int, nfreq: int) -> list[tuple[int, int]]:
    """(src, freq) pairs in the reference's column order (src fastest, PDEfunc.m:341)."""
    return [(s, k) for k in range(nfreq) for s in range(nsrc)]


def global_sum(t: torch.Tensor, group=None) -> torch.Tensor:
    """pSPOT.utils.global_sum: the elementwise sum over ranks (identity without a group)."""
    if dist.is_available() and dist.is_initialized():
        t = t.clone()
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t


def distributed_objective(pair_fn: Callable[[Sequence[int]], tuple[float, torch.Tensor]],
                          npairs: int, grad_shape, device=None, scale_by_pairs: bool = True,
                          group=None):
    """Sum over ranks of pair_fn(my pairs) -> (f, g); scaled by 1/npairs like misfit_setup.

    ``pair_fn`` receives the list of pair indices this rank owns and returns its partial
    objective and gradient (zero for an empty list).
    """
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    mine = partition(npairs, world, rank)
    if mine:
        f, g = pair_fn(mine)
    else:
        f, g = 0.0, torch.zeros(grad_shape, dtype=torch.float64, device=device)
    buf = torch.cat([torch.tensor([float(f)], dtype=torch.float64, device=g.device), g.reshape(-1).to(torch.float64)])
    buf = global_sum(buf, group)
    c = 1.0 / npairs if scale_by_pairs else 1.0
    return c * float(buf[0]), c * buf[1:].reshape(grad_shape)
