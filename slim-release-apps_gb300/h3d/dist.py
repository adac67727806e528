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


def _default_device(group=None):
    """Device of a rank's zero contribution: the current CUDA device under NCCL (which reduces
    CUDA tensors only), else the CPU."""
    if dist.is_available() and dist.is_initialized() and dist.get_backend(group) == "nccl":
        return torch.device("cuda", torch.cuda.current_device())
    return torch.device("cpu")


def distributed_objective(pair_fn: Callable[[Sequence[int]], tuple[float, torch.Tensor]],
                          npairs: int, grad_shape, device=None, scale_by_pairs: bool = True,
                          group=None):
    """Sum over ranks of pair_fn(my pairs) -> (f, g); scaled by 1/npairs like misfit_setup.

    ``pair_fn`` receives the list of pair indices this rank owns and returns its partial
    objective and gradient.  A rank that owns no pairs contributes zeros on ``device``
    (default: the current CUDA device under NCCL, else the CPU).
    """
    world = dist.get_world_size(group) if dist.is_initialized() else 1
    rank = dist.get_rank(group) if dist.is_initialized() else 0
    mine = partition(npairs, world, rank)
    if mine:
        f, g = pair_fn(mine)
    else:
        dev = device if device is not None else _default_device(group)
        f, g = 0.0, torch.zeros(grad_shape, dtype=torch.float64, device=dev)
    buf = torch.cat([torch.tensor([float(f)], dtype=torch.float64, device=g.device), g.reshape(-1).to(torch.float64)])
    buf = global_sum(buf, group)
    c = 1.0 / npairs if scale_by_pairs else 1.0
    return c * float(buf[0]), c * buf[1:].reshape(grad_shape)


def by_frequency(pairs: Sequence[tuple[int, int]]) -> list[tuple[int, list[int]]]:
    """Group (src, freq) pairs by frequency, frequencies and sources ascending: the unit one
    batched solve handles (all owned sources of one frequency as right-hand sides)."""
    out: dict[int, list[int]] = {}
    for s, k in pairs:
        out.setdefault(int(k), []).append(int(s))
    return [(k, sorted(out[k])) for k in sorted(out)]


def pair_objective(evaluate: Callable[[int, list[int]], tuple[float, torch.Tensor]], nsrc: int,
                   nfreq: int) -> Callable[[Sequence[int]], tuple[float, torch.Tensor]]:
    """The pair function of an FWI problem for distributed_objective: pair indices (in the
    order of pairs_of) -> the sum over their frequencies of evaluate(freq index, sources),
    each of which returns the PDEfunc OBJ contribution (f, g) of those sources at that
    frequency (PDEfunc_dist.m:120-164 hands every worker such a (src, freq) subset)."""
    pairs = pairs_of(nsrc, nfreq)

    def fn(mine: Sequence[int]):
        f, g = 0.0, None
        for k, srcs in by_frequency([pairs[i] for i in mine]):
            fk, gk = evaluate(k, srcs)
            f += float(fk)
            g = gk.to(torch.float64).clone() if g is None else g + gk.to(torch.float64)
        return f, g

    return fn


def fwi_objective(problem, v_phys: torch.Tensor, Dobs: torch.Tensor, group=None):
    """misfit_setup's objective over this process group: (1/#pairs) sum over all (src, freq)
    pairs of PDEfunc OBJ, each rank solving its round-robin share of the pairs on its own GPU
    (``problem``: an h3d.fwi.FWIProblem; Dobs: nrec x nsrc*nfreq, column src + nsrc*freq)."""
    nsrc, nfreq = problem.nsrc, len(problem.geom.freqs)

    def evaluate(k, srcs):
        return problem.objective_pairs(v_phys, Dobs, k, srcs)

    shape = tuple(int(n) for n in problem.geom.n)
    return distributed_objective(pair_objective(evaluate, nsrc, nfreq), nsrc * nfreq, shape,
                                 device=problem.dev, group=group)
