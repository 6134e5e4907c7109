"""Path-range shards across ranks, merged exactly.

The paths of one request are independent (path k draws only from the
stream seeded {seed + k, stream, 0, 0}), so a request splits into contiguous path ranges, one per
rank, with no exchange during simulation.  Each rank produces the exact
integer limb sums of its range (``Engine.partial``, hexo_price_partial); a
single SUM all-reduce of those integers and the host finaliser
(hexo_finalize_limbs) give every rank prices bit-identical to one launch on
one GPU.  The reference itself has no multi-device path: its
HSimulation::price splits paths across host threads and adds the threads'
float sums (src/HSimulation.tpp:10-51); the integer limbs are what make the
split result independent of the number of shards.

The all-reduce is the only collective, one per call, of n_options * 6
integers.  A whole batch shards the same way in one launch per rank
(``price_batch_sharded``): range `rank` of every request, one all-reduce of
all requests' limbs.
"""
from __future__ import annotations

from typing import Callable, Sequence

import numpy as np

from . import engine as E


def shard_range(n_paths: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous, balanced [lo, hi) of n_paths for rank of world."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(int(n_paths), world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def max_paths(request: E.Request, cfg: E.Config) -> int:
    n = request.options.n_paths.astype(np.uint64)
    n = np.where(n == 0, np.uint64(cfg.n_paths), n)
    return int(n.max()) if len(n) else 0


def _all_reduce_sum(limbs: np.ndarray, group=None) -> np.ndarray:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return limbs
    backend = dist.get_backend(group)
    dev = torch.device("cuda", torch.cuda.current_device()) if backend == "nccl" else torch.device("cpu")
    # limb sums stay below 2^63 (25-bit limbs, fewer than 2^38 paths per option)
    t = torch.from_numpy(limbs.astype(np.int64)).to(dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t.cpu().numpy().astype(np.uint64)


def price_sharded(request: E.Request, cfg: E.Config, *, rank: int | None = None, world: int | None = None,
                  partial: Callable | None = None, engine: E.Engine | None = None, group=None):
    """Prices one request with its paths split over the ranks of the default
    process group (or the given rank/world).  ``partial(request, cfg, lo, hi)``
    returns the [n_options, 6] uint64 limbs of paths [lo, hi); by default
    the engine's GPU partial.  Returns (price, stderr), identical on every rank
    and identical bit for bit to pricing the request in one launch."""
    import torch.distributed as dist
    if rank is None or world is None:
        if dist.is_available() and dist.is_initialized():
            rank, world = dist.get_rank(group), dist.get_world_size(group)
        else:
            rank, world = 0, 1
    if partial is None:
        if engine is None:
            raise ValueError("pass the engine (or a partial function)")

        def partial(rq, c, lo, hi):
            return engine.partial(rq.params, rq.S0, rq.options, c, lo, hi)
    lo, hi = shard_range(max_paths(request, cfg), rank, world)
    limbs = np.ascontiguousarray(partial(request, cfg, lo, hi), dtype=np.uint64).reshape(len(request.options), 6)
    total = _all_reduce_sum(limbs, group)
    return E.finalize_limbs(request.params, request.S0, request.options, cfg, total)


def finalize_batch(requests: Sequence[E.Request], cfg: E.Config, limbs: np.ndarray):
    """Prices and standard errors of every request from the batch's merged
    limbs (options of all requests in order): [(price, stderr)] per request."""
    out, row = [], 0
    for rq in requests:
        n = len(rq.options)
        out.append(E.finalize_limbs(rq.params, rq.S0, rq.options, cfg, limbs[row:row + n]))
        row += n
    return out


def price_batch_sharded(requests: Sequence[E.Request], cfg: E.Config, *, rank: int | None = None,
                        world: int | None = None, batch_partial: Callable | None = None,
                        engine: E.Engine | None = None, group=None):
    """Prices a whole batch with every request's paths split over the ranks:
    each rank runs one persistent launch over range `rank` of every request
    (``Engine.batch_partial``, hexo_price_batch_partial), then one SUM
    all-reduce of all requests' limbs and the host finaliser give every rank
    the prices of one launch on one GPU, bit for bit.  ``batch_partial(requests,
    cfg, rank, world)`` returns the [options of all requests, 6] uint64 limbs of
    the rank's share; by default the engine's GPU launch."""
    import torch.distributed as dist
    if rank is None or world is None:
        if dist.is_available() and dist.is_initialized():
            rank, world = dist.get_rank(group), dist.get_world_size(group)
        else:
            rank, world = 0, 1
    if batch_partial is None:
        if engine is None:
            raise ValueError("pass the engine (or a batch_partial function)")
        batch_partial = engine.batch_partial
    n = sum(len(rq.options) for rq in requests)
    limbs = np.ascontiguousarray(batch_partial(requests, cfg, rank, world), dtype=np.uint64).reshape(n, 6)
    return finalize_batch(requests, cfg, _all_reduce_sum(limbs, group))
