"""Multi-rank path shards on CPU: two gloo ranks each take a contiguous path
range, produce its exact limb sums (here from the oracle, standing in for
the GPU partial), merge them with one SUM all-reduce and finalise on the
host.  The merged prices must equal, bit for bit, the finalisation of the
full-range limbs, on every rank; shard ranges must tile the paths.
"""
import os
import socket

import numpy as np
import pytest

from hestonexotics_gb300 import engine as E
from hestonexotics_gb300 import shard as S
from hestonexotics_gb300 import workloads as W


def test_shard_range_tiles_paths():
    for n in (0, 1, 7, 64, 1000, 65537):
        for world in (1, 2, 3, 8):
            rs = [S.shard_range(n, r, world) for r in range(world)]
            assert rs[0][0] == 0 and rs[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(rs, rs[1:]))
            sizes = [hi - lo for lo, hi in rs]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        S.shard_range(10, 2, 2)


def _request():
    reqs, cfg = W.uneven_batch(n_sets=1, seed=5, precision=E.FP64, path_scale=1.0 / 4096)
    rq = reqs[0]
    keep = slice(0, 12)   # a dozen options keep the oracle quick
    o = rq.options
    rq = E.Request(rq.params, rq.S0, E.Options(o.strike[keep], o.T[keep], o.payoff[keep], o.n_paths[keep]),
                   seed=rq.seed, stream=7)
    return rq, cfg


def _oracle_partial(rq, cfg, lo, hi):
    from oracle import oracle as O
    o = rq.options
    _, _, limbs = O.price_paths(rq.params.as_array(), rq.S0, o.strike, o.T, o.payoff.astype(np.uint8), o.n_paths,
                                n_default=cfg.n_paths, step_mode=cfg.step_mode, steps=cfg.steps,
                                steps_per_year=cfg.steps_per_year, seed=rq.seed, stream=rq.stream, path_lo=lo,
                                path_hi=hi)
    return limbs


def _rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rq, cfg = _request()
        price, se = S.price_sharded(rq, cfg, partial=_oracle_partial)
        np.save(os.path.join(out_dir, f"r{rank}.npy"), np.stack([price, se]))
    finally:
        dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("world", [2, 3])
def test_gloo_shards_merge_bit_identical(tmp_path, oracle, world):
    import torch.multiprocessing as mp
    pytest.importorskip("torch.distributed")
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    rq, cfg = _request()
    full = _oracle_partial(rq, cfg, 0, S.max_paths(rq, cfg))
    want = np.stack(E.finalize_limbs(rq.params, rq.S0, rq.options, cfg, full))
    for r in range(world):
        got = np.load(tmp_path / f"r{r}.npy")
        assert np.array_equal(got, want), r
    # and the merged limbs price like the oracle's own finaliser
    p_or, se_or, _ = oracle.price_paths(rq.params.as_array(), rq.S0, rq.options.strike, rq.options.T,
                                        rq.options.payoff.astype(np.uint8), rq.options.n_paths,
                                        n_default=cfg.n_paths, step_mode=cfg.step_mode, steps=cfg.steps,
                                        steps_per_year=cfg.steps_per_year, seed=rq.seed, stream=rq.stream)
    np.testing.assert_allclose(want[0], p_or, rtol=1e-14, atol=1e-14)


def _batch():
    reqs, cfg = W.uneven_batch(n_sets=3, seed=6, precision=E.FP64, path_scale=1.0 / 4096)
    out = []
    for rq in reqs:   # a few options each keep the oracle quick
        o = rq.options
        k = slice(0, 5)
        out.append(E.Request(rq.params, rq.S0, E.Options(o.strike[k], o.T[k], o.payoff[k], o.n_paths[k]),
                             seed=rq.seed, stream=rq.stream))
    return out, cfg


def _oracle_batch_partial(reqs, cfg, rank, world):
    # range `rank` of every request's paths, as hexo_price_batch_partial cuts them
    rows = []
    for rq in reqs:
        lo, hi = S.shard_range(S.max_paths(rq, cfg), rank, world)
        rows.append(_oracle_partial(rq, cfg, lo, hi))
    return np.concatenate(rows)


def _batch_rank_main(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        reqs, cfg = _batch()
        got = S.price_batch_sharded(reqs, cfg, batch_partial=_oracle_batch_partial)
        np.save(os.path.join(out_dir, f"b{rank}.npy"), np.concatenate([np.stack(x) for x in got], axis=1))
    finally:
        dist.destroy_process_group()


def test_gloo_batch_shards_merge_bit_identical(tmp_path, oracle):
    import torch.multiprocessing as mp
    pytest.importorskip("torch.distributed")
    world = 2
    mp.start_processes(_batch_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    reqs, cfg = _batch()
    want = np.concatenate([np.stack(x) for x in S.finalize_batch(reqs, cfg, _oracle_batch_partial(reqs, cfg, 0, 1))],
                          axis=1)
    for r in range(world):
        assert np.array_equal(np.load(tmp_path / f"b{r}.npy"), want), r
    # one rank's share is range r of every request: the two shares add to the whole
    a = _oracle_batch_partial(reqs, cfg, 0, 2)
    b = _oracle_batch_partial(reqs, cfg, 1, 2)
    assert np.array_equal(a + b, _oracle_batch_partial(reqs, cfg, 0, 1))
