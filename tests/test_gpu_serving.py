"""Serving loop (hexo_server_*): continuous batching must not change results.

A request priced through the server, batched with whatever else is queued
and split into path blocks that run in different launches, gives
bit-identical prices and standard errors to the same request priced alone
with hexo_price_batch (each path draws from its own stream, sums are exact
integers and a request's running sums stay on the device between its
blocks).  Admission: a request that can never fit the device-memory cap
fails with HEXO_ERR_ADMISSION; requests that fit only one at a time are
queued and all complete.
"""
import threading
import time

import numpy as np
import pytest

from hestonexotics_gb300 import engine as E
from hestonexotics_gb300 import workloads as W
from hestonexotics_gb300._lib import HEXO_ERR_ADMISSION, HEXO_ERR_NOT_FOUND, HexoError

pytestmark = pytest.mark.gpu


def small_requests(n=8, precision=E.FP32):
    reqs, cfg = W.uneven_batch(n_sets=n, seed=11, precision=precision, path_scale=1.0 / 256)
    return reqs, cfg


@pytest.mark.parametrize("precision", [E.FP32, E.FP64])
def test_mixed_equals_alone(engine, precision):
    reqs, cfg = small_requests(precision=precision)
    alone = [engine.price_batch([rq], cfg)[0] for rq in reqs]
    with engine.server(cfg, max_batch_requests=3, max_inflight=2) as srv:
        tickets = [srv.submit(rq) for rq in reqs]
        mixed = [srv.wait(t) for t in tickets]
        st = srv.stats()
    for (pa, sa), (pm, sm) in zip(alone, mixed):
        assert np.array_equal(pa, pm) and np.array_equal(sa, sm)
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["batches"] >= 3
    assert 0 < st["p50_ms"] <= st["p99_ms"]


@pytest.mark.parametrize("precision", [E.FP32, E.FP64])
def test_blocks_across_launches_equal_alone(engine, precision):
    # a small launch budget cuts every request into several path blocks that
    # continue across launches (and across the server's streams)
    reqs, cfg = small_requests(n=6, precision=precision)
    alone = [engine.price_batch([rq], cfg)[0] for rq in reqs]
    with engine.server(cfg, max_batch_requests=4, max_inflight=3, launch_path_steps=1 << 21) as srv:
        tickets = [srv.submit(rq) for rq in reqs]
        got = [srv.wait(t) for t in tickets]
        st = srv.stats()
    for (pa, sa), (pm, sm) in zip(alone, got):
        assert np.array_equal(pa, pm) and np.array_equal(sa, sm)
    assert st["chunks"] >= 2 * len(reqs) and st["completed"] == len(reqs)
    # and the same requests, never split: the same bits again
    with engine.server(cfg, launch_path_steps=(1 << 64) - 1) as srv:
        whole = [srv.wait(srv.submit(rq)) for rq in reqs]
        st = srv.stats()
    assert st["chunks"] == len(reqs)
    for (pa, sa), (pm, sm) in zip(alone, whole):
        assert np.array_equal(pa, pm) and np.array_equal(sa, sm)


def test_large_request_does_not_hold_small_ones(engine):
    # one request much larger than the launch budget, then small ones: the
    # small ones finish in launches that run between the large one's blocks
    reqs, cfg = small_requests(n=5)
    big = W.uneven_batch(n_sets=1, seed=12, precision=E.FP32, path_scale=1.0 / 4)[0][0]
    want_big = engine.price_batch([big], cfg)[0]
    done_order = []
    with engine.server(cfg, max_batch_requests=8, max_inflight=2, launch_path_steps=1 << 26) as srv:
        tb = srv.submit(big)
        ts = [srv.submit(rq) for rq in reqs]
        pending = {tb: "big", **{t: k for k, t in enumerate(ts)}}
        while pending:
            for t in list(pending):
                if srv.poll(t):
                    done_order.append(pending.pop(t))
            time.sleep(0.0005)
        st = srv.stats()
    assert done_order[-1] == "big", done_order
    assert st["chunks"] > len(reqs) + 1
    with engine.server(cfg) as srv:
        p, se = srv.wait(srv.submit(big))
    assert np.array_equal(p, want_big[0]) and np.array_equal(se, want_big[1])


def test_order_and_threads_do_not_matter(engine):
    reqs, cfg = small_requests(n=6)
    alone = [engine.price_batch([rq], cfg)[0] for rq in reqs]
    out = [None] * len(reqs)
    with engine.server(cfg, max_batch_requests=64, max_inflight=3) as srv:
        def worker(idx):
            for i in idx:
                out[i] = srv.wait(srv.submit(reqs[i]))
        ths = [threading.Thread(target=worker, args=(list(range(len(reqs)))[k::3][::-1],)) for k in range(3)]
        for t in ths:
            t.start()
        for t in ths:
            t.join()
    for (pa, sa), (pm, sm) in zip(alone, out):
        assert np.array_equal(pa, pm) and np.array_equal(sa, sm)


def test_admission_by_memory_cap(engine):
    reqs, cfg = small_requests(n=4)
    big = reqs[0]
    small = E.Request(big.params, big.S0, E.Options(np.array([100.0]), np.array([0.5]), E.ASIAN,
                                                   np.array([4096], dtype=np.uint64)), seed=5)
    want = engine.price_batch([small], cfg)[0]
    # room for one small request at a time, never for the large chain
    with engine.server(cfg, mem_cap_bytes=256 << 10, max_inflight=2) as srv:
        tb = srv.submit(big)
        ts = [srv.submit(small) for _ in range(4)]
        with pytest.raises(HexoError) as ei:
            srv.wait(tb)
        assert ei.value.status == HEXO_ERR_ADMISSION
        for t in ts:
            p, s = srv.wait(t)
            assert np.array_equal(p, want[0]) and np.array_equal(s, want[1])
        st = srv.stats()
    assert st["failed"] == 1 and st["completed"] == 4
    assert st["mem_peak"] <= 256 << 10


def test_invalid_request_and_unknown_ticket(engine):
    reqs, cfg = small_requests(n=1)
    bad = E.Request(reqs[0].params, 100.0, E.Options(np.array([100.0]), np.array([-1.0]), E.ASIAN), seed=1)
    with engine.server(cfg) as srv:
        t = srv.submit(bad)
        with pytest.raises(HexoError):
            srv.wait(t)
        with pytest.raises(HexoError) as ei:
            srv.wait(t)   # reported once, then forgotten
        assert ei.value.status == HEXO_ERR_NOT_FOUND
        good = srv.wait(srv.submit(reqs[0]))
    want = engine.price_batch([reqs[0]], cfg)[0]
    assert np.array_equal(good[0], want[0])


def test_requests_from_paramsdb(engine, tmp_path):
    # the serving loop fed by the reference's parameter database (HParams.db)
    from hestonexotics_gb300.paramsdb import ParamsDB
    reqs, cfg = small_requests(n=3)
    with ParamsDB(tmp_path / "HParams.db") as db:
        for k, rq in enumerate(reqs):
            db.insertupdate(rq.params, f"U{k}")
        # the table holds the five Heston parameters; the rate comes with the request
        from_db = [db.request(f"U{k}", rq.S0, rq.options, seed=rq.seed, r=rq.params.r,
                              stream=rq.stream) for k, rq in enumerate(reqs)]
    with engine.server(cfg) as srv:
        got = [srv.wait(srv.submit(rq)) for rq in from_db]
    for rq, (p, s) in zip(reqs, got):
        want = engine.price_batch([rq], cfg)[0]
        assert np.array_equal(p, want[0]) and np.array_equal(s, want[1])
