"""hexo_price_noalloc: pricing for callers that cannot let a library allocate
GPU memory (a framework's pool owns the device, or a latency-critical loop
must not pay cudaMalloc's synchronisation).  It keeps its device-side work in
one fixed array compiled into the library, shared by every call, so these
tests call it through the C ABI twice in a row, on requests of different
sizes, and check each result against hexo_price, the allocating entry point,
to the FP64 tolerance of the other parity tests (the two share the kernels
and the launch shape, so they agree bit for bit).  The file is collected last
so that a stop at the first failure has run everything else first.
"""
import ctypes as C

import numpy as np
import pytest

from hestonexotics_gb300 import _lib as L
from hestonexotics_gb300 import engine as E
from hestonexotics_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def noalloc(params, S0, options, cfg):
    lib = L.load()
    n = len(options)
    price = np.zeros(n)
    se = np.zeros(n)
    p = params.c()
    c = cfg.c()
    st = lib.hexo_price_noalloc(C.byref(p), float(S0), options.c_array(), n, C.byref(c),
                                price.ctypes.data_as(C.POINTER(C.c_double)),
                                se.ctypes.data_as(C.POINTER(C.c_double)), None)
    return st, price, se


def cases():
    req0, cfg0 = W.plain_asian(n_paths=1 << 16)
    req1, cfg1 = W.single_chain(n_paths=5000)
    keep = np.arange(0, len(req1.options), 7)[:100]          # 3 maturities' worth, both payoffs
    opts1 = E.Options(req1.options.strike[keep], req1.options.T[keep], req1.options.payoff[keep])
    cfg1.precision = E.FP32
    return [(req0.params, req0.S0, req0.options, cfg0), (req1.params, req1.S0, opts1, cfg1)]


def test_noalloc_matches_hexo_price_on_consecutive_calls(engine):
    # a large request, then a smaller one with more options, then the first again
    for params, S0, opts, cfg in cases() + cases()[:1]:
        st, p, se = noalloc(params, S0, opts, cfg)
        assert st == 0, L.STATUS_NAMES.get(st, st)
        want_p, want_se = engine.price(params, S0, opts, cfg)
        np.testing.assert_allclose(p, want_p, rtol=1e-10, atol=1e-12 * S0)
        np.testing.assert_allclose(se, want_se, rtol=1e-10, atol=1e-12 * S0)


def test_noalloc_rejects_sizes_beyond_its_limits():
    params = E.Params(0.04, 0.04, -0.7, 1.5, 0.5)
    too_many = E.Options(np.full(129, 100.0), 1.0, 0)
    st, _, _ = noalloc(params, 100.0, too_many, E.Config(n_paths=1024, steps=10))
    assert st == 10  # HEXO_ERR_TOO_LARGE
    one = E.Options(np.array([100.0]), 1.0, 0)
    st, _, _ = noalloc(params, 100.0, one, E.Config(n_paths=(1 << 20) + 1, steps=10))
    assert st == 10


def test_noalloc_after_calls_with_smaller_launch_shapes(engine):
    # the allocating entry points launch the same path kernels with other
    # launch shapes (here 128-thread CTAs, whose shared memory is smaller);
    # the kernels' shared-memory limit is the same for every caller, so the
    # no-allocation call after them still launches its 256-thread CTAs
    params, S0, opts, cfg = cases()[1]
    for prec in (E.FP64, E.FP32):
        small = E.Config(**{**cfg.__dict__, "precision": prec, "block": 128})
        want_p, want_se = engine.price(params, S0, opts, small)
        st, p, se = noalloc(params, S0, opts, E.Config(**{**cfg.__dict__, "precision": prec}))
        assert st == 0, L.STATUS_NAMES.get(st, st)
        assert np.array_equal(p, want_p) and np.array_equal(se, want_se)
