"""The SWIFT restatement (oracle/swift.cpp) against the reference's own known
answers: pricing_test's 40 prices and gradient_test's 200 gradient entries
(src/UnitTest.cpp:219-321), with the reference's tolerances (sum of absolute
differences below 1e-9 over all entries)."""
import numpy as np

from conftest import golden, unhex


def _cases(g):
    for i, (T, K, sp) in enumerate(zip(g["expiries"], g["strikes"], g["swift_params"])):
        yield i, T, np.array(K), np.array(sp)


def test_swift_golden_prices(oracle):
    g = golden("swift_golden.json")
    want = unhex(g["prices"])
    got = np.concatenate([oracle.swift_price(g["params5"], T, g["r"], g["S"], K, sp) for _, T, K, sp in _cases(g)])
    assert np.sum(np.abs(got - want)) < g["price_tolerance_sum_abs"]


def test_swift_golden_gradients(oracle):
    g = golden("swift_golden.json")
    want = unhex(g["grad"]).reshape(40, 5)
    imap = g["grad_index_map"]   # the golden rows list the components in another order
    got = np.concatenate([oracle.swift_price(g["params5"], T, g["r"], g["S"], K, sp, grad=True)[1]
                          for _, T, K, sp in _cases(g)])
    diff = sum(abs(want[i, imap[j]] - got[i, j]) for i in range(40) for j in range(5))
    assert diff < g["grad_tolerance_sum_abs"]


def test_swift_dynamic_parameters_converge(oracle):
    # the dynamic wavelet parameters (SWIFT.cpp:21-35) price the same chain
    # to well within the truncation tolerance of the predefined ones
    g = golden("swift_golden.json")
    for _, T, K, sp in _cases(g):
        dyn = oracle.swift_params(g["params5"], T, g["r"], g["S"], K.min(), K.max())
        assert dyn[7] >= 16 and dyn[5] < dyn[6]
        a = oracle.swift_price(g["params5"], T, g["r"], g["S"], K, sp)
        b = oracle.swift_price(g["params5"], T, g["r"], g["S"], K, dyn)
        np.testing.assert_allclose(a, b, atol=1e-6)


def test_chf_is_a_characteristic_function(oracle):
    p5 = [0.04, 0.05, -0.7, 1.5, 0.5]
    c0 = oracle.heston_chf_grad(p5, 1.0, 0.0 + 0j)[0]
    assert abs(c0 - 1.0) < 1e-12
    # E[exp(i u X)] at u = -i gives E[S_T/S_0] = 1 with no drift
    c1 = oracle.heston_chf_grad(p5, 1.0, 0.0 + 1j)[0]
    assert abs(c1 - 1.0) < 1e-9 or abs(oracle.heston_chf_grad(p5, 1.0, 0.0 - 1j)[0] - 1.0) < 1e-9
