"""GPU random numbers against the oracle, bit for bit, through the C ABI.

* SHISHUA words of streams seed + k (the device generator vs the oracle's).
* The two-buffer RNG as the path kernel runs it (shared-memory ring with a
  warp-synchronous look-ahead block) against the oracle's restatement of the
  reference RNG class, for draw-kind sequences with few and many uniforms.
* AS241 of every word: the device's integer-rounded float32 evaluation
  against the oracle's Fortran-semantics restatement, including the edge
  words where rounding decides P = 1, |Q| = 0.425 or the far tail.
"""
import numpy as np
import pytest

from conftest import golden, unhex

pytestmark = pytest.mark.gpu


def test_shishua_words(engine, oracle):
    seed, n_streams, n_words = 42, 300, 80
    got = engine.rng_words(seed, n_streams, n_words)
    for k in (0, 1, 7, 128, 299):
        want = oracle.shishua_words([(seed + k) & 0xFFFFFFFF, 0, 0, 0], n_words)
        assert np.array_equal(got[k], want), k


def test_shishua_seed_wraps_mod_2_32(engine, oracle):
    seed = 0xFFFFFFF0
    got = engine.rng_words(seed, 40, 16)
    for k in (0, 15, 16, 39):
        want = oracle.shishua_words([(seed + k) & 0xFFFFFFFF, 0, 0, 0], 16)
        assert np.array_equal(got[k], want), k


@pytest.mark.parametrize("stream", [1, 63, 0xFFFFFFFF])
def test_shishua_words_with_stream_word(engine, oracle, stream):
    # seed word 1 (the request's stream number) enters the state as SHISHUA's
    # init places it; stream 0 is the reference class's {seed, 0, 0, 0}
    seed = 3035318956
    got = engine.rng_words(seed, 64, 48, stream=stream)
    for k in (0, 5, 63):
        want = oracle.shishua_words([(seed + k) & 0xFFFFFFFF, stream, 0, 0], 48)
        assert np.array_equal(got[k], want), (k, stream)
    base = engine.rng_words(seed, 64, 48)
    assert not any(np.array_equal(got[k], base[k]) for k in range(64))


def test_two_buffer_draws_with_stream_word(engine, oracle):
    rng = np.random.default_rng(9)
    kinds = (rng.random(900) < 0.2).astype(np.uint8)
    seed, n_streams, stream = 77, 64, 12345
    got = engine.rng_draws(seed, n_streams, kinds, stream=stream)
    for k in range(0, n_streams, 9):
        want = oracle.rng_draws(seed + k, 16, kinds, stream=stream)
        assert np.array_equal(got[k].view(np.uint64), want.view(np.uint64)), k


@pytest.mark.parametrize("p_uniform", [0.0, 0.02, 0.3, 0.5, 1.0])
def test_two_buffer_draws(engine, oracle, p_uniform):
    rng = np.random.default_rng(int(p_uniform * 1000) + 1)
    kinds = (rng.random(1500) < p_uniform).astype(np.uint8)
    seed, n_streams = 1234, 96
    got = engine.rng_draws(seed, n_streams, kinds)
    for k in range(0, n_streams, 7):
        want = oracle.rng_draws(seed + k, 16, kinds)
        assert np.array_equal(got[k].view(np.uint64), want.view(np.uint64)), (k, p_uniform)


def test_draws_match_reference_golden(engine):
    for case in golden("rng_draws.json"):
        if case["size"] != 16:
            continue
        got = engine.rng_draws(case["seed"], 1, np.array(case["kinds"], dtype=np.uint8))[0]
        assert np.array_equal(got.view(np.uint64), unhex(case["draws"]).view(np.uint64)), case["seed"]


def edge_words():
    two64 = 1 << 64
    w = [0, 1, 2, 3, (1 << 53) - 1, 1 << 53, (1 << 53) + 1, 1 << 63, (1 << 63) - 1, (1 << 63) + 1,
         two64 - 1, two64 - 1024, two64 - 1025, two64 - 2048, two64 - 2049, 1 << 11, (1 << 11) + 1]
    # around |Q| = 0.425 (P = 0.075, 0.925) and the 5.0 split of the tail (R = e^-25)
    for p in (0.075, 0.925, np.exp(-25.0), 1 - np.exp(-25.0), 1e-15, 1 - 1e-15):
        c = int(p * 2.0 ** 64)
        w += [max(0, min(two64 - 1, c + d)) for d in range(-3000, 3001, 97)]
    return np.array(w, dtype=np.uint64)


def test_normals_edge_words(engine, oracle):
    w = edge_words()
    got = engine.normals(w)
    want = oracle.normals(w)
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))


def test_normals_random_words(engine, oracle):
    rng = np.random.default_rng(77)
    w = rng.integers(0, 2 ** 64 - 1, size=1 << 21, dtype=np.uint64, endpoint=True)
    # also dense tails: small and large words
    w[: 1 << 18] >>= rng.integers(3, 60, size=1 << 18).astype(np.uint64)
    w[1 << 18: 1 << 19] = ~(w[1 << 18: 1 << 19] >> rng.integers(3, 60, size=1 << 18).astype(np.uint64))
    got = engine.normals(w)
    want = oracle.normals(w)
    bad = np.flatnonzero(got.view(np.uint64) != want.view(np.uint64))
    assert bad.size == 0, (bad[:5], w[bad[:5]], got[bad[:5]], want[bad[:5]])


F32_0425 = 0x3ED9999A   # float(0.425): the largest |Q| of the central branch
F32_2M54 = 0x24800000   # 2^-54: P - 0.5 = (W - 2^63) 2^-64 with W = (double)w a multiple of 2^10 there
F32_2M64 = 0x1F800000   # 2^-64: the smallest P, and 1 - P >= 2^-53
F32_HALF = 0x3F000000


def test_as241_division_and_root_on_every_input(engine):
    """The kernels' AS241 divides and takes its square root with MUFU estimates and Newton/Markstein
    corrections instead of the IEEE intrinsics.  On every float the central branch can receive
    (Q = +0, P - 0.5 = 0 rounding to +0, or 2^-54 <= |Q| <= 0.425, both signs) and the tail
    (2^-64 <= R <= 0.5) the two must agree in every bit."""
    none = (0, 2 ** 64 - 1)
    assert engine.as241_check(0, 0, 1) == none
    for sign in (0, 0x80000000):
        assert engine.as241_check(0, sign + F32_2M54, sign + F32_0425 + 1) == none
    assert engine.as241_check(1, F32_2M64, F32_HALF + 1) == none


def test_as241_32bit_stage_on_every_high_word(engine):
    """The conversion certifies most words' Q in 32-bit arithmetic (2|s| +- 1 converted once, s the high
    word less 2^31); for all 2^32 high words, with low words at both ends of the accepted range, at 2^31
    and hashed, every certified Q must equal the exact stage's (the reference's double arithmetic)."""
    assert engine.as241_check(2, 0, 2 ** 32) == (0, 2 ** 64 - 1)


def test_draw_moments_across_streams(engine):
    # moments of the per-path streams the kernels use (RNG(16, seed + k)),
    # 4096 streams x 2048 draws of each kind, within 5 standard errors;
    # stream means must not drift with k
    n_streams, m = 4096, 2048
    kinds = np.concatenate([np.ones(m, dtype=np.uint8), np.zeros(m, dtype=np.uint8)])
    d = engine.rng_draws(77, n_streams, kinds)
    u, z = d[:, :m], d[:, m:]
    n = u.size
    assert abs(u.mean() - 0.5) < 5 * np.sqrt(1 / 12 / n)
    assert abs(u.var() - 1 / 12) < 5 * np.sqrt(1 / 180 / n)
    assert abs(z.mean()) < 5 / np.sqrt(n)
    assert abs(z.var() - 1.0) < 5 * np.sqrt(2.0 / n)
    half = n_streams // 2   # first and second half of the stream indices agree
    assert abs(z[:half].mean() - z[half:].mean()) < 5 * np.sqrt(2.0 / (n / 2))
