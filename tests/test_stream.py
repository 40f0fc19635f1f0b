"""The shared random source (siminf_stream.h) through the oracle library:
Philox4x32-10 known-answer vectors, logarithm accuracy, uniform range and
the samplers' distributions."""
import math

import numpy as np
import pytest


# Known-answer vectors published with Random123 (Salmon et al., SC 2011).
KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,want", KAT)
def test_philox_known_answers(oracle_lib, ctr, key, want):
    assert tuple(oracle_lib.philox(ctr, key)) == want


def _ulp(x):
    return math.ulp(abs(x))


def test_log_accuracy(oracle_lib):
    rng = np.random.default_rng(7)
    xs = list(rng.uniform(1e-6, 1.0, 20000))
    xs += list(1.0 + rng.uniform(-0.02, 0.02, 20000))
    xs += list(np.exp(rng.uniform(-700, 700, 20000)))
    xs += [1.0, 2.0, 0.5, 1e-300, 5e-324, 1.7976931348623157e308, 1.0 + 2 ** -52, 1.0 - 2 ** -53]
    worst = 0.0
    for x in xs:
        got = oracle_lib.si_log(float(x))
        want = math.log(float(x))
        if got != want:
            worst = max(worst, abs(got - want) / _ulp(want))
    assert worst <= 1.0
    assert oracle_lib.si_log(1.0) == 0.0
    assert oracle_lib.si_log(0.0) == -math.inf
    assert math.isnan(oracle_lib.si_log(-1.0))
    assert oracle_lib.si_log(math.inf) == math.inf


def test_neglog_u32_accuracy(oracle_lib):
    """-log(u) of a 32-bit uniform u = (2w+1) 2^-33, against 60-digit
    arithmetic: within one ulp on random words and on the edges of the
    table reduction (the powers of two, the hand-over to si_log at
    u = 1 - 2^-8, the extremes)."""
    mp = pytest.importorskip("mpmath")
    mp.mp.dps = 60
    rng = np.random.default_rng(11)
    words = list(rng.integers(0, 2 ** 32, 20000, dtype=np.uint64))
    words += list(rng.integers(2 ** 32 - 2 ** 24 - 4096, 2 ** 32 - 2 ** 24 + 4096, 2000, dtype=np.uint64))
    edges = [0, 1, 2, 2 ** 32 - 1, 2 ** 32 - 2, 2 ** 32 - 2 ** 24 - 1, 2 ** 32 - 2 ** 24]
    for b in range(1, 33):
        edges += [2 ** (b - 1) - 1, 2 ** (b - 1), max(0, 2 ** (b - 1) - 2)]
    words = np.array(words + [e for e in edges if e < 2 ** 32], dtype=np.uint32)
    got = oracle_lib.neglog_u32(words)
    worst = 0.0
    for w, g in zip(words, got):
        want = -mp.log(mp.mpf(2 * int(w) + 1) / mp.mpf(2) ** 33)
        worst = max(worst, float(abs(mp.mpf(g) - want)) / math.ulp(g))
    assert worst < 1.0
    # the same value the general logarithm gives, almost always bit for bit
    u = (2 * words.astype(np.float64) + 1) * 2.0 ** -33
    general = np.array([-oracle_lib.si_log(x) for x in u[:5000]])
    assert np.mean(general == got[:5000]) > 0.99


def test_uniform_pos_open_interval_and_moments(oracle_lib):
    u = oracle_lib.uniform_pos(42, 3, 0, 200000)
    assert (u > 0).all() and (u < 1).all()
    assert abs(u.mean() - 0.5) < 0.005
    assert abs(u.var() - 1 / 12) < 0.002
    # a stream started mid-block continues the same sequence
    v = oracle_lib.uniform_pos(42, 3, 5, 100)
    assert np.array_equal(u[5:105], v)
    # 32-bit resolution: (2w+1) * 2^-33
    w = u * 2 ** 33
    assert np.array_equal(w, np.round(w)) and (np.round(w) % 2 == 1).all()


def test_hypergeometric_distribution(oracle_lib):
    scipy_stats = pytest.importorskip("scipy.stats")
    for n1, n2, t in ((30, 70, 10), (5, 3, 6), (200, 50, 180), (1, 1000, 400)):
        k = oracle_lib.hypergeometric(9, 11, n1, n2, t, 40000)
        assert k.min() >= max(0, t - n2) and k.max() <= min(n1, t)
        support = np.arange(max(0, t - n2), min(n1, t) + 1)
        pmf = scipy_stats.hypergeom(n1 + n2, n1, t).pmf(support)
        obs = np.array([(k == s).sum() for s in support])
        keep = pmf * len(k) >= 5
        exp = pmf[keep] * len(k)
        chi2 = ((obs[keep] - exp) ** 2 / exp).sum()
        assert scipy_stats.chi2.sf(chi2, max(keep.sum() - 1, 1)) > 1e-4, (n1, n2, t)


def test_binomial_distribution(oracle_lib):
    scipy_stats = pytest.importorskip("scipy.stats")
    for p, n in ((0.1, 20), (0.5, 1500), (0.93, 40), (0.003, 100000)):
        k = oracle_lib.binomial(5, 17, p, n, 20000)
        assert k.min() >= 0 and k.max() <= n
        assert abs(k.mean() - n * p) < 5 * math.sqrt(n * p * (1 - p) / len(k)) + 1e-9
        assert abs(k.var() / (n * p * (1 - p)) - 1) < 0.06
    assert (oracle_lib.binomial(1, 1, 0.0, 50, 10) == 0).all()
    assert (oracle_lib.binomial(1, 1, 1.0, 50, 10) == 50).all()
