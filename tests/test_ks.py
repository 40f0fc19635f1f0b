"""Distributions against the unmodified reference: the reference's solver
sources (oracle/_ref) drawing from per-thread Mersenne twisters, seeded as
the reference seeds its GSL generators, against the oracle's per-node
Philox stream (which the GPU reproduces bit for bit).  A two-sample KS test
per compartment per tspan point over 10,000 replicates must not reject,
with the family-wise level 0.001 split over the tests (Bonferroni)."""
import os

import numpy as np
import pytest

from helpers import run_oracle
from siminf_gb300 import abi
from siminf_gb300 import model as M

REPLICATES = 10_000


def _have_ref():
    from oracle import oracle
    return os.path.exists(oracle.REF_LIB)


def _ks_all(m, seed_ours, seed_ref, nodes=(0,)):
    stats = pytest.importorskip("scipy.stats")
    from oracle import oracle
    mr = m.replicate(REPLICATES)
    code, _, ho = run_oracle(mr, seed=seed_ours, threads=8)
    assert code == 0
    hr = abi.build_args(mr, seed_ref)
    assert oracle.run_ref(hr, m.name, 8, independent=True) == 0
    tlen = len(m.tspan)
    U_o = ho.U.reshape((m.Nn * m.Nc, REPLICATES * tlen), order="F")
    U_r = hr.U.reshape((m.Nn * m.Nc, REPLICATES * tlen), order="F")
    tests = []
    for node in nodes:
        for c in range(m.Nc):
            for k in range(tlen):
                a = U_o[node * m.Nc + c, k::tlen]
                b = U_r[node * m.Nc + c, k::tlen]
                if a.min() == a.max() == b.min() == b.max():
                    continue            # a point mass in both: nothing to test
                tests.append(stats.ks_2samp(a, b).pvalue)
    level = 1e-3 / max(1, len(tests))
    assert len(tests) > 0
    assert min(tests) > level, (min(tests), level, len(tests))
    return tests


@pytest.mark.skipif(not _have_ref(), reason="the reference sources are not compiled here")
def test_ks_sir_against_reference(oracle_lib):
    u0 = {"S": np.full(4, 200), "I": np.full(4, 5), "R": np.zeros(4, int)}
    m = M.SIR(u0, np.array([3.0, 6.0, 10.0, 15.0, 22.0, 30.0]), 0.16, 0.077)
    _ks_all(m, seed_ours=101, seed_ref=202, nodes=(0, 3))


@pytest.mark.skipif(not _have_ref(), reason="the reference sources are not compiled here")
def test_ks_seir_events_against_reference(oracle_lib):
    from helpers import random_events
    rng = np.random.default_rng(4)
    Nn, days = 8, 20
    u0 = {"S": rng.poisson(150, Nn), "E": 0, "I": rng.poisson(4, Nn), "R": 0}
    ev = random_events(rng, Nn, days, p_enter=0.05, p_exit=0.05, p_exit_prop=0.02, n_e2=4,
                       n_e2_prop=1)
    m = M.SEIR(u0, np.array([5.0, 10.0, 15.0, 20.0]), 0.3, 0.25, 0.077, events=ev)
    _ks_all(m, seed_ours=7, seed_ref=8, nodes=(0, 5))


def _ks_nodes(m, seed_ours, seed_ref):
    """aem (one replicate only): a model of many identical, uncoupled nodes
    gives one sample per node; the oracle's aem against the reference's
    unmodified aem with independent generators, per compartment and tspan
    point."""
    stats = pytest.importorskip("scipy.stats")
    from oracle import oracle
    ho = abi.build_args(m, seed_ours, solver=1)
    code, _ = oracle.run(ho, m.name, 8)
    assert code == 0
    hr = abi.build_args(m, seed_ref, solver=1)
    assert oracle.run_ref(hr, m.name, 8, independent=True) == 0
    tlen = len(m.tspan)
    U_o = ho.U.reshape((m.Nc, m.Nn, tlen), order="F")     # [compartment, node, column]
    U_r = hr.U.reshape((m.Nc, m.Nn, tlen), order="F")
    tests = []
    for c in range(m.Nc):
        for k in range(tlen):
            a, b = U_o[c, :, k], U_r[c, :, k]
            if a.min() == a.max() == b.min() == b.max():
                continue
            tests.append(stats.ks_2samp(a, b).pvalue)
    level = 1e-3 / max(1, len(tests))
    assert len(tests) > 0
    assert min(tests) > level, (min(tests), level, len(tests))


@pytest.mark.skipif(not _have_ref(), reason="the reference sources are not compiled here")
def test_ks_sir_aem_against_reference(oracle_lib):
    n = REPLICATES
    u0 = {"S": np.full(n, 200), "I": np.full(n, 5), "R": np.zeros(n, int)}
    m = M.SIR(u0, np.array([3.0, 6.0, 10.0, 15.0, 22.0, 30.0]), 0.16, 0.077)
    _ks_nodes(m, seed_ours=11, seed_ref=12)


@pytest.mark.skipif(not _have_ref(), reason="the reference sources are not compiled here")
def test_ks_sise_aem_against_reference(oracle_lib):
    """SISe: time-dependent rates and a post-time-step function that
    changes phi every day, so every day ends with a rescaling refresh."""
    n = REPLICATES
    u0 = {"S": np.full(n, 120), "I": np.full(n, 6)}
    m = M.SISe(u0, np.arange(1, 41, 4), phi=0.2, upsilon=0.02, gamma=0.1, alpha=1,
               beta_t1=0.19, beta_t2=0.085, beta_t3=0.075, beta_t4=0.185, end_t1=10,
               end_t2=20, end_t3=30, end_t4=365, epsilon=0.0005)
    _ks_nodes(m, seed_ours=13, seed_ref=14)
