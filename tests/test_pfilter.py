"""Particle filter: the oracle restatement of pfilter_internal
(R/pfilter.R:315-499) and systematic resampling
(src/misc/SimInf_particle_filter.c:33-67), and the GPU version bit for bit
against it."""
import numpy as np
import pytest

from siminf_gb300 import model as M
from oracle import oracle


def small_case(nodes=20, particles=64, weeks=8, seed=3):
    rng = np.random.default_rng(seed)
    u0 = np.vstack([rng.poisson(60, nodes), rng.poisson(3, nodes)]).astype(np.int32)
    m = M.SISe_pf(u0, np.array([0.0]), upsilon=0.02, gamma=0.1)
    obs_time = np.arange(7, 7 * weeks + 1, 7, dtype=np.int32)
    obs = rng.binomial(4, 0.5, size=(weeks, nodes)).astype(np.int32)
    gdata = np.column_stack([rng.uniform(0.005, 0.03, particles),
                             rng.uniform(0.05, 0.2, particles)])
    return m, gdata, obs_time, obs


def test_oracle_pfilter_runs_and_is_deterministic(oracle_lib):
    m, gdata, t, obs = small_case()
    c1, ll1, ess1, a1 = oracle.pfilter(m, 64, t, obs, 1, 0.8, seed=5, gdata=gdata)
    c2, ll2, ess2, a2 = oracle.pfilter(m, 64, t, obs, 1, 0.8, seed=5, gdata=gdata, threads=4)
    assert c1 == 0 and c2 == 0
    assert np.isfinite(ll1) and ll1 == ll2
    assert np.array_equal(ess1, ess2) and np.array_equal(a1, a2)
    assert ((ess1 >= 1.0 - 1e-9) & (ess1 <= 64 + 1e-9)).all()
    assert a1.min() >= 1 and a1.max() <= 64
    # ancestors are non-decreasing: systematic resampling walks the cumsum
    assert (np.diff(a1, axis=1) >= 0).all()


def test_oracle_pfilter_shared_gdata_and_gap_one(oracle_lib):
    """Consecutive observation days use one-point intervals (R/pfilter.R:
    187-192)."""
    m, _, _, _ = small_case()
    t = np.array([3, 4, 5, 9], dtype=np.int32)
    obs = np.ones((4, m.Nn), dtype=np.int32)
    code, ll, ess, anc = oracle.pfilter(m, 32, t, obs, 1, 0.5, seed=1)
    assert code == 0 and np.isfinite(ll)


@pytest.mark.gpu
def test_gpu_pfilter_matches_oracle(gpu, oracle_lib):
    from siminf_gb300.run import pfilter
    m, gdata, t, obs = small_case()
    code, ll, ess, anc = oracle.pfilter(m, 64, t, obs, 1, 0.8, seed=5, gdata=gdata, threads=4)
    r = pfilter(m, 64, t, obs, 1, 0.8, seed=5, gdata=gdata)
    assert code == 0
    assert r.loglik == ll
    assert np.array_equal(r.ess, ess)
    assert np.array_equal(r.ancestors, anc)


@pytest.mark.gpu
def test_gpu_pfilter_workload_small(gpu, oracle_lib):
    """The particle-filter workload generator at 2% of its size."""
    from siminf_gb300 import workloads
    from siminf_gb300.run import pfilter
    m, gdata, t, obs = workloads.sise_pfilter(nodes=50, particles=128, weeks=12)
    code, ll, ess, anc = oracle.pfilter(m, 128, t, obs, 1, 0.8, seed=11, gdata=gdata, threads=4)
    r = pfilter(m, 128, t, obs, 1, 0.8, seed=11, gdata=gdata)
    assert code == 0 and r.loglik == ll and np.array_equal(r.ancestors, anc)
