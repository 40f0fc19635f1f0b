"""PMCMC (R/pmcmc.R:470-600): a chain resident on the GPU whose particle
filter session stays on the device across iterations and calls.  The
chain equals the oracle's restatement (the same proposals and acceptance
on the oracle's particle filter) row for row, a continued chain equals an
uninterrupted one, and a continuation through the server equals the call
made directly."""
import numpy as np
import pytest

from oracle import oracle
from siminf_gb300 import model as M

pytestmark = pytest.mark.gpu


def case(nodes=25, weeks=6, particles=64, seed=3):
    rng = np.random.default_rng(seed)
    u0 = np.vstack([rng.poisson(60, nodes), rng.poisson(3, nodes)]).astype(np.int32)
    m = M.SISe_pf(u0, np.array([0.0]), upsilon=0.02, gamma=0.1)
    obs_time = np.arange(7, 7 * weeks + 1, 7, dtype=np.int32)
    obs = rng.binomial(4, 0.5, size=(weeks, nodes)).astype(np.int32)
    covmat = np.array([[2e-5, 0.0], [0.0, 4e-4]])
    return dict(model=m, n_particles=particles, obs_time=obs_time, obs=obs,
                obs_compartment=1, detect_p=0.8, pars=[0, 1], theta=[0.02, 0.1],
                prior_lo=[0.005, 0.05], prior_hi=[0.03, 0.2], covmat=covmat, seed=11)


def gpu_chain(kw):
    from siminf_gb300.run import Pmcmc
    return Pmcmc(**kw)


def test_gpu_pmcmc_matches_oracle(gpu, oracle_lib):
    kw = case()
    ch = gpu_chain(kw)
    rows = ch.run(8)
    chol = np.linalg.cholesky(kw["covmat"]).T
    want = oracle.pmcmc(kw["model"], kw["n_particles"], kw["obs_time"], kw["obs"],
                        kw["obs_compartment"], kw["detect_p"], kw["pars"], kw["theta"],
                        kw["prior_lo"], kw["prior_hi"], chol, kw["seed"], 8, threads=4)
    assert np.array_equal(rows, want)
    assert rows[:, 3].sum() >= 1                      # some proposal accepted
    ch.close()


def test_gpu_pmcmc_continued_equals_uninterrupted(gpu):
    kw = case()
    whole = gpu_chain(kw)
    a = whole.run(7)
    parts = gpu_chain(kw)
    b = np.vstack([parts.run(3), parts.run(1), parts.run(3)])
    assert np.array_equal(a, b)
    assert np.array_equal(parts.chain, whole.chain)
    whole.close()
    parts.close()


def test_gpu_pmcmc_served_continuation(gpu):
    """Continuations of two resident chains submitted to the server,
    interleaved with particle filters, give the rows of the chains run
    directly."""
    from siminf_gb300.serve import Server
    kw = case()
    direct = gpu_chain(kw).run(6)
    kw2 = dict(kw, seed=99)
    direct2 = gpu_chain(kw2).run(6)
    c1, c2 = gpu_chain(kw), gpu_chain(kw2)
    srv = Server(slots=4)
    tickets = []
    for _ in range(3):
        tickets.append(srv.pmcmc(c1, 2))
        tickets.append(srv.pfilter(kw["model"], 32, kw["obs_time"], kw["obs"], 1, 0.8, seed=5))
        tickets.append(srv.pmcmc(c2, 2))
        # a chain's continuations run one after another: wait before the next
        for t in tickets[-3:]:
            srv.wait(t)
    srv.close()
    assert np.array_equal(c1.chain, direct)
    assert np.array_equal(c2.chain, direct2)
