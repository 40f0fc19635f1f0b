"""The ABC-SMC driver (siminf_gb300/abc.py) on the CPU: its proposal and
weight kernels against loops written the way src/misc/SimInf_abc.c writes
them, and the generation loop (R/abc.R:742-843) on a stand-in for the
device batch.  The GPU test runs the loop over real batches."""
import math

import numpy as np
import pytest

from siminf_gb300 import abc


def loop_weights(priors, x_anc, xx, x, w, sigma):
    """SimInf_abc_weights written out per particle, as the C code loops."""
    n, d = xx.shape
    inv = np.linalg.inv(sigma)
    det = np.linalg.det(sigma)
    ww = np.zeros(n)
    mx = 0.0
    for i in range(n):
        acc = 0.0
        for k, p in enumerate(priors):
            acc += float(p.log_density(xx[i, k], x_anc[i, k]))
        s = 0.0
        for j in range(len(x)):
            diff = xx[i] - x[j]
            s += w[j] * math.exp(-0.5 * diff @ inv @ diff) / math.sqrt((2 * math.pi) ** d * det)
        ww[i] = acc - math.log(s)
        mx = max(mx, ww[i])
    ww = np.exp(ww - mx)
    return ww / ww.sum()


def test_weights_match_the_c_loops():
    rng = np.random.default_rng(3)
    priors = [abc.Prior("beta", "uniform", 0.05, 0.5), abc.Prior("eps", "normal", 0.3, 0.1),
              abc.Prior("gamma", "uniform", 0.02, 0.2)]
    x = np.column_stack([rng.uniform(0.05, 0.5, 40), rng.normal(0.3, 0.1, 40),
                         rng.uniform(0.02, 0.2, 40)])
    w = rng.random(40)
    w /= w.sum()
    sigma = 2.0 * np.cov(x, rowvar=False)
    xx, anc = abc.proposals(priors, 30, rng, x, w, sigma)
    got = abc.weights(priors, x[anc], xx, x, w, sigma)
    want = loop_weights(priors, x[anc], xx, x, w, sigma)
    assert np.allclose(got, want, rtol=1e-12, atol=0)
    assert abs(got.sum() - 1.0) < 1e-12


def test_proposals_stay_in_the_prior_support():
    rng = np.random.default_rng(4)
    priors = [abc.Prior("a", "uniform", 0.0, 1.0), abc.Prior("b", "uniform", 2.0, 3.0)]
    x, anc = abc.proposals(priors, 500, rng)
    assert (anc == -1).all() and (x[:, 0] >= 0).all() and (x[:, 1] <= 3).all()
    w = np.full(500, 1 / 500)
    xx, anc = abc.proposals(priors, 2000, rng, x, w, 2.0 * np.cov(x, rowvar=False))
    assert ((xx[:, 0] >= 0) & (xx[:, 0] <= 1) & (xx[:, 1] >= 2) & (xx[:, 1] <= 3)).all()
    assert anc.min() >= 0 and anc.max() < 500
    # ancestors drawn by weight: a particle of weight 0 is never picked
    w0 = w.copy()
    w0[:250] = 0
    _, anc = abc.proposals(priors, 1000, rng, x, w0 / w0.sum(), 2.0 * np.cov(x, rowvar=False))
    assert anc.min() >= 250
    with pytest.raises(ValueError):
        abc.proposals(priors, 10, rng, x, -w, np.eye(2))


def test_generation_loop_on_a_stand_in_batch(monkeypatch):
    """Tolerances fall, every generation keeps n_particles accepted
    particles within its tolerance, weights are normalised, and the
    posterior of a known parameter tightens around it."""
    truth = 0.3

    class Stub:
        def __init__(self, th):
            self.th = th
            self.Nn, self.tspan = 10, np.arange(5)

    def fake_batch(models, seeds, targets, cap_transfers=False):
        th = np.array([m.th for m in models])
        noise = np.random.default_rng(int(seeds[0])).normal(0, 0.01, len(th))
        return None, np.abs(th - truth) + np.abs(noise)

    monkeypatch.setattr(abc, "run_batch", fake_batch)

    def simulate(theta, rng):
        seeds = [int(rng.integers(1, 2 ** 31))] * len(theta)
        return [Stub(t[0]) for t in theta], seeds, [None] * len(theta)

    gens = abc.abc_smc(simulate, [abc.Prior("th", "uniform", 0.0, 1.0)], n_particles=200,
                       generations=4, batch=256, n_init=800, seed=9)
    tols = [g.tolerance for g in gens]
    assert all(b <= a for a, b in zip(tols, tols[1:]))
    for g in gens:
        assert g.x.shape == (200, 1) and (g.distance <= g.tolerance).all()
        assert abs(g.w.sum() - 1.0) < 1e-12
    assert abs(np.average(gens[-1].x[:, 0], weights=gens[-1].w) - truth) < 0.02


@pytest.mark.gpu
def test_abc_smc_on_device_batches(gpu):
    """Three generations over real batches of small uneven SEIR models:
    every accepted particle's distance, which the device computed, is within
    its generation's tolerance, and equals the distance of the same model
    run alone."""
    import copy
    from siminf_gb300 import model as M
    from siminf_gb300 import workloads
    from siminf_gb300.run import run, run_batch
    rng = np.random.default_rng(2)
    pool = [workloads.seir_events_fast(int(n), int(T), int(n) // 2, rng)
            for n, T in zip(rng.choice((50, 200), 6), rng.integers(20, 41, 6))]
    target = np.linspace(0.0, 0.02, 41)
    made = []

    def simulate(theta, g):
        models, seeds, targets = [], [], []
        for b, e, gm in theta:
            s = copy.copy(pool[int(g.integers(0, len(pool)))])
            s.ldata = M._rep_ldata(s.Nn, b, e, gm)
            models.append(s)
            seeds.append(int(g.integers(1, 2 ** 62)))
            targets.append(target[:len(s.tspan)])
        made.append((models, seeds, targets))
        return models, seeds, targets

    priors = [abc.Prior("beta", "uniform", 0.05, 0.5), abc.Prior("epsilon", "uniform", 0.1, 0.5),
              abc.Prior("gamma", "uniform", 0.02, 0.2)]
    gens = abc.abc_smc(simulate, priors, n_particles=32, generations=3, batch=64, n_init=64,
                       seed=4)
    for g in gens:
        assert len(g.x) == 32 and (g.distance <= g.tolerance).all()
    # one proposal of the first batch, run alone, gives the batch's distance
    models, seeds, targets = made[0]
    _, d_batch = run_batch(models[:3], seeds[:3], targets[:3], cap_transfers=True)
    for m, sd, tg, db in zip(models[:3], seeds[:3], targets[:3], d_batch):
        r = run(m, seed=sd, cap_transfers=True)
        I = r.U[2::4].sum(axis=0).astype(float)
        N = r.U.sum(axis=0).astype(float)
        prev = np.where(N > 0, I / np.maximum(N, 1.0), 0.0)
        assert abs(np.sqrt(np.sum((prev - tg) ** 2)) - db) < 1e-12


def test_continue_abc_equals_the_longer_run(monkeypatch):
    """continue_abc (R/abc.R:996-1027) from a 3-generation run, for 2 more,
    gives the 5-generation run's particles, weights and tolerances: the
    quantile rule's next tolerance and the random generator carry over."""
    truth = 0.4

    class Stub:
        def __init__(self, th):
            self.th = th
            self.Nn, self.tspan = 10, np.arange(5)

    def fake_batch(models, seeds, targets, cap_transfers=False):
        th = np.array([m.th for m in models])
        noise = np.random.default_rng(int(seeds[0])).normal(0, 0.01, len(th))
        return None, np.abs(th - truth) + np.abs(noise)

    monkeypatch.setattr(abc, "run_batch", fake_batch)

    def simulate(theta, rng):
        seeds = [int(rng.integers(1, 2 ** 31))] * len(theta)
        return [Stub(t[0]) for t in theta], seeds, [None] * len(theta)

    priors = [abc.Prior("th", "uniform", 0.0, 1.0)]
    whole = abc.abc_smc(simulate, priors, n_particles=100, generations=5, batch=128, n_init=400,
                        seed=11, quantile=0.6)
    part = abc.abc_smc(simulate, priors, n_particles=100, generations=3, batch=128, n_init=400,
                       seed=11, quantile=0.6)
    more = abc.continue_abc(part, simulate, 2)
    assert len(more) == 5 and len(part) == 3
    for a, b in zip(whole, more):
        assert a.tolerance == b.tolerance and a.nprop == b.nprop
        assert np.array_equal(a.x, b.x) and np.array_equal(a.w, b.w)
    # given tolerances: one per new generation
    given = abc.continue_abc(part, simulate, 2, tolerance=[0.05, 0.03])
    assert [g.tolerance for g in given[3:]] == [0.05, 0.03]
    with pytest.raises(ValueError):
        abc.continue_abc(part, simulate, 3, tolerance=[0.05])
