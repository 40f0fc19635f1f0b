"""Batches of independent models (siminf_gpu_run_batch): every model's
prevalence series and distance equal those of the oracle run of that model
alone and of the GPU run of that model alone, bit for bit; uneven node
counts, tspan lengths, events, parameters and seeds."""
import math

import numpy as np
import pytest

from helpers import random_events, run_gpu, run_oracle
from siminf_gb300 import model as M


def batch_models(seed=3, n=5):
    rng = np.random.default_rng(seed)
    sizes = [30, 200, 7, 150, 64, 90, 12][:n]
    lengths = [20, 45, 10, 60, 33, 41, 5][:n]
    models = []
    for Nn, T in zip(sizes, lengths):
        u0 = {"S": rng.poisson(200, Nn), "E": 0,
              "I": rng.poisson(3, Nn) * (rng.random(Nn) < 0.3), "R": 0}
        ev = random_events(rng, Nn, T, n_e2=max(2, Nn // 5), n_e2_prop=1)
        beta, eps, gamma = rng.uniform(0.05, 0.5), rng.uniform(0.1, 0.5), rng.uniform(0.02, 0.2)
        models.append(M.SEIR(u0, np.arange(1, T + 1), beta, eps, gamma, events=ev))
    return models


def prevalence_of(m, U, num=(2,), den=(0, 1, 2, 3)):
    """The batch's reduction restated on a U matrix: integer sums over nodes,
    one IEEE division per column."""
    U = np.asarray(U).reshape((m.Nn * m.Nc, len(m.tspan)), order="F")
    out = []
    for k in range(len(m.tspan)):
        col = U[:, k].astype(np.int64)
        a = int(sum(col[c::m.Nc].sum() for c in num))
        b = int(sum(col[c::m.Nc].sum() for c in den))
        out.append(a / b if b else 0.0)
    return np.array(out)


def distance_of(prev, target):
    acc = 0.0
    for p, t in zip(prev, target):
        d = float(p) - float(t)
        acc = acc + d * d
    return math.sqrt(acc)


def test_batch_rejects_mixed_tspan_start(oracle_lib):
    from siminf_gb300.run import run_batch
    from siminf_gb300 import abi, native
    ms = batch_models(n=2)
    ms[1].tspan = ms[1].tspan + 0.5
    with pytest.raises(abi.SimInfError):
        run_batch(ms, [1, 2])
    assert b"tspan starts" in native.last_status().message


@pytest.mark.gpu
@pytest.mark.parametrize("two_pass", ["-1", "1"])
def test_batch_matches_oracle_and_alone(gpu, oracle_lib, monkeypatch, two_pass):
    monkeypatch.setenv("SIMINF_TWO_PASS", two_pass)
    from siminf_gb300.run import run_batch
    models = batch_models()
    seeds = [11, 12, 13, 2 ** 33 + 1, 99]
    rng = np.random.default_rng(5)
    targets = [rng.uniform(0, 0.05, len(m.tspan)) for m in models]
    prevs, dists = run_batch(models, seeds, targets, cap_transfers=False)
    for j, (m, s) in enumerate(zip(models, seeds)):
        code_o, _, ho = run_oracle(m, seed=s, threads=2)
        code_g, hg, _ = run_gpu(m, seed=s)
        assert code_o == 0 and code_g == 0
        want = prevalence_of(m, ho.U)
        assert np.array_equal(prevalence_of(m, hg.U), want), j     # alone on the GPU
        assert np.array_equal(prevs[j], want), j                    # in the batch
        assert dists[j] == distance_of(want, targets[j]), j


@pytest.mark.gpu
def test_batch_without_events_and_targets(gpu, oracle_lib):
    from siminf_gb300.run import run_batch
    rng = np.random.default_rng(8)
    models = []
    for Nn, T in [(40, 30), (5, 12), (300, 50)]:
        u0 = {"S": rng.poisson(90, Nn), "I": rng.poisson(3, Nn), "R": np.zeros(Nn, int)}
        models.append(M.SIR(u0, np.arange(1, T + 1), rng.uniform(0.1, 0.4), 0.077))
    prevs, dists = run_batch(models, [1, 2, 3], numerator=(1,))
    for j, m in enumerate(models):
        _, _, ho = run_oracle(m, seed=j + 1, threads=2)
        assert np.array_equal(prevs[j], prevalence_of(m, ho.U, num=(1,), den=(0, 1, 2)))
        assert dists[j] == 0.0
