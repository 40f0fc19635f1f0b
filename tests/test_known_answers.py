"""Known answers of the solver's semantics that hold whatever the random
draws: every node's population changes only by its own events (enter,
exit, external transfers in and out, SimInf_solver.c:681-902) because
transitions move individuals between compartments of one node; states stay
non-negative; with zero rates and one populated compartment every event
moves exactly its n individuals, so the trajectory is fixed.  Column k of
U holds the state after the events of time tspan[k] (SimInf_solver_ssm.c:
262-334).  Checked on the oracle and, where they were built, on the
reference's own sources; the GPU path is held bit-exact to the oracle
elsewhere and checked for conservation at scale in the parity tests."""
import numpy as np
import pytest

from siminf_gb300 import model as M
from helpers import U_matrix, run_oracle, run_ref
from oracle import oracle


def seir_with_events(seed, Nn=300, days=60, rates=(0.16, 0.25, 0.077), infected=True):
    rng = np.random.default_rng(seed)
    u0 = {"S": rng.poisson(300, Nn) + 100, "E": 0,
          "I": rng.poisson(3, Nn) if infected else 0, "R": 0}
    ev = {k: [] for k in M.EVENT_FIELDS}

    def add(*vals):
        for key, val in zip(M.EVENT_FIELDS, vals):
            ev[key].append(val)

    for t in range(1, days + 1):
        for node in np.nonzero(rng.random(Nn) < 0.02)[0]:
            add(1, t, node + 1, 0, int(rng.integers(1, 4)), 0.0, 1, 0)     # enter into S
        for node in np.nonzero(rng.random(Nn) < 0.02)[0]:
            add(0, t, node + 1, 0, 1, 0.0, 2, 0)                            # exit from any
        src = rng.integers(1, Nn + 1, 40)
        dst = rng.integers(1, Nn + 1, 40)
        for s_, d_ in zip(src, dst):
            if s_ != d_:
                add(3, t, s_, d_, 1 + int(rng.poisson(2)), 0.0, 2, 0)
    events = M.make_events(**{k: np.array(v) for k, v in ev.items()})
    return M.SEIR(u0, np.arange(1, days + 1), *rates, events=events)


def expected_population(m):
    """Population of every node after each tspan point, from u0 and the
    events alone: [Nn, tlen]."""
    ev = m.events
    u0 = np.asarray(m.u0).reshape(m.Nc, m.Nn, order="F") if np.asarray(m.u0).ndim == 1 \
        else np.asarray(m.u0)
    pop0 = u0.sum(axis=0).astype(np.int64)
    out = np.zeros((m.Nn, len(m.tspan)), dtype=np.int64)
    delta = np.zeros(m.Nn, dtype=np.int64)
    order = np.argsort(ev["time"], kind="stable")
    i = 0
    for k, t in enumerate(m.tspan):
        while i < len(order) and ev["time"][order[i]] <= t:
            j = order[i]
            node, n = ev["node"][j] - 1, ev["n"][j]
            if ev["event"][j] == 1:
                delta[node] += n
            elif ev["event"][j] == 0:
                delta[node] -= n
            elif ev["event"][j] == 3:
                delta[node] -= n
                delta[ev["dest"][j] - 1] += n
            i += 1
        out[:, k] = pop0 + delta
    return out


def node_population(m, h):
    U = U_matrix(m, h).reshape(m.Nn, m.Nc, -1)
    return U.sum(axis=1), U


def check_population(m, h):
    pop, U = node_population(m, h)
    assert (U >= 0).all()
    assert np.array_equal(pop, expected_population(m))


@pytest.mark.parametrize("seed", [1, 2])
def test_oracle_population_follows_events(oracle_lib, seed):
    m = seir_with_events(seed)
    code, res, h = run_oracle(m, threads=2)
    assert code == 0
    assert res.transitions > 1000
    check_population(m, h)


def test_reference_population_follows_events(oracle_lib):
    if not oracle.ref_available():
        pytest.skip("reference build not available")
    m = seir_with_events(3)
    code, h = run_ref(m, threads=2)
    assert code == 0
    check_population(m, h)


def test_zero_rates_one_compartment_is_deterministic(oracle_lib):
    """Zero rates and everyone in S: every exit and transfer takes exactly
    n out of S, so S after each day is u0 plus the events' sums, whatever
    the seed."""
    m = seir_with_events(4, rates=(0.0, 0.0, 0.0), infected=False)
    runs = []
    for seed in (1, 99):
        code, res, h = run_oracle(m, seed=seed)
        assert code == 0 and res.transitions == 0
        pop, U = node_population(m, h)
        assert (U[:, 1:, :] == 0).all()                   # E, I, R stay empty
        assert np.array_equal(U[:, 0, :], expected_population(m))
        runs.append(U_matrix(m, h).copy())
    assert np.array_equal(runs[0], runs[1])
