"""The event table's ordering on the device (siminf_gpu_sort_events)
against the oracle (numpy's stable lexsort), which is checked here against
the definition in R/SimInf_events.R:396: sort by (time, event, select),
ties in input order."""
import numpy as np
import pytest

from oracle import events as ref


def random_table(rng, n, tspan=(-5, 40), nsel=6, nev=4):
    return {"event": rng.integers(0, nev, n), "time": rng.integers(*tspan, n),
            "node": rng.integers(1, 1000, n), "dest": rng.integers(0, 1000, n),
            "n": rng.integers(0, 9, n), "proportion": rng.random(n),
            "select": rng.integers(1, nsel + 1, n), "shift": rng.integers(0, 3, n)}


def test_oracle_is_the_stable_order():
    rng = np.random.default_rng(2)
    ev = random_table(rng, 400)
    want = sorted(range(400), key=lambda i: (ev["time"][i], ev["event"][i], ev["select"][i]))
    got = ref.sort_events(ev)
    for k in ref.COLUMNS:
        assert np.array_equal(got[k], np.asarray(ev[k])[want])


@pytest.mark.gpu
@pytest.mark.parametrize("n,tspan,nsel", [(0, (0, 2), 2), (1, (0, 2), 2), (2, (3, 4), 1),
                                          (1000, (-5, 40), 6), (100_003, (1, 366), 3),
                                          (3_000_000, (-(2 ** 30), 2 ** 30), 2000),
                                          (500_000, (7, 8), 1)])
def test_gpu_sort_matches_the_oracle(gpu, n, tspan, nsel):
    from siminf_gb300.events import sort_events
    rng = np.random.default_rng(n)
    ev = random_table(rng, n, tspan, nsel)
    got = sort_events(ev)
    want = ref.sort_events(ev)
    for k in ref.COLUMNS:
        assert np.array_equal(got[k], want[k]), k


@pytest.mark.gpu
def test_gpu_sort_of_a_shuffled_workload_schedule(gpu):
    """The headline generator's schedule at a tenth of its size, shuffled:
    sorting restores an order equal to the oracle's, and sorting a sorted
    table changes nothing."""
    from siminf_gb300 import workloads
    from siminf_gb300.events import sort_events
    m = workloads.seir_events(nodes=100_000, days=60, transfers=50_000)
    ev = {k: np.asarray(v) for k, v in m.events.items()}
    rng = np.random.default_rng(9)
    perm = rng.permutation(len(ev["time"]))
    shuffled = {k: v[perm] for k, v in ev.items()}
    got = sort_events(shuffled)
    want = ref.sort_events(shuffled)
    for k in ref.COLUMNS:
        assert np.array_equal(got[k], want[k]), k
    again = sort_events(got)
    for k in ref.COLUMNS:
        assert np.array_equal(again[k], got[k]), k
