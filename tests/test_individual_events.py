"""Cleaning of individual-based event data (SimInf_individual_events,
src/misc/SimInf_individual_events.c; individual_events(),
R/SimInf_individual_events.R:383-436).

CPU: the oracle's restatement against the reference's own test cases
(tests/individual_events.R, lifted into tests/golden/individual_events.json)
and against the reference's C file compiled unmodified (oracle/_ref, where
it was built), plus the host-side checks and their messages.  GPU: the
device path, bit-exact against the oracle on the golden cases, on random
tables with deep searches and on a table larger than L2, and its error for
an invalid event type."""
import datetime
import json
import os

import numpy as np
import pytest

from oracle import oracle
from siminf_gb300 import individual as I
from siminf_gb300.workloads import livestock_register

HERE = os.path.dirname(os.path.abspath(__file__))
NA = I.NA


def golden_cases():
    with open(os.path.join(HERE, "golden", "individual_events.json")) as f:
        return json.load(f)["cases"]


def normalise(col, values):
    out = []
    for v in (values.tolist() if hasattr(values, "tolist") else values):
        if isinstance(v, dict):
            v = v["date"]
        elif col == "dest" and v == NA:
            v = None                          # R's NA_integer_ in an int32 column
        elif col == "time" and not isinstance(v, (int, str)):
            v = str(v)
        out.append(v)
    return out


def compare(out, expected, time_dates):
    for col in ("id", "event", "time", "node", "dest"):
        got = out[col]
        if col == "time" and time_dates:
            got = [str(np.datetime64(v, "D")) for v in got]
        assert normalise(col, got) == normalise(col, expected[col]), col


def random_table(rng, n_ind, max_events, n_nodes, t_max):
    """Sorted, de-duplicated int32 columns of random individuals: few nodes
    and times make long, tied and inconsistent paths likely."""
    m = rng.integers(1, max_events + 1, size=n_ind)
    n = int(m.sum())
    id_ = np.repeat(np.arange(1, n_ind + 1), m)
    event = rng.choice(np.array([0, 1, 3]), size=n, p=[0.25, 0.25, 0.5])
    time = rng.integers(0, t_max, size=n)
    node = rng.integers(1, n_nodes + 1, size=n)
    dest = np.where(event == 3, rng.integers(1, n_nodes + 1, size=n), NA)
    dkey = np.where(dest == NA, np.int64(1) << 40, dest)
    o = np.lexsort((dkey, node, event, time, id_))
    cols = [np.asarray(c)[o] for c in (id_, event, time, node, dest)]
    same = np.ones(n - 1, dtype=bool)
    for c in cols:
        same &= c[1:] == c[:-1]
    first = np.concatenate(([True], ~same))
    return [np.ascontiguousarray(c[first], dtype=np.int32) for c in cols]


# ---------------------------------------------------------------- CPU ---

def test_golden_cases_through_the_oracle():
    cases = golden_cases()
    assert len(cases) >= 20
    for c in cases:
        prep = I.prepare(c["input"])
        keep, bad = oracle.individual_events(*prep.keys)
        assert bad == -1
        compare(I.finish(prep, keep), c["expected"], prep.time_dates)


def test_oracle_matches_the_reference_c_file():
    if not oracle.ref_available():
        pytest.skip("reference build not available")
    rng = np.random.default_rng(11)
    total = 0
    for trial in range(150):
        cols = random_table(rng, int(rng.integers(1, 40)), int(rng.integers(1, 16)),
                            int(rng.integers(1, 5)), int(rng.integers(1, 12)))
        k1, bad = oracle.individual_events(*cols, threads=2)
        k2, msg = oracle.ref_individual_events(*cols, threads=2)
        assert bad == -1 and msg is None
        assert np.array_equal(k1, k2), trial
        total += len(k1)
    assert total > 5000


def test_oracle_invalid_event_matches_the_reference_message():
    cols = random_table(np.random.default_rng(3), 4, 5, 3, 5)
    cols[1][2] = 2
    keep, bad = oracle.individual_events(*cols)
    assert bad == 2 and not keep.any()
    if oracle.ref_available():
        _, msg = oracle.ref_individual_events(*cols)
        assert msg == "'event[3]' is invalid."


def test_oracle_empty_and_single():
    z = [np.zeros(0, np.int32)] * 5
    keep, bad = oracle.individual_events(*z)
    assert len(keep) == 0 and bad == -1
    one = [np.array([v], np.int32) for v in (1, 3, 1, 1, 2)]
    assert oracle.individual_events(*one)[0].tolist() == [1]


@pytest.mark.parametrize("events, message", [
    ({"id": [1], "event": [1], "time": [1], "node": [1]}, "Missing columns in 'events'."),
    ({"id": [1, None], "event": [1, 0], "time": [1, 2], "node": [1, 1], "dest": [0, 0]},
     "'id' must be an integer or character vector with non-NA values."),
    ({"id": [1.5], "event": [1], "time": [1], "node": [1], "dest": [0]},
     "'id' must be an integer or character vector with non-NA values."),
    ({"id": [1], "event": [2], "time": [1], "node": [1], "dest": [0]},
     "'event' must be an integer or character vector with non-NA values."),
    ({"id": [1], "event": ["intTrans"], "time": [1], "node": [1], "dest": [0]},
     "'event' type must be 'enter', 'exit', or 'extTrans'."),
    ({"id": [1], "event": [1], "time": [1.2], "node": [1], "dest": [0]},
     "'time' must be an integer or character vector with non-NA values."),
    ({"id": [1], "event": [3], "time": [1], "node": [1], "dest": [None]},
     "'node' or 'dest' contain NA values."),
    ({"id": [1], "event": [3], "time": [1], "node": [1.1], "dest": [2]},
     "'node' and 'dest' must both be integer or character."),
    ({"id": [1], "event": [3], "time": [1], "node": [1], "dest": ["2"]},
     "'node' and 'dest' must both be integer or character."),
])
def test_host_checks_give_the_reference_messages(events, message):
    with pytest.raises(ValueError) as e:
        I.prepare(events)
    assert str(e.value) == message


def test_golden_rejections():
    """Every literal table tests/individual_events.R:84-330 expects
    individual_events() to reject, with its message."""
    with open(os.path.join(HERE, "golden", "individual_events.json")) as f:
        errors = json.load(f)["errors"]
    assert len(errors) >= 10
    for case in errors:
        with pytest.raises(ValueError) as e:
            I.prepare(case["input"])
        assert str(e.value) == case["message"], case["line"]
        # the same table as numpy arrays where numpy keeps the R types
        arrays = {k: np.array(v) for k, v in case["input"].items()}
        if all(a.dtype.kind in "iufbU" for a in arrays.values()):
            with pytest.raises(ValueError) as e:
                I.prepare(arrays)
            assert str(e.value) == case["message"], case["line"]


def test_prepare_orders_and_removes_repeats():
    ev = {"id": [2, 1, 1, 1], "event": [1, 3, 1, 3], "time": [5, 2, 1, 2],
          "node": [4, 1, 1, 1], "dest": [9, 2, 7, 2]}
    p = I.prepare(ev)
    ids, events, times, nodes, dests = (k.tolist() for k in p.keys)
    assert ids == [1, 1, 2] and events == [1, 3, 1] and times == [1, 2, 5]
    assert dests == [NA, 2, NA]              # dest is NA except for transfers
    assert p.rows.tolist() == [2, 1, 0]


def test_vectorised_and_elementwise_paths_agree():
    rng = np.random.default_rng(21)
    for trial in range(20):
        cols = random_table(rng, int(rng.integers(1, 300)), 8, 5, 30)
        n = len(cols[0])
        pick = rng.permutation(np.concatenate((np.arange(n),
                                               rng.integers(0, n, size=n // 3))))  # repeats
        ev = dict(zip(("id", "event", "time", "node", "dest"), (c[pick] for c in cols)))
        ev["time"] = ev["time"].astype(np.float64)            # numeric columns of mixed types
        ev["dest"] = np.where(ev["event"] == 3, ev["dest"], np.nan)
        a = I.prepare(ev)
        b = I.prepare({k: [None if isinstance(x, float) and np.isnan(x) else x
                           for x in v.tolist()] for k, v in ev.items()}, elementwise=True)
        assert a.arrays and not b.arrays
        assert np.array_equal(a.rows, b.rows)
        for x, y in zip(a.keys, b.keys):
            assert np.array_equal(x, y)
        for x, y in zip(a.keys, cols):
            assert np.array_equal(x, y)                       # sorted, repeats gone


def test_dates_with_character_ids():
    """Date times with character ids (or a list of datetime.date with
    numeric ids) take the value-by-value path and are read as R's Date
    columns: days since 1970-01-01, the same keys as numeric days."""
    ids = ["b", "a", "a", "b"]
    days = np.array(["2020-01-05", "2020-01-01", "2020-02-01", "2020-01-09"],
                    dtype="datetime64[D]")
    base = {"id": ids, "event": [1, 1, 0, 0], "node": [1, 2, 2, 1], "dest": [None] * 4}
    a = I.prepare(dict(base, time=days))
    assert a.time_dates
    b = I.prepare(dict(base, time=[d.astype(object) for d in days]))
    c = I.prepare(dict(base, time=days.astype(np.int64).tolist()))
    for x, y, z in zip(a.keys, b.keys, c.keys):
        assert np.array_equal(x, y) and np.array_equal(x, z)
    d = I.prepare({"id": [2, 1], "event": [1, 0], "node": [1, 1], "dest": [0, 0],
                   "time": [datetime.date(2020, 1, 2), datetime.date(2020, 1, 1)]})
    assert d.time_dates and d.keys[2].tolist() == [18262, 18263]


def test_character_nodes_with_numeric_dest_rejected():
    """No transfers, character nodes and a numeric dest column: R's check
    sees a numeric dest and rejects the table."""
    with pytest.raises(ValueError, match="'node' and 'dest' must both be integer or character."):
        I.prepare({"id": [1, 1], "event": ["enter", "exit"], "time": [1, 2],
                   "node": ["x", "x"], "dest": [0, 0]})


def test_order_is_rs_order():
    rng = np.random.default_rng(4)
    for trial in range(30):
        n = int(rng.integers(1, 4000))
        keys = [rng.integers(-5, 5, n), rng.integers(-2 ** 40, 2 ** 40, n),
                rng.integers(0, 3, n), rng.integers(0, 2 ** 31, n), rng.integers(0, 2, n)]
        keys = [k.astype(np.int64) for k in keys]
        assert np.array_equal(I._order(keys), np.lexsort(tuple(reversed(keys))))
    sorted_keys = [np.sort(rng.integers(0, 9, 500)).astype(np.int64)]
    assert np.array_equal(I._order(sorted_keys), np.arange(500))


def test_vectorised_checks_and_rs_whole_numbers():
    base = {"id": np.array([1, 1]), "event": np.array([1, 3]), "time": np.array([1.0, 2.0]),
            "node": np.array([1, 1]), "dest": np.array([np.nan, 2.0])}
    for col, value, message in [
            ("id", np.array([1.0, np.nan]),
             "'id' must be an integer or character vector with non-NA values."),
            ("event", np.array([1, 2]),
             "'event' must be an integer or character vector with non-NA values."),
            ("time", np.array([1.0, 2.5]),
             "'time' must be an integer or character vector with non-NA values."),
            ("dest", np.array([0.0, np.nan]), "'node' or 'dest' contain NA values."),
            ("node", np.array([1.0, 1.5]),
             "'node' and 'dest' must both be integer or character.")]:
        ev = dict(base, **{col: value})
        with pytest.raises(ValueError) as e:
            I.prepare(ev)
        assert str(e.value) == message
    # within sqrt(eps) of a whole number counts as whole, and is truncated
    ev = dict(base, time=np.array([1.0, 2.9999999999]))
    assert I.prepare(ev).keys[2].tolist() == [1, 2]
    ev = {k: v.tolist() for k, v in ev.items()}
    ev["dest"] = [None, 2.0]
    assert I.prepare(ev, elementwise=True).keys[2].tolist() == [1, 2]


def test_boundary_rejects_bad_tables_before_any_device_call():
    """Argument checks of siminf_gpu_individual_events run on the host,
    before any CUDA call, so they answer without a GPU."""
    import ctypes as C
    from siminf_gb300 import abi, native
    L = native.lib()
    st = abi.ReduceStats()
    nul = C.POINTER(C.c_int)()
    assert L.siminf_gpu_individual_events(-1, nul, nul, nul, nul, nul, nul, None,
                                          C.byref(st)) == -9
    assert "invalid individual event table" in native.last_status().message.decode()
    assert L.siminf_gpu_individual_events(1 << 31, nul, nul, nul, nul, nul, nul, None,
                                          None) == -9
    assert L.siminf_gpu_individual_events(3, nul, nul, nul, nul, nul, nul, None, None) == -9
    assert L.siminf_gpu_individual_events(0, nul, nul, nul, nul, nul, nul, None, None) == 0


def test_livestock_generator_is_sorted_and_mostly_consistent():
    cols = livestock_register(2000, 50, seed=1)
    keep, bad = oracle.individual_events(*cols)
    assert bad == -1
    assert 0.8 < keep.mean() <= 1.0


# ---------------------------------------------------------------- GPU ---

@pytest.mark.gpu
def test_gpu_golden_cases():
    for c in golden_cases():
        prep = I.prepare(c["input"])
        out = I.individual_events(c["input"])
        compare(out, c["expected"], prep.time_dates)


@pytest.mark.gpu
@pytest.mark.parametrize("seed, n_ind, max_events, n_nodes, t_max", [
    (1, 40, 12, 3, 8),        # deep searches, many ties
    (2, 2000, 6, 4, 20),
    (3, 5, 28, 2, 30),        # long single histories
    (4, 30000, 4, 40, 400),
])
def test_gpu_matches_oracle_random(seed, n_ind, max_events, n_nodes, t_max):
    cols = random_table(np.random.default_rng(seed), n_ind, max_events, n_nodes, t_max)
    want, _ = oracle.individual_events(*cols, threads=4)
    got = I.longest_paths(*cols)
    assert np.array_equal(got, want)


@pytest.mark.gpu
def test_gpu_matches_oracle_larger_than_l2():
    # ~10^7 events: the five int32 columns hold ~200 MB, above the 129 MB L2
    cols = livestock_register(2_500_000, 200_000, seed=7)
    assert len(cols[0]) > 9_000_000
    want, _ = oracle.individual_events(*cols, threads=os.cpu_count() or 1)
    got, st = I.longest_paths(*cols, stats=True)
    assert np.array_equal(got, want)
    assert st.ms_kernel > 0 and st.bytes_read == 20 * len(cols[0])


@pytest.mark.gpu
def test_gpu_invalid_event_type_is_the_reference_error():
    from siminf_gb300 import abi, native
    cols = random_table(np.random.default_rng(5), 10, 5, 3, 5)
    cols[1][3] = 2
    cols[1][7] = 5
    with pytest.raises(abi.SimInfError) as e:
        I.longest_paths(*cols)
    assert e.value.code == -3
    assert "'event[4]' is invalid." in str(e.value)
    assert native.last_status().event_index == 3


def exploding_individual(layers, who=2):
    """One individual whose search has 2^layers paths and no pruning: it
    enters at node 1, then at each layer moves to node a or node b and from
    either on to the next layer's first node; its one exit is at a node no
    path reaches, so no path is kept longer than the lone exit."""
    rows = [(who, 1, 0, 1, NA)]
    t, at = 1, 1
    for k in range(layers):
        a, b, nxt = 1000 + 3 * k, 1001 + 3 * k, 1002 + 3 * k
        rows += [(who, 3, t + 1, at, a), (who, 3, t + 1, at, b),
                 (who, 3, t + 2, a, nxt), (who, 3, t + 2, b, nxt)]
        t, at = t + 2, nxt
    rows.append((who, 0, t + 5, 999, NA))
    rows.sort(key=lambda r: (r[0], r[2], r[1], r[3], r[4]))
    return [np.array(c, np.int32) for c in zip(*rows)]


@pytest.mark.gpu
def test_gpu_search_budget_stops_an_exploding_individual():
    """An individual with 2^20 paths and an unreachable exit: with a budget
    of 10^4 steps its search gives up, the call returns the timeout error
    naming its first event, and the other individuals' keep is the
    oracle's; with the default budget a small case of the same shape
    finishes and equals the oracle."""
    from siminf_gb300 import abi, native
    good = random_table(np.random.default_rng(8), 40, 8, 6, 30)
    bad = exploding_individual(20, who=int(good[0].max()) + 1)
    cols = [np.concatenate([g, b]) for g, b in zip(good, bad)]
    want, _ = oracle.individual_events(*good)
    n_good = len(good[0])
    keep = np.zeros(len(cols[0]), np.int32)
    pi = lambda a: a.ctypes.data_as(__import__("ctypes").POINTER(__import__("ctypes").c_int))
    code = native.lib().siminf_gpu_individual_events_ex(
        len(cols[0]), *[pi(c) for c in cols], pi(keep), 10_000, None, None)
    assert code == -33
    st = native.last_status()
    assert st.event_index == n_good
    assert np.array_equal(keep[:n_good], want)
    assert not keep[n_good:].any()
    small = exploding_individual(6)
    got = I.longest_paths(*small)
    assert np.array_equal(got, oracle.individual_events(*small)[0])
    with pytest.raises(abi.SimInfError) as e:
        I.longest_paths(*small, max_steps=50)
    assert e.value.code == -33


@pytest.mark.gpu
def test_gpu_empty_and_single():
    z = [np.zeros(0, np.int32)] * 5
    assert len(I.longest_paths(*z)) == 0
    for ev, keep in ((1, 1), (0, 1), (3, 1)):
        one = [np.array([v], np.int32) for v in (1, ev, 1, 1, 2 if ev == 3 else NA)]
        assert I.longest_paths(*one).tolist() == [keep]
