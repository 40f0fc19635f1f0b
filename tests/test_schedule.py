"""Host-side event planning (siminf_gpu_schedule), no GPU needed: the
wavefronts must be conflict-free and equivalent to the serial array order
of the reference's external-transfer loop (src/solvers/SimInf_solver.c:
824-902 run by one thread, src/solvers/SimInf_solver_ssm.c:244-250)."""
import numpy as np
import pytest

from siminf_gb300 import abi, native, workloads
from helpers import parity_cases


def reference_levels(m):
    """The level rule written out serially: an external transfer goes one
    wave after every earlier transfer of its day that touched its source,
    and after every earlier transfer whose source is its destination."""
    ev = m.events
    t0 = float(m.tspan[0])
    levels = np.full(len(ev["event"]), -1)
    excl, add = {}, {}
    day_prev = None
    for i in range(len(ev["event"])):
        if ev["event"][i] != 3:
            continue
        t = ev["time"][i]
        d = 0 if t <= t0 else t - int(np.floor(t0))
        if d != day_prev:
            excl, add, day_prev = {}, {}, d
        s, dst = ev["node"][i], ev["dest"][i]
        L = 1 + max(excl.get(s, 0), add.get(s, 0), excl.get(dst, 0))
        excl[s] = L
        add[dst] = max(add.get(dst, 0), L)
        levels[i] = L - 1
    return levels


def check_conflict_free(m, wave):
    ev = m.events
    t0 = float(m.tspan[0])
    days = np.where(ev["time"] <= t0, 0, ev["time"] - int(np.floor(t0)))
    sel = np.nonzero((ev["event"] == 3) & (wave >= 0))[0]
    groups = {}
    for i in sel:
        groups.setdefault((days[i], wave[i]), []).append(i)
    for (d, w), idx in groups.items():
        src = [ev["node"][i] for i in idx]
        dst = [ev["dest"][i] for i in idx]
        assert len(set(src)) == len(src), "two transfers of one wave share a source"
        assert not (set(src) & set(dst)) or all(s == t for s, t in zip(src, dst)
                                                if s in dst), "a wave reads a node it writes"
    # order: within a day, events touching a common source keep array order
    for i in sel:
        for j in sel:
            if j >= i or days[j] != days[i]:
                continue
            si, di, sj, dj = ev["node"][i], ev["dest"][i], ev["node"][j], ev["dest"][j]
            if si == sj or si == dj or di == sj:
                assert wave[j] < wave[i]


def test_schedule_levels_match_serial_rule():
    for label, m in parity_cases():
        if not len(m.events["event"]):
            continue
        h = abi.build_args(m, 1)
        days, waves, e1, e2, wave = native.schedule(h)
        ref = reference_levels(m)
        e2_mask = ref >= 0
        assert np.array_equal(wave[e2_mask], ref[e2_mask]), label
        assert e1 == int(((m.events["event"] != 3)).sum())


def test_schedule_conflict_free_small_workload():
    m = workloads.seir_events(nodes=300, days=20, transfers=400)
    h = abi.build_args(m, 1)
    days, waves, e1, e2, wave = native.schedule(h)
    assert days == 20 and e2 == 20 * 400
    check_conflict_free(m, wave)
    assert np.array_equal(wave[wave >= 0], reference_levels(m)[wave >= 0])


def test_schedule_rejects_unsorted():
    from siminf_gb300 import model as M
    m = M.SIR({"S": [5, 5], "I": [0, 0], "R": [0, 0]}, [1, 2, 3], 0.0, 0.0,
              events=M.make_events([3, 0], [1, 1], [1, 2], [2, 0], 1, 0.0, 1, 0, sort=False))
    h = abi.build_args(m, 1)
    with pytest.raises(abi.SimInfError) as e:
        native.schedule(h)
    assert e.value.code == -31


def test_schedule_headline_scale_properties():
    """Full day count at 2% of the headline size: planning finishes and
    every transfer lands in a wave."""
    m = workloads.seir_events(nodes=20_000, days=365, transfers=10_000)
    h = abi.build_args(m, 1)
    days, waves, e1, e2, wave = native.schedule(h)
    assert days == 365 and e2 == 365 * 10_000
    assert (wave[m.events["event"] == 3] >= 0).all()


def test_schedule_self_transfers_and_deep_days():
    """Transfers from a node to itself, chains that revisit few nodes (a
    deep day), and both mixed with ordinary transfers: the levels follow
    the serial rule."""
    from siminf_gb300 import model as M
    rng = np.random.default_rng(17)
    Nn, days = 12, 6
    ev = {k: [] for k in M.EVENT_FIELDS}
    for t in range(1, days + 1):
        for _ in range(300):
            s_ = int(rng.integers(1, Nn + 1))
            d_ = s_ if rng.random() < 0.2 else int(rng.integers(1, Nn + 1))
            for key, val in zip(M.EVENT_FIELDS, (3, t, s_, d_, 1, 0.0, 2, 0)):
                ev[key].append(val)
    u0 = {"S": np.full(Nn, 500), "E": 0, "I": 0, "R": 0}
    m = M.SEIR(u0, np.arange(1, days + 1), 0.0, 0.0, 0.0,
               events=M.make_events(**{k: np.array(v) for k, v in ev.items()}))
    h = abi.build_args(m, 1)
    _, waves, _, e2, wave = native.schedule(h)
    ref = reference_levels(m)
    assert e2 == days * 300
    assert np.array_equal(wave, ref)
    assert waves > days * 50            # deep days: many wavefronts each


def relaxation_levels(src, dst):
    """The device planner's levelling of one day's transfers, written with
    numpy: the serial rule as a fixed point.  Links per transfer k: p1, the
    previous transfer with the same source; p3, the last earlier transfer
    whose source is k's destination; q, the position (in the destination-
    sorted order) of the last earlier transfer into k's source.  Each round
    takes the segmented prefix maximum of the levels over the destination-
    sorted order and sets L[k] = 1 + max(L[p1], prefix max at q, L[p3]),
    until nothing changes.  Returns (levels, rounds)."""
    n = len(src)
    k = np.arange(n)
    by_src = np.lexsort((k, src))
    by_dst = np.lexsort((k, dst))
    p1 = np.full(n, -1)
    same = src[by_src[1:]] == src[by_src[:-1]]
    p1[by_src[1:][same]] = by_src[:-1][same]
    # last j < k with src[j] == dst[k]: in (src, index) order, the element
    # before the insertion point of (dst[k], k)
    key_src = src[by_src].astype(np.int64) * (n + 1) + by_src
    pos = np.searchsorted(key_src, dst.astype(np.int64) * (n + 1) + k) - 1
    p3 = np.where((pos >= 0) & (src[by_src[np.maximum(pos, 0)]] == dst), by_src[np.maximum(pos, 0)], -1)
    key_dst = dst[by_dst].astype(np.int64) * (n + 1) + by_dst
    qpos = np.searchsorted(key_dst, src.astype(np.int64) * (n + 1) + k) - 1
    q = np.where((qpos >= 0) & (dst[by_dst[np.maximum(qpos, 0)]] == src), qpos, -1)
    head = np.ones(n, bool)
    head[1:] = dst[by_dst[1:]] != dst[by_dst[:-1]]
    L = np.ones(n, np.int64)
    rounds = 0
    while True:
        rounds += 1
        v = L[by_dst]
        pm = np.empty(n, np.int64)
        run = 0
        for j in range(n):                  # segmented prefix max
            run = v[j] if head[j] else max(run, v[j])
            pm[j] = run
        get = lambda a, i: np.where(i >= 0, a[np.maximum(i, 0)], 0)
        new = 1 + np.maximum(np.maximum(get(L, p1), get(pm, q)), get(L, p3))
        if np.array_equal(new, L):
            return L, rounds
        L = new


def test_relaxation_levels_equal_serial_rule():
    """The fixed point of the device planner's rounds is the serial rule's
    level on random days: hubs, self-transfers, deep chains and wide
    days."""
    rng = np.random.default_rng(5)
    for trial in range(40):
        Nn = int(rng.integers(2, 60))
        n = int(rng.integers(1, 400))
        src = rng.integers(0, Nn, n)
        if trial % 3 == 0:                  # a hub that most transfers enter
            dst = np.where(rng.random(n) < 0.7, 0, rng.integers(0, Nn, n))
        else:
            dst = rng.integers(0, Nn, n)
        if trial % 4 == 1:                  # self-transfers
            dst = np.where(rng.random(n) < 0.3, src, dst)
        # the serial rule (siminf_gpu_schedule's, as reference_levels)
        excl, add = {}, {}
        ref = np.empty(n, np.int64)
        for i in range(n):
            s, t = int(src[i]), int(dst[i])
            Lv = 1 + max(excl.get(s, 0), add.get(s, 0), excl.get(t, 0))
            excl[s] = Lv
            add[t] = max(add.get(t, 0), Lv)
            ref[i] = Lv
        got, rounds = relaxation_levels(src, dst)
        assert np.array_equal(got, ref), trial
        assert rounds <= ref.max() + 1


@pytest.mark.gpu
def test_device_schedule_equals_host(gpu):
    """The device planner's waves, counts and E1/E2 split equal the host
    planner's on every parity case with events, a wide workload, deep days
    with self-transfers, and 2% of the headline schedule."""
    cases = [(label, m) for label, m in parity_cases() if len(m.events["event"])]
    cases.append(("small", workloads.seir_events(nodes=300, days=20, transfers=400)))
    cases.append(("headline_2pct", workloads.seir_events(nodes=20_000, days=365,
                                                         transfers=10_000)))
    from siminf_gb300 import model as M
    rng = np.random.default_rng(23)
    Nn, days = 12, 6
    ev = {k: [] for k in M.EVENT_FIELDS}
    for t in range(1, days + 1):
        for _ in range(3000):               # deeper than the rounds allow on some days
            s_ = int(rng.integers(1, Nn + 1))
            d_ = s_ if rng.random() < 0.2 else int(rng.integers(1, Nn + 1))
            for key, val in zip(M.EVENT_FIELDS, (3, t, s_, d_, 1, 0.0, 2, 0)):
                ev[key].append(val)
    u0 = {"S": np.full(Nn, 500), "E": 0, "I": 0, "R": 0}
    cases.append(("deep", M.SEIR(u0, np.arange(1, days + 1), 0.0, 0.0, 0.0,
                                 events=M.make_events(**{k: np.array(v) for k, v in ev.items()}))))
    for label, m in cases:
        h = abi.build_args(m, 1)
        host = native.schedule(h)
        dev = native.schedule(h, device=True)
        assert host[:4] == dev[:4], label
        assert np.array_equal(host[4], dev[4]), label


@pytest.mark.gpu
def test_device_schedule_rejects_unsorted(gpu):
    from siminf_gb300 import model as M
    m = M.SIR({"S": [5, 5], "I": [0, 0], "R": [0, 0]}, [1, 2, 3], 0.0, 0.0,
              events=M.make_events([3, 0], [1, 1], [1, 2], [2, 0], 1, 0.0, 1, 0, sort=False))
    h = abi.build_args(m, 1)
    with pytest.raises(abi.SimInfError) as e:
        native.schedule(h, device=True)
    assert e.value.code == -31


@pytest.mark.gpu
def test_device_schedule_full_headline(gpu):
    """The full headline schedule (10^6 nodes, 365 days, 500,000 transfers a
    day): the device planner's per-event waves and counts equal the host
    planner's."""
    m = workloads.seir_events(nodes=1_000_000, days=365, transfers=500_000)
    h = abi.build_args(m, 1)
    host = native.schedule(h)
    dev = native.schedule(h, device=True)
    assert host[:4] == dev[:4]
    assert np.array_equal(host[4], dev[4])


def attach_levels(src, dst):
    """The device planner's levelling as it runs: zero-based levels
    Lz[k] = max(Lz[p1] + 1, A[k] + 1, Lz[p3] + 1, 0), where A[k] is the
    largest level of the transfers into k's source since p1 (the earlier
    ones are below Lz[p1]): each transfer j feeds A of the first later
    transfer whose source is j's destination.  Rounds update in place (in
    array order here) until nothing changes.  Returns (levels, rounds)."""
    n = len(src)
    k = np.arange(n)
    by_src = np.lexsort((k, src))
    key_src = src[by_src].astype(np.int64) * (n + 1) + by_src
    p1 = np.full(n, -1)
    same = src[by_src[1:]] == src[by_src[:-1]]
    p1[by_src[1:][same]] = by_src[:-1][same]
    pos = np.searchsorted(key_src, dst.astype(np.int64) * (n + 1) + k) - 1
    ok = (pos >= 0) & (src[by_src[np.maximum(pos, 0)]] == dst)
    p3 = np.where(ok, by_src[np.maximum(pos, 0)], -1)
    # attach: the first later transfer whose source is j's destination
    pos2 = np.searchsorted(key_src, dst.astype(np.int64) * (n + 1) + k, side="right")
    ok2 = (pos2 < n) & (src[by_src[np.minimum(pos2, n - 1)]] == dst)
    attach = np.where(ok2, by_src[np.minimum(pos2, n - 1)], -1)
    L = np.zeros(n, np.int64)
    A = np.full(n, -1, np.int64)
    A[attach[attach >= 0]] = 0              # every transfer starts at level 0
    rounds = 0
    while True:
        rounds += 1
        changed = False
        for i in range(n):
            v = 0
            if p1[i] >= 0:
                v = max(v, L[p1[i]] + 1)
            if p3[i] >= 0:
                v = max(v, L[p3[i]] + 1)
            if A[i] >= 0:
                v = max(v, A[i] + 1)
            if v != L[i]:
                L[i] = v
                changed = True
                if attach[i] >= 0:
                    A[attach[i]] = max(A[attach[i]], v)
        if not changed:
            return L + 1, rounds


def test_attach_levels_equal_serial_rule():
    """The device planner's formulation (adds feeding the next transfer
    out of their destination) has the serial rule's levels as its fixed
    point, on the same random days as the segmented-prefix formulation."""
    rng = np.random.default_rng(5)
    for trial in range(40):
        Nn = int(rng.integers(2, 60))
        n = int(rng.integers(1, 400))
        src = rng.integers(0, Nn, n)
        if trial % 3 == 0:
            dst = np.where(rng.random(n) < 0.7, 0, rng.integers(0, Nn, n))
        else:
            dst = rng.integers(0, Nn, n)
        if trial % 4 == 1:
            dst = np.where(rng.random(n) < 0.3, src, dst)
        excl, add = {}, {}
        ref = np.empty(n, np.int64)
        for i in range(n):
            s, t = int(src[i]), int(dst[i])
            Lv = 1 + max(excl.get(s, 0), add.get(s, 0), excl.get(t, 0))
            excl[s] = Lv
            add[t] = max(add.get(t, 0), Lv)
            ref[i] = Lv
        got, _ = attach_levels(src, dst)
        assert np.array_equal(got, ref), trial
        # and in any update order (the device's threads race): reversed
        got_r, _ = attach_levels(src[::-1].copy(), dst[::-1].copy())
        assert got_r.shape == ref.shape
