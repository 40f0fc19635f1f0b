"""Cleaning of individual-based event data, the counterpart of SimInf's
individual_events() (R/SimInf_individual_events.R:383-436) and of its C
core SimInf_individual_events (src/misc/SimInf_individual_events.c), which
here runs on the device through siminf_gpu_individual_events.

    ev = individual_events({"id": [...], "event": [...], "time": [...],
                            "node": [...], "dest": [...]})

The columns are checked with the reference's messages, coded (event names
'exit', 'enter', 'extTrans' to 0, 1, 3; character ids and nodes to factor
codes; character times to days since 1970-01-01), dest is set to NA except
for external transfers, the rows are ordered by (id, time, event, node,
dest) with NA last and exact duplicates removed, and the device keeps each
individual's longest consistent path.  The result holds the kept rows with
the caller's own id, node and dest values (None for NA); time comes back
as numpy datetime64[D] when it was given as dates.

Character ids and nodes are coded in code-point order, where R's factor()
sorts in the session's collation: the kept rows are the same, but
individuals can come out in another order for mixed-case names.
"""
import ctypes as C

import numpy as np

from . import abi, native

NA = np.iinfo(np.int32).min
EVENT_CODES = {"exit": 0, "enter": 1, "extTrans": 3}
EVENT_NAMES = {v: k for k, v in EVENT_CODES.items()}


def longest_paths(id, event, time, node, dest, stream=None, stats=False):
    """siminf_gpu_individual_events on sorted, de-duplicated int32 columns
    (dest NA = INT_MIN): keep, a 0/1 int32 array (with the ReduceStats when
    stats=True)."""
    cols = [np.ascontiguousarray(x, dtype=np.int32) for x in (id, event, time, node, dest)]
    n = len(cols[0])
    if any(len(c) != n for c in cols):
        raise ValueError("columns differ in length")
    keep = np.zeros(n, dtype=np.int32)
    st = abi.ReduceStats()
    pi = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))
    native.check(native.lib().siminf_gpu_individual_events(
        n, *[pi(c) for c in cols], pi(keep), stream, C.byref(st)))
    return (keep, st) if stats else keep


def _is_na(x):
    return x is None or (isinstance(x, float) and np.isnan(x))


def _kind(values):
    """'str', 'num' or 'empty' for the non-NA values of a column."""
    kinds = {isinstance(v, str) for v in values if not _is_na(v)}
    if not kinds:
        return "empty"
    if kinds == {True}:
        return "str"
    if kinds == {False}:
        return "num"
    return "mixed"


def _whole(values):
    try:
        return all(float(v) == int(float(v)) for v in values)
    except (TypeError, ValueError, OverflowError):
        return False


def _factor(values, levels):
    index = {v: k + 1 for k, v in enumerate(levels)}
    return np.array([NA if _is_na(v) else index[v] for v in values], dtype=np.int64)


def check_id(id):
    msg = "'id' must be an integer or character vector with non-NA values."
    if any(_is_na(v) for v in id):
        raise ValueError(msg)
    kind = _kind(id)
    if kind == "num" and _whole(id):
        return np.array([int(v) for v in id], dtype=np.int64)
    if kind == "str":
        return _factor(id, sorted(set(id)))
    if kind == "empty":
        return np.zeros(0, dtype=np.int64)
    raise ValueError(msg)


def check_event(event):
    msg = "'event' must be an integer or character vector with non-NA values."
    if any(_is_na(v) for v in event):
        raise ValueError(msg)
    kind = _kind(event)
    if kind == "num":
        if not _whole(event) or any(int(v) not in (0, 1, 3) for v in event):
            raise ValueError(msg)
        return np.array([int(v) for v in event], dtype=np.int64), False
    if kind == "str":
        if any(v not in EVENT_CODES for v in event):
            raise ValueError("'event' type must be 'enter', 'exit', or 'extTrans'.")
        return np.array([EVENT_CODES[v] for v in event], dtype=np.int64), True
    if kind == "empty":
        return np.zeros(0, dtype=np.int64), False
    raise ValueError(msg)


def check_time(time):
    msg = "'time' must be an integer or character vector with non-NA values."
    if any(_is_na(v) for v in time):
        raise ValueError(msg)
    kind = _kind(time)
    if kind == "num":
        if not _whole(time):
            raise ValueError(msg)
        return np.array([int(v) for v in time], dtype=np.int64), False
    if kind == "str":
        try:
            days = np.array(time, dtype="datetime64[D]").astype(np.int64)
        except ValueError:
            raise ValueError(msg)
        return days, True
    if kind == "empty":
        return np.zeros(0, dtype=np.int64), False
    raise ValueError(msg)


def check_nodes(event, node, dest):
    if any(_is_na(v) for v in node) or any(_is_na(d) for e, d in zip(event, dest) if e == 3):
        raise ValueError("'node' or 'dest' contain NA values.")
    msg = "'node' and 'dest' must both be integer or character."
    kn, kd = _kind(node), _kind(dest)
    if kn in ("num", "empty") and kd in ("num", "empty"):
        if not _whole(node) or not _whole([d for e, d in zip(event, dest) if e == 3]):
            raise ValueError(msg)
        to = lambda vs: np.array([NA if _is_na(v) else int(v) for v in vs], dtype=np.int64)
        return to(node), to(dest)
    if kn in ("str", "empty") and kd in ("str", "empty"):
        levels = sorted({v for v in list(node) + list(dest) if not _is_na(v)})
        return _factor(node, levels), _factor(dest, levels)
    raise ValueError(msg)


class Prepared:
    """The coded, ordered, de-duplicated columns of an individual event
    table (`keys`: id, event, time, node, dest as int32, dest NA =
    INT_MIN), the rows of the caller's table they came from, and what
    finish() needs to give the kept rows back in the caller's terms."""

    def __init__(self, raw, rows, keys, event_named, time_dates):
        self.raw, self.rows, self.keys = raw, rows, keys
        self.event_named, self.time_dates = event_named, time_dates


def prepare(events):
    """The host half of individual_events() (R/SimInf_individual_events.R:
    383-410): checks, coding, ordering and removal of exact repeats."""
    columns = ("id", "event", "time", "node", "dest")
    if not all(c in events for c in columns):
        raise ValueError("Missing columns in 'events'.")
    raw = {c: list(events[c]) for c in columns}
    n = len(raw["id"])
    if any(len(raw[c]) != n for c in columns):
        raise ValueError("columns differ in length")
    id_code = check_id(raw["id"])
    event, event_named = check_event(raw["event"])
    time, time_dates = check_time(raw["time"])
    raw["dest"] = [d if e == 3 else None for e, d in zip(event, raw["dest"])]
    node_code, dest_code = check_nodes(event, raw["node"], raw["dest"])

    # order(id, time, event, node, dest), NA last; then drop exact repeats
    dest_key = np.where(dest_code == NA, np.int64(1) << 40, dest_code)
    order = np.lexsort((dest_key, node_code, event, time, id_code))
    if n > 1:
        repeat = np.ones(n - 1, dtype=bool)
        for k in (id_code, time, event, node_code, dest_code):
            s = k[order]
            repeat &= s[1:] == s[:-1]
        order = order[np.concatenate(([True], ~repeat))]
    keys = [np.ascontiguousarray(k[order], dtype=np.int32)
            for k in (id_code, event, time, node_code, dest_code)]
    raw["event_code"], raw["time_code"] = event, time
    return Prepared(raw, order, keys, event_named, time_dates)


def finish(prep, keep):
    """The kept rows, in the caller's own values."""
    rows = prep.rows[np.asarray(keep).astype(bool)]
    raw, event, time = prep.raw, prep.raw["event_code"], prep.raw["time_code"]
    return {
        "id": [raw["id"][i] for i in rows],
        "event": ([EVENT_NAMES[int(event[i])] for i in rows] if prep.event_named
                  else event[rows].astype(np.int32)),
        "time": (time[rows].astype("datetime64[D]") if prep.time_dates
                 else time[rows].astype(np.int32)),
        "node": [raw["node"][i] for i in rows],
        "dest": [raw["dest"][i] for i in rows],
    }


def individual_events(events, stream=None):
    """individual_events(events): the kept rows of a table with the columns
    id, event, time, node and dest (a dict of sequences; None is NA), as a
    dict of columns ordered by (id, time, event, node, dest)."""
    prep = prepare(events)
    return finish(prep, longest_paths(*prep.keys, stream=stream))
