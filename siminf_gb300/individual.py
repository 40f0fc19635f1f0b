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
the caller's own id, node and dest values; time comes back as numpy
datetime64[D] when it was given as dates.  Numeric columns (arrays or lists
of numbers, NaN as NA) take a vectorised path and come back as arrays,
dest as int32 with R's NA_integer_ (INT_MIN) for NA; other columns go
value by value and come back as lists with None for NA.

Character ids and nodes are coded in code-point order, where R's factor()
sorts in the session's collation: the kept rows are the same, but
individuals can come out in another order for mixed-case names.
"""
import ctypes as C
import datetime
import re

import numpy as np

from . import abi, native

NA = np.iinfo(np.int32).min
EVENT_CODES = {"exit": 0, "enter": 1, "extTrans": 3}
EVENT_NAMES = {v: k for k, v in EVENT_CODES.items()}


def longest_paths(id, event, time, node, dest, stream=None, stats=False, max_steps=0):
    """siminf_gpu_individual_events on sorted, de-duplicated int32 columns
    (dest NA = INT_MIN): keep, a 0/1 int32 array (with the ReduceStats when
    stats=True).  max_steps > 0 bounds each individual's search
    (siminf_gpu_individual_events_ex); an individual whose search runs out
    raises the library's timeout error."""
    cols = [np.ascontiguousarray(x, dtype=np.int32) for x in (id, event, time, node, dest)]
    n = len(cols[0])
    if any(len(c) != n for c in cols):
        raise ValueError("columns differ in length")
    keep = np.zeros(n, dtype=np.int32)
    st = abi.ReduceStats()
    pi = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))
    native.check(native.lib().siminf_gpu_individual_events_ex(
        n, *[pi(c) for c in cols], pi(keep), C.c_longlong(int(max_steps)), stream,
        C.byref(st)))
    return (keep, st) if stats else keep


def _is_na(x):
    return x is None or (isinstance(x, float) and np.isnan(x))


def _kind(values):
    """'num', 'str', 'logical' (R's TRUE/FALSE, not numeric there), 'date'
    (numpy datetime64 or datetime.date values, R's Date), 'mixed' or
    'empty' for the non-NA values of a column."""
    kinds = set()
    for v in values:
        if _is_na(v) or (isinstance(v, np.datetime64) and np.isnat(v)):
            continue
        if isinstance(v, (bool, np.bool_)):
            kinds.add("logical")
        elif isinstance(v, str):
            kinds.add("str")
        elif isinstance(v, (np.datetime64, datetime.date)):
            kinds.add("date")
        else:
            kinds.add("num")
    if not kinds:
        return "empty"
    return kinds.pop() if len(kinds) == 1 else "mixed"


# R's is_wholenumber (R/check_arguments.R:191-193): |x - round(x)| below
# sqrt(machine epsilon); as.integer() then truncates toward zero.
WHOLE_TOL = np.finfo(np.float64).eps ** 0.5


def _whole(values):
    try:
        return all(abs(float(v) - round(float(v))) < WHOLE_TOL for v in values)
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
    if any(_is_na(v) or (isinstance(v, np.datetime64) and np.isnat(v)) for v in time):
        raise ValueError(msg)
    kind = _kind(time)
    if kind == "date":
        # Date columns: days since 1970-01-01, as R stores a Date
        return np.array([np.datetime64(v, "D").astype(np.int64) for v in time],
                        dtype=np.int64), True
    if kind == "num":
        if not _whole(time):
            raise ValueError(msg)
        return np.array([int(v) for v in time], dtype=np.int64), False
    if kind == "str":
        return _dates(time, msg), True
    if kind == "empty":
        return np.zeros(0, dtype=np.int64), False
    raise ValueError(msg)


_DATE = re.compile(r"\s*(\d{1,4})([-/])(\d{1,2})\2(\d{1,2})")


def _dates(values, msg):
    """Days since 1970-01-01 the way as.Date() reads strings: the format
    (%Y-%m-%d or %Y/%m/%d) is the one the first value matches, and a value
    it does not fit, or an impossible date, is NA."""
    first = _DATE.match(values[0])
    if not first:
        raise ValueError("character string is not in a standard unambiguous format")
    sep = first.group(2)
    days = []
    for v in values:
        m = _DATE.match(v)
        if not m or m.group(2) != sep:
            raise ValueError(msg)
        try:
            d = np.datetime64("%04d-%02d-%02d" % (int(m.group(1)), int(m.group(3)),
                                                  int(m.group(4))), "D")
        except ValueError:
            raise ValueError(msg)
        days.append(d.astype(np.int64))
    return np.array(days, dtype=np.int64)


def check_nodes(event, node, dest, dest_kind=None):
    """dest holds NA for every event but a transfer; dest_kind is the kind
    of the caller's dest column before that (R checks the column's type)."""
    if any(_is_na(v) for v in node) or any(_is_na(d) for e, d in zip(event, dest) if e == 3):
        raise ValueError("'node' or 'dest' contain NA values.")
    msg = "'node' and 'dest' must both be integer or character."
    kn, kd = _kind(node), _kind(dest)
    if dest_kind is not None and kd == "empty":
        kd = dest_kind
    if kn in ("num", "empty") and kd in ("num", "empty"):
        if not _whole(node) or not _whole([d for e, d in zip(event, dest) if e == 3]):
            raise ValueError(msg)
        to = lambda vs: np.array([NA if _is_na(v) else int(v) for v in vs], dtype=np.int64)
        return to(node), to(dest)
    if kn in ("str", "empty") and kd in ("str", "empty"):
        levels = sorted({v for v in list(node) + list(dest) if not _is_na(v)})
        return _factor(node, levels), _factor(dest, levels)
    raise ValueError(msg)


def _order(keys):
    """Stable order by the int64 keys, most significant first (R's
    order()).  The keys are offset by their minimum and packed into as few
    64-bit words as their ranges allow, then sorted word by word from the
    least significant, each pass stable."""
    words, word, used = [], None, 0
    for k in reversed(keys):
        lo = int(k.min()) if k.size else 0
        span = (int(k.max()) - lo) if k.size else 0
        bits = max(1, span.bit_length())
        v = (k - lo).astype(np.uint64)
        if word is None or used + bits > 64:
            if word is not None:
                words.append(word)
            word, used = v, bits
        else:
            word = word | (v << np.uint64(used))
            used += bits
    words.append(word)
    n = len(words[0])
    if n > 1:
        # registers often come sorted already: check before sorting
        out_of_order = np.zeros(n - 1, dtype=bool)
        tied = np.ones(n - 1, dtype=bool)
        for w in reversed(words):
            out_of_order |= tied & (w[1:] < w[:-1])
            tied &= w[1:] == w[:-1]
        if not out_of_order.any():
            return np.arange(n)
    order = None
    for w in words:
        if order is None:
            order = np.argsort(w, kind="stable")
        else:
            order = order[np.argsort(w[order], kind="stable")]
    return order


class Prepared:
    """The coded, ordered, de-duplicated columns of an individual event
    table (`keys`: id, event, time, node, dest as int32, dest NA =
    INT_MIN), the rows of the caller's table they came from, and what
    finish() needs to give the kept rows back in the caller's terms."""

    def __init__(self, raw, rows, keys, event_named, time_dates):
        self.raw, self.rows, self.keys = raw, rows, keys
        self.event_named, self.time_dates = event_named, time_dates


def _numeric(a, msg, na_ok=False):
    """int64 values of a numeric column (NaN is NA, kept as INT_MIN when
    na_ok) with R's whole-number check and truncation, or ValueError(msg)."""
    if a.dtype.kind in "iu":
        out = a.astype(np.int64)
    else:
        na = np.isnan(a)
        if na.any() and not na_ok:
            raise ValueError(msg)
        f = np.where(na, 0.0, a)
        if not np.all(np.abs(f - np.round(f)) < WHOLE_TOL):
            raise ValueError(msg)
        out = np.where(na, NA, np.trunc(f)).astype(np.int64)
    live = out[out != NA] if na_ok else out
    if live.size and (live.min() <= NA or live.max() > np.iinfo(np.int32).max):
        raise ValueError(msg)
    return out


def _arrays(events, columns):
    """The columns as numpy arrays when all are numeric (time may also be
    datetime64[D]), for the vectorised path; None otherwise."""
    out = {}
    for c in columns:
        a = np.asarray(events[c])
        ok = a.dtype.kind in "iuf" or (c == "time" and a.dtype.kind == "M")
        if not ok or a.ndim != 1:
            return None
        out[c] = a
    return out


def _code_arrays(a):
    """id, event, time, node and dest codes of numeric columns, with the
    checks of R/SimInf_individual_events.R:227-345 vectorised."""
    id_code = _numeric(a["id"], "'id' must be an integer or character vector with "
                                "non-NA values.")
    event = _numeric(a["event"], "'event' must be an integer or character vector with "
                                 "non-NA values.")
    if not np.isin(event, (0, 1, 3)).all():
        raise ValueError("'event' must be an integer or character vector with non-NA values.")
    tmsg = "'time' must be an integer or character vector with non-NA values."
    if a["time"].dtype.kind == "M":
        days = a["time"].astype("datetime64[D]")
        if np.isnat(days).any():
            raise ValueError(tmsg)
        time, time_dates = days.astype(np.int64), True
    else:
        time, time_dates = _numeric(a["time"], tmsg), False
    transfer = event == 3
    node, dest = a["node"], a["dest"]
    if (node.dtype.kind == "f" and np.isnan(node).any()) or \
            (dest.dtype.kind == "f" and np.isnan(dest[transfer]).any()):
        raise ValueError("'node' or 'dest' contain NA values.")
    nmsg = "'node' and 'dest' must both be integer or character."
    node_code = _numeric(node, nmsg)
    dest_code = np.full(len(dest), NA, dtype=np.int64)
    dest_code[transfer] = _numeric(dest[transfer], nmsg)
    return id_code, event, time, time_dates, node_code, dest_code


def prepare(events, elementwise=False):
    """The host half of individual_events() (R/SimInf_individual_events.R:
    383-410): checks, coding, ordering and removal of exact repeats.
    Numeric columns (numpy arrays or lists of numbers; time also
    datetime64) are checked and coded as arrays; any other column, or
    elementwise=True, goes value by value (strings, None as NA)."""
    columns = ("id", "event", "time", "node", "dest")
    if not all(c in events for c in columns):
        raise ValueError("Missing columns in 'events'.")
    n = len(events["id"])
    if any(len(events[c]) != n for c in columns):
        raise ValueError("columns differ in length")
    arrays = None if elementwise else _arrays(events, columns)
    if arrays is not None:
        id_code, event, time, time_dates, node_code, dest_code = _code_arrays(arrays)
        event_named = False
        raw = dict(arrays)
    else:
        raw = {c: list(events[c]) for c in columns}
        id_code = check_id(raw["id"])
        event, event_named = check_event(raw["event"])
        time, time_dates = check_time(raw["time"])
        dest_kind = _kind(raw["dest"])
        raw["dest"] = [d if e == 3 else None for e, d in zip(event, raw["dest"])]
        node_code, dest_code = check_nodes(event, raw["node"], raw["dest"], dest_kind)

    # order(id, time, event, node, dest), NA last; then drop exact repeats
    live = dest_code[dest_code != NA]
    dest_key = np.where(dest_code == NA, (int(live.max()) + 1) if live.size else 0, dest_code)
    order = _order((id_code, time, event, node_code, dest_key))
    keys = [k.astype(np.int32)[order] for k in (id_code, event, time, node_code, dest_code)]
    if n > 1:
        repeat = np.ones(n - 1, dtype=bool)
        for k in keys:
            repeat &= k[1:] == k[:-1]
        if repeat.any():
            first = np.concatenate(([True], ~repeat))
            order = order[first]
            keys = [k[first] for k in keys]
    raw["event_code"], raw["time_code"], raw["dest_code"] = event, time, dest_code
    prep = Prepared(raw, order, keys, event_named, time_dates)
    prep.arrays = arrays is not None
    return prep


def finish(prep, keep):
    """The kept rows, in the caller's own values: arrays for numeric input
    (dest int32 with NA as INT_MIN, R's NA_integer_), lists with None as NA
    otherwise."""
    rows = prep.rows[np.asarray(keep).astype(bool)]
    raw, event, time = prep.raw, prep.raw["event_code"], prep.raw["time_code"]
    if prep.arrays:
        return {"id": raw["id"][rows], "event": event[rows].astype(np.int32),
                "time": (time[rows].astype("datetime64[D]") if prep.time_dates
                         else time[rows].astype(np.int32)),
                "node": raw["node"][rows],
                "dest": raw["dest_code"][rows].astype(np.int32)}
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
    id, event, time, node and dest (a dict of sequences; None or NaN is
    NA), as a dict of columns ordered by (id, time, event, node, dest)."""
    prep = prepare(events)
    return finish(prep, longest_paths(*prep.keys, stream=stream))
