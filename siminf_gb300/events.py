"""The ordering of a scheduled-event table on the device
(siminf_gpu_sort_events): SimInf_events sorts events by (time, event,
select), equal keys in input order (R/SimInf_events.R:396), before a model
may run them.

    ev = sort_events(ev)    # dict of the eight event columns
"""
import ctypes as C

import numpy as np

from . import abi, native

COLUMNS = ("event", "time", "node", "dest", "n", "proportion", "select", "shift")


def sort_events(events, stream=None, stats=False):
    """Sorted copies of the event columns (a dict with the eight columns of
    a SimInf_events table); with stats=True also the ReduceStats."""
    cols = {k: np.ascontiguousarray(np.array(events[k], dtype=np.float64 if k == "proportion"
                                             else np.int32)) for k in COLUMNS}
    n = len(cols["time"])
    if any(len(v) != n for v in cols.values()):
        raise ValueError("event columns differ in length")
    st = abi.ReduceStats()
    pi = lambda k: cols[k].ctypes.data_as(C.POINTER(C.c_int))
    native.check(native.lib().siminf_gpu_sort_events(
        n, pi("event"), pi("time"), pi("node"), pi("dest"), pi("n"),
        cols["proportion"].ctypes.data_as(C.POINTER(C.c_double)), pi("select"), pi("shift"),
        stream, C.byref(st)))
    return (cols, st) if stats else cols
