"""CPU restatement of SimInf_events' ordering (test infrastructure only:
the oracle for siminf_gpu_sort_events).

R/SimInf_events.R:396 orders the table by (time, event, select) with R's
`order`, which leaves ties in their original order; numpy's lexsort is
stable in the same way (the last key is the primary one).
"""
import numpy as np

COLUMNS = ("event", "time", "node", "dest", "n", "proportion", "select", "shift")


def sort_events(events):
    order = np.lexsort((np.asarray(events["select"]), np.asarray(events["event"]),
                        np.asarray(events["time"])))
    return {k: np.asarray(events[k])[order] for k in COLUMNS}
