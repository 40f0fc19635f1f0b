"""ctypes mirror of include/siminf_gb300.h.

``SolverArgs`` is field for field the C struct ``siminf_gpu_solver_args``,
which is itself layout-identical to the reference's ``SimInf_solver_args``
(src/SimInf_internal.h:44-200).  ``build_args`` fills it from numpy arrays
and keeps those arrays alive for as long as the struct is used.
"""
import ctypes as C

import numpy as np

c_int_p = C.POINTER(C.c_int)
c_double_p = C.POINTER(C.c_double)

# inst/include/SimInf.h:56-59
EXIT_EVENT, ENTER_EVENT, INTERNAL_TRANSFER_EVENT, EXTERNAL_TRANSFER_EVENT = 0, 1, 2, 3

# Messages of SimInf_raise_error (src/SimInf.c:28-97) for the codes of
# inst/include/SimInf.h:66-89, plus the GPU-only codes of siminf_gb300.h
ERRORS = {
    -1: "Negative state detected.",
    -2: "Unable to allocate memory buffer.",
    -3: "Undefined event type.",
    -7: "The continuous state 'v' is not finite.",
    -8: "Unable to sample individuals for event.",
    -9: "Invalid model.",
    -10: "The continuous state 'v' is negative.",
    -11: "Invalid rate detected (non-finite or < 0.0).",
    -12: "Invalid 'solver' value.",
    -13: "'dest' is out of bounds.",
    -14: "'node' is out of bounds.",
    -15: "'N' is invalid.",
    -16: "'shift' is invalid.",
    -17: "'shift' is out of bounds.",
    -18: "Invalid proportion detected (< 0.0 or > 1.0).",
    -19: "Cannot run the 'aem' solver on a replicated model.",
    -30: "A CUDA runtime call failed.",
    -31: "Events must be sorted by time, with E1 events before external transfers.",
    -32: "Unknown device model.",
    -33: "A bounded device wait timed out.",
    -34: "No CUDA device is available.",
    -35: "The run does not fit the allocation-free solver's scratch.",
}


class SimInfError(RuntimeError):
    """Raised with the reference's message for a negative solver code."""

    def __init__(self, code, detail=""):
        self.code = code
        msg = ERRORS.get(code, "Unknown error code: %d." % code)
        super().__init__(msg + (("\n" + detail) if detail else ""))


class SolverArgs(C.Structure):
    _fields_ = [
        ("u0", c_int_p),
        ("v0", c_double_p),
        ("irG", c_int_p),
        ("jcG", c_int_p),
        ("irS", c_int_p),
        ("jcS", c_int_p),
        ("prS", c_int_p),
        ("tspan", c_double_p),
        ("tlen", C.c_int),
        ("U", c_int_p),
        ("irU", c_int_p),
        ("jcU", c_int_p),
        ("prU", c_double_p),
        ("V", c_double_p),
        ("irV", c_int_p),
        ("jcV", c_int_p),
        ("prV", c_double_p),
        ("ldata", c_double_p),
        ("gdata", c_double_p),
        ("Nn", C.c_int),
        ("Nc", C.c_int),
        ("Nt", C.c_int),
        ("Nd", C.c_int),
        ("Nld", C.c_int),
        ("Nrep", C.c_int),
        ("irE", c_int_p),
        ("jcE", c_int_p),
        ("prE", c_double_p),
        ("N", c_int_p),
        ("len", C.c_int),
        ("event", c_int_p),
        ("time", c_int_p),
        ("node", c_int_p),
        ("dest", c_int_p),
        ("n", c_int_p),
        ("proportion", c_double_p),
        ("select", c_int_p),
        ("shift", c_int_p),
        ("Nthread", C.c_int),
        ("solver", C.c_int),
        ("crn", C.c_int),
        ("rng_type", C.c_int),
        ("seed", C.c_ulong),
        ("tr_fun", C.c_void_p),
        ("pts_fun", C.c_void_p),
    ]


class Status(C.Structure):
    _fields_ = [
        ("error", C.c_int),
        ("node", C.c_int),
        ("transition", C.c_int),
        ("event_index", C.c_int),
        ("time", C.c_double),
        ("rate", C.c_double),
        ("message", C.c_char * 512),
    ]


class Options(C.Structure):
    _fields_ = [("cap_transfers", C.c_int), ("heavy_rate", C.c_int),
                ("gdata_per_replicate", C.c_int), ("two_pass", C.c_int),
                ("max_node_day_transitions", C.c_int), ("streamed", C.c_int),
                ("ssa_variant", C.c_int), ("wave_block", C.c_int), ("heavy_lanes", C.c_int)]


class PfilterArgs(C.Structure):
    _fields_ = [
        ("n_particles", C.c_int),
        ("gdata_per_particle", C.c_int),
        ("n_obs", C.c_int),
        ("obs_time", C.POINTER(C.c_int)),
        ("obs", C.POINTER(C.c_int)),
        ("obs_compartment", C.c_int),
        ("detect_p", C.c_double),
        ("seed", C.c_ulong),
        ("loglik", C.POINTER(C.c_double)),
        ("ess", C.POINTER(C.c_double)),
        ("ancestors", C.POINTER(C.c_int)),
        ("ms_total", C.c_double),
    ]


class BatchJob(C.Structure):
    """siminf_gpu_batch_job."""
    _fields_ = [
        ("args", C.c_void_p),
        ("target", C.POINTER(C.c_double)),
        ("prevalence", C.POINTER(C.c_double)),
        ("distance", C.POINTER(C.c_double)),
    ]


class BatchOptions(C.Structure):
    """siminf_gpu_batch_options."""
    _fields_ = [
        ("prevalence_num_mask", C.c_uint),
        ("prevalence_den_mask", C.c_uint),
        ("cap_transfers", C.c_int),
        ("heavy_rate", C.c_int),
        ("reserved", C.c_int * 4),
    ]


class Stats(C.Structure):
    _fields_ = [
        ("transitions", C.c_uint64),
        ("node_days", C.c_uint64),
        ("e1_events", C.c_uint64),
        ("e2_events", C.c_uint64),
        ("e2_waves", C.c_int),
        ("days", C.c_int),
        ("ms_upload", C.c_double),
        ("ms_plan", C.c_double),
        ("ms_solve", C.c_double),
        ("ms_download", C.c_double),
    ]


TUNE_CANDIDATES = 16


class TuneResult(C.Structure):
    """siminf_gpu_tune_result."""
    _fields_ = [
        ("heavy_rate", C.c_double * TUNE_CANDIDATES),
        ("two_pass", C.c_int * TUNE_CANDIDATES),
        ("ssa_variant", C.c_int * TUNE_CANDIDATES),
        ("wave_block", C.c_int * TUNE_CANDIDATES),
        ("heavy_lanes", C.c_int * TUNE_CANDIDATES),
        ("ms", C.c_double * TUNE_CANDIDATES),
        ("n_candidates", C.c_int),
        ("chosen", C.c_int),
        ("probe_days", C.c_int),
        ("cached", C.c_int),
    ]


class ReduceStats(C.Structure):
    """siminf_gpu_reduce_stats."""
    _fields_ = [("ms_kernel", C.c_double), ("ms_total", C.c_double),
                ("bytes_read", C.c_longlong), ("bytes_written", C.c_longlong)]


class PrevalenceSpec(C.Structure):
    """siminf_gpu_prevalence_spec."""
    _fields_ = [("cases", C.c_uint), ("population", C.c_uint), ("level", C.c_int),
                ("n_condition", C.c_int), ("condition", C.POINTER(C.c_int))]


# Operators of a prevalence condition (SIMINF_GPU_COND_*).
COND_OPS = {"compartment": 1, "const": 2, "+": 3, "-": 4, "*": 5, "neg": 6, "==": 7,
            "!=": 8, "<": 9, "<=": 10, ">": 11, ">=": 12, "&": 13, "|": 14, "!": 15}


class ServerOptions(C.Structure):
    """siminf_gpu_server_options."""
    _fields_ = [
        ("slots", C.c_int),
        ("reserved0", C.c_int),
        ("hbm_budget_bytes", C.c_longlong),
        ("reserved", C.c_int * 4),
    ]


class Request(C.Structure):
    """siminf_gpu_request."""
    _fields_ = [
        ("kind", C.c_int),
        ("args", C.c_void_p),
        ("model", C.c_void_p),
        ("options", Options),
        ("pfilter", C.c_void_p),
        ("plan", C.c_void_p),
        ("bytes", C.c_longlong),
        ("status", C.c_int),
        ("finished", C.c_int),
        ("ms_wait", C.c_double),
        ("ms_run", C.c_double),
        ("submit_ns", C.c_longlong),
        ("stats", Stats),
        ("message", C.c_char * 200),
        ("pmcmc", C.c_void_p),
        ("pmcmc_iterations", C.c_int),
        ("pmcmc_rows", C.c_void_p),
    ]


REQUEST_RUN, REQUEST_PFILTER, REQUEST_PLAN, REQUEST_PMCMC = 0, 1, 2, 3


class PmcmcArgs(C.Structure):
    """siminf_gpu_pmcmc_args."""
    _fields_ = [
        ("n_pars", C.c_int),
        ("gdata_index", C.POINTER(C.c_int)),
        ("theta", C.POINTER(C.c_double)),
        ("prior_lo", C.POINTER(C.c_double)),
        ("prior_hi", C.POINTER(C.c_double)),
        ("chol", C.POINTER(C.c_double)),
        ("seed", C.c_ulong),
        ("reserved", C.c_int * 4),
    ]


def csc(dense):
    """Dense matrix -> (ir, jc, pr) in compressed-sparse-column form, the
    storage of R's dgCMatrix slots i, p, x."""
    d = np.asarray(dense)
    ir, pr, jc = [], [], [0]
    for j in range(d.shape[1]):
        rows = np.nonzero(d[:, j])[0]
        ir.extend(rows.tolist())
        pr.extend(d[rows, j].tolist())
        jc.append(len(ir))
    return (np.asarray(ir, dtype=np.int32), np.asarray(jc, dtype=np.int32),
            np.asarray(pr, dtype=np.float64))


def _ptr(a, ctype):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


class ArgsHolder:
    """A filled SolverArgs plus the numpy arrays it points into."""

    def __init__(self, args, keep, U=None, V=None, prU=None, prV=None):
        self.args = args
        self.keep = keep
        self.U = U
        self.V = V
        self.prU = prU
        self.prV = prV

    def ref(self):
        return C.byref(self.args)


def build_args(model, seed, U_sparse=None, V_sparse=None, solver=0):
    """Fill a SolverArgs for ``model`` (a siminf_gb300.model.SimInfModel).

    U and V are allocated here as the caller-owned output buffers: dense
    (Nn*Nc) x (Nrep*tlen) column-major, or sparse over the (ir, jc)
    pattern given in U_sparse / V_sparse, as SimInf_run allocates them
    (src/SimInf.c:325-354).
    """
    m = model
    keep = []

    def arr(a, dtype):
        if a is None:
            return None
        b = np.ascontiguousarray(a, dtype=dtype)
        keep.append(b)
        return b

    Nn, Nc, Nt, Nd = m.Nn, m.Nc, m.Nt, m.Nd
    Nrep = m.replicates
    tlen = len(m.tspan)
    u0 = arr(np.asarray(m.u0, dtype=np.int32).reshape(-1, order="F"), np.int32)
    v0 = arr(np.asarray(m.v0, dtype=np.float64).reshape(-1, order="F"), np.float64)
    irG, jcG, _ = csc(m.G)
    irS, jcS, prS = csc(m.S)
    irG, jcG, irS, jcS = arr(irG, np.int32), arr(jcG, np.int32), arr(irS, np.int32), arr(jcS, np.int32)
    prS = arr(prS.astype(np.int32), np.int32)
    tspan = arr(m.tspan, np.float64)
    ldata = arr(np.asarray(m.ldata, dtype=np.float64).reshape(-1, order="F"), np.float64)
    if ldata.size == 0:
        # SimInf_run passes a one-element {INFINITY} sentinel when Nld == 0
        # (src/SimInf.c:244,361-364).
        ldata = arr(np.array([np.inf]), np.float64)
    gdata = arr(np.asarray(m.gdata, dtype=np.float64).reshape(-1), np.float64)
    if gdata.size == 0:
        gdata = arr(np.array([0.0]), np.float64)
    irE, jcE, prE = csc(m.E) if m.E is not None and np.asarray(m.E).size else (
        np.zeros(0, np.int32), np.zeros(1, np.int32), np.zeros(0))
    irE, jcE, prE = arr(irE, np.int32), arr(jcE, np.int32), arr(prE, np.float64)
    Nmat = None
    if m.N is not None and np.asarray(m.N).size:
        Nmat = arr(np.asarray(m.N, dtype=np.int32).reshape(-1, order="F"), np.int32)
    ev = m.events
    ne = len(ev["event"]) if ev is not None else 0
    evf = {}
    for k, dt in (("event", np.int32), ("time", np.int32), ("node", np.int32),
                  ("dest", np.int32), ("n", np.int32), ("proportion", np.float64),
                  ("select", np.int32), ("shift", np.int32)):
        evf[k] = arr(ev[k] if ne else np.zeros(1), dt)

    U = V = prU = prV = None
    irU = jcU = irV = jcV = None
    if U_sparse is None:
        U = np.zeros(Nn * Nc * Nrep * tlen, dtype=np.int32)
        keep.append(U)
    else:
        irU, jcU = arr(U_sparse[0], np.int32), arr(U_sparse[1], np.int32)
        prU = np.zeros(len(U_sparse[0]), dtype=np.float64)
        keep.append(prU)
    if V_sparse is None:
        V = np.zeros(max(Nn * Nd * Nrep * tlen, 1), dtype=np.float64)
        keep.append(V)
    else:
        irV, jcV = arr(V_sparse[0], np.int32), arr(V_sparse[1], np.int32)
        prV = np.zeros(max(len(V_sparse[0]), 1), dtype=np.float64)
        keep.append(prV)

    a = SolverArgs()
    a.u0 = _ptr(u0, C.c_int)
    a.v0 = _ptr(v0, C.c_double) if v0.size else _ptr(arr(np.zeros(1), np.float64), C.c_double)
    a.irG, a.jcG = _ptr(irG, C.c_int), _ptr(jcG, C.c_int)
    a.irS, a.jcS, a.prS = _ptr(irS, C.c_int), _ptr(jcS, C.c_int), _ptr(prS, C.c_int)
    a.tspan, a.tlen = _ptr(tspan, C.c_double), tlen
    a.U = _ptr(U, C.c_int)
    a.irU, a.jcU, a.prU = _ptr(irU, C.c_int), _ptr(jcU, C.c_int), _ptr(prU, C.c_double)
    a.V = _ptr(V, C.c_double)
    a.irV, a.jcV, a.prV = _ptr(irV, C.c_int), _ptr(jcV, C.c_int), _ptr(prV, C.c_double)
    a.ldata, a.gdata = _ptr(ldata, C.c_double), _ptr(gdata, C.c_double)
    a.Nn, a.Nc, a.Nt, a.Nd = Nn, Nc, Nt, Nd
    a.Nld = m.Nld
    a.Nrep = Nrep
    a.irE, a.jcE, a.prE = _ptr(irE, C.c_int), _ptr(jcE, C.c_int), _ptr(prE, C.c_double)
    a.N = _ptr(Nmat, C.c_int)
    a.len = ne
    for k in ("event", "time", "node", "dest", "n", "select", "shift"):
        setattr(a, k, _ptr(evf[k], C.c_int))
    a.proportion = _ptr(evf["proportion"], C.c_double)
    a.Nthread = 1
    a.solver = solver
    a.crn = 0
    a.rng_type = 0
    a.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
    return ArgsHolder(a, keep, U=U, V=V, prU=prU, prV=prV)
