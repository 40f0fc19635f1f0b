"""ctypes access to the oracle libraries (test infrastructure only).

- ``liboracle.so``: the C restatement (siminf_oracle.c) of the reference's
  ssm/mssm day loop and event engine.
- ``_ref/libsiminf_ref.so``: the reference's own solver sources compiled
  unmodified against stub R/GSL headers (Makefile target ``ref``); present
  only where the reference tree was available at build time.

Only the test suite, the smoke check and the CPU-baseline leg of bench.py
may import this module.
"""
import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libsiminf_ref.so")


class OracleResult(C.Structure):
    _fields_ = [
        ("error", C.c_int),
        ("err_node", C.c_int),
        ("err_transition", C.c_int),
        ("err_event", C.c_int),
        ("err_time", C.c_double),
        ("err_rate", C.c_double),
        ("transitions", C.c_uint64),
        ("node_days", C.c_uint64),
        ("e1_events", C.c_uint64),
        ("e2_events", C.c_uint64),
        ("seconds_e2", C.c_double),
    ]


def build(ref=None):
    """Compile liboracle.so, and _ref from the reference tree at `ref` (or
    $SIMINF_REFERENCE) when one is given and present."""
    subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"])
    ref_dir = ref or os.environ.get("SIMINF_REFERENCE")
    if ref_dir and os.path.isdir(os.path.join(ref_dir, "src", "solvers")):
        subprocess.check_call(["make", "-s", "-C", HERE, "ref", "REF=" + ref_dir])


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        _lib = C.CDLL(LIB)
        _lib.oracle_run.restype = C.c_int
        _lib.oracle_run.argtypes = [C.c_void_p, C.c_char_p, C.c_int, C.POINTER(OracleResult)]
        _lib.oracle_run_ex.restype = C.c_int
        _lib.oracle_run_ex.argtypes = [C.c_void_p, C.c_char_p, C.c_int, C.c_int,
                                       C.POINTER(OracleResult)]
        _lib.oracle_si_log.restype = C.c_double
        _lib.oracle_si_log.argtypes = [C.c_double]
        _lib.oracle_neglog_u32.restype = None
        _lib.oracle_neglog_u32.argtypes = [C.c_void_p, C.c_void_p, C.c_int64]
        _lib.oracle_philox.argtypes = [C.POINTER(C.c_uint32), C.c_uint32, C.c_uint32]
        _lib.oracle_uniform_pos.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64, C.c_int,
                                            C.POINTER(C.c_double)]
        _lib.oracle_hypergeometric.argtypes = [C.c_uint64, C.c_uint64, C.c_int, C.c_int,
                                               C.c_int, C.c_int, C.POINTER(C.c_int)]
        _lib.oracle_binomial.argtypes = [C.c_uint64, C.c_uint64, C.c_double, C.c_int, C.c_int,
                                         C.POINTER(C.c_int)]
        _lib.oracle_pfilter.restype = C.c_int
        _lib.oracle_pfilter.argtypes = [C.c_void_p, C.c_char_p, C.c_int, C.c_int, C.c_int,
                                        C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_int,
                                        C.c_double, C.c_uint64, C.c_int, C.POINTER(C.c_double),
                                        C.POINTER(C.c_double), C.POINTER(C.c_int)]
        _lib.oracle_set_node_counters.argtypes = [C.c_void_p]
        _lib.oracle_set_day_max.argtypes = [C.c_void_p]
        assert _lib.oracle_result_size() == C.sizeof(OracleResult)
    return _lib


def ref_available():
    return os.path.exists(REF_LIB)


def ref_lib():
    global _ref
    if _ref is None:
        _ref = C.CDLL(REF_LIB)
        _ref.ref_run.restype = C.c_int
        _ref.ref_run.argtypes = [C.c_void_p, C.c_char_p, C.c_int]
        _ref.shim_set_independent.argtypes = [C.c_int]
        _ref.shim_set_independent.restype = None
    return _ref


def run(holder, model_name, threads=1, cap_transfers=False):
    """Run the oracle on a filled abi.ArgsHolder; returns (code, OracleResult)."""
    res = OracleResult()
    code = lib().oracle_run_ex(C.cast(holder.ref(), C.c_void_p), model_name.encode(),
                               int(threads), int(bool(cap_transfers)), C.byref(res))
    return code, res


def run_ref(holder, model_name, threads=1, independent=False):
    """Run the reference's unmodified solver sources; returns the code.
    independent: draw from per-thread Mersenne twisters seeded as the
    reference seeds its GSL generators, instead of the shared per-node
    stream (for distribution tests rather than bit-exact ones)."""
    lib_ = ref_lib()
    lib_.shim_set_independent(int(bool(independent)))
    try:
        return lib_.ref_run(C.cast(holder.ref(), C.c_void_p), model_name.encode(), int(threads))
    finally:
        lib_.shim_set_independent(0)


MODELS_DIR = os.path.join(HERE, "_models")
SHIM_DIR = os.path.join(HERE, "model_shim")
_model_libs = []


def register_c_model(name, c_code, Nc, Nt, Nd):
    """Build model C code on the host with gcc, as R CMD SHLIB builds it for
    the reference (R/run.R:22-73), against the stub R headers of
    model_shim/include, and register its rate and post-time-step functions
    under `name` with the oracle and, when built, with oracle/_ref, so that
    run()/run_ref() can run the model."""
    import hashlib
    import re
    key = hashlib.sha256(c_code.encode()).hexdigest()[:16]
    os.makedirs(MODELS_DIR, exist_ok=True)
    src = os.path.join(MODELS_DIR, "model_%s.c" % key)
    so = os.path.join(MODELS_DIR, "model_%s.so" % key)
    if not os.path.exists(so):
        with open(src, "w") as f:
            f.write(c_code)
        m = re.search(r"(\w+)\s*\(\s*SEXP\s+\w+\s*,\s*SEXP\s+\w+\s*\)\s*\{", c_code)
        if not m:
            raise ValueError("model code without a run function")
        wrap = os.path.join(MODELS_DIR, "capture_%s.c" % key)
        with open(wrap, "w") as f:
            f.write('#include "model_%s.c"\n'
                    "int shim_model_capture(SEXP (*)(SEXP, SEXP), int, TRFun *, PTSFun *);\n"
                    "int shim_model_entry(int nt, TRFun *tr, PTSFun *pts)\n"
                    "{\n    return shim_model_capture(&%s, nt, tr, pts);\n}\n"
                    % (key, m.group(1)))
        tmp = so + ".%d.tmp" % os.getpid()
        subprocess.check_call(["gcc", "-O2", "-fPIC", "-shared", "-std=gnu11",
                               "-ffp-contract=off", "-w", "-I", os.path.join(SHIM_DIR, "include"),
                               "-DSIMINF_MODEL_RUN=shim_model_run",
                               "-DSIMINF_R_INIT=R_init_shim_model",
                               "-DSIMINF_FORCE_SYMBOLS=FALSE", wrap,
                               os.path.join(SHIM_DIR, "model_shim.c"), "-o", tmp, "-lm"])
        os.replace(tmp, so)
    mlib = C.CDLL(so)
    _model_libs.append(mlib)
    tr = (C.c_void_p * 32)()
    pts = C.c_void_p()
    if mlib.shim_model_entry(Nt, tr, C.byref(pts)) != 0:
        raise ValueError("the model code's run function passed no post-time-step function")
    targets = [lib()] + ([ref_lib()] if ref_available() else [])
    for L in targets:
        f = L.oracle_register_model
        f.restype = C.c_int
        f.argtypes = [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
        if f(name.encode(), Nc, Nt, Nd, C.cast(tr, C.c_void_p), pts) != 0:
            raise ValueError("could not register model %s" % name)


def si_log(x):
    return lib().oracle_si_log(float(x))


def neglog_u32(words):
    """si_neglog_u32 over an array of 32-bit words."""
    w = np.ascontiguousarray(words, dtype=np.uint32)
    out = np.empty(len(w))
    lib().oracle_neglog_u32(w.ctypes.data, out.ctypes.data, len(w))
    return out


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    lib().oracle_philox(c, key[0], key[1])
    return list(c)


def uniform_pos(seed, sid, ctr, n):
    out = np.zeros(n, dtype=np.float64)
    lib().oracle_uniform_pos(seed, sid, ctr, n, out.ctypes.data_as(C.POINTER(C.c_double)))
    return out


def hypergeometric(seed, sid, n1, n2, t, count):
    out = np.zeros(count, dtype=np.int32)
    lib().oracle_hypergeometric(seed, sid, n1, n2, t, count, out.ctypes.data_as(C.POINTER(C.c_int)))
    return out


def binomial(seed, sid, p, n, count):
    out = np.zeros(count, dtype=np.int32)
    lib().oracle_binomial(seed, sid, p, n, count, out.ctypes.data_as(C.POINTER(C.c_int)))
    return out


def pfilter(model, n_particles, obs_time, obs, obs_compartment, detect_p, seed=42,
            gdata=None, threads=1):
    """The particle filter restated on the CPU (same interface as
    siminf_gb300.run.pfilter); returns (code, loglik, ess, ancestors)."""
    from siminf_gb300 import abi
    m = model
    if gdata is not None:
        m = type(model).__new__(type(model))
        m.__dict__.update(model.__dict__)
        m.gdata = np.ascontiguousarray(gdata, dtype=np.float64).reshape(-1)
    h = abi.build_args(m, seed)
    obs = np.ascontiguousarray(obs, dtype=np.int32)
    obs_time = np.ascontiguousarray(obs_time, dtype=np.int32)
    n_obs = len(obs_time)
    ll = np.zeros(1)
    ess = np.zeros(n_obs)
    anc = np.zeros((n_obs, n_particles), dtype=np.int32)
    stride = 0 if gdata is None else int(np.asarray(gdata).shape[1])
    code = lib().oracle_pfilter(C.cast(h.ref(), C.c_void_p), m.name.encode(), n_particles,
                                stride, n_obs, obs_time.ctypes.data_as(C.POINTER(C.c_int)),
                                obs.ctypes.data_as(C.POINTER(C.c_int)), obs_compartment,
                                detect_p, seed, threads,
                                ll.ctypes.data_as(C.POINTER(C.c_double)),
                                ess.ctypes.data_as(C.POINTER(C.c_double)),
                                anc.ctypes.data_as(C.POINTER(C.c_int)))
    return code, float(ll[0]), ess, anc


PMCMC_SID = 5 << 60


def pmcmc(model, n_particles, obs_time, obs, obs_compartment, detect_p, pars, theta,
          prior_lo, prior_hi, chol, seed, n_iterations, threads=1):
    """The PMCMC chain (R/pmcmc.R:470-600 with the adaptive part off) on the
    oracle's particle filter, iteration for iteration as the library's
    siminf_gpu_pmcmc_run: rows of logPost, logLik, logPrior, accept and
    theta.  chol is the upper Cholesky factor of the proposal covariance."""
    import math
    n = len(pars)
    gdata = np.array(model.gdata, dtype=np.float64)
    m = type(model).__new__(type(model))
    m.__dict__.update(model.__dict__)

    def loglik(th, it):
        g = gdata.copy()
        for k in range(n):
            g[pars[k]] = th[k]
        m.gdata = g
        s = (seed ^ ((it * 0xD1B54A32D192ED03) & 0xFFFFFFFFFFFFFFFF)) & 0xFFFFFFFFFFFFFFFF
        code, ll, _, _ = pfilter(m, n_particles, obs_time, obs, obs_compartment, detect_p,
                                 seed=s, threads=threads)
        assert code == 0, code
        return ll

    def log_prior(th):
        lp = 0.0
        for k in range(n):
            if not (prior_lo[k] <= th[k] <= prior_hi[k]):
                return -math.inf
            lp -= math.log(prior_hi[k] - prior_lo[k])
        return lp

    rows = []
    th = [float(x) for x in theta]
    ll = lp = 0.0
    for it in range(1, n_iterations + 1):
        accept = 0.0
        if it == 1:
            ll = loglik(th, it)
            lp = log_prior(th)
        else:
            u = uniform_pos(seed, PMCMC_SID + it, 0, 2 * n + 1)
            z = [math.sqrt(-2.0 * math.log(u[2 * k])) * math.cos(6.283185307179586 * u[2 * k + 1])
                 for k in range(n)]
            prop = []
            for j in range(n):
                acc = th[j]
                for k in range(j + 1):
                    acc = acc + z[k] * chol[k][j]
                prop.append(acc)
            lp_p = log_prior(prop)
            if math.isfinite(lp_p):
                ll_p = loglik(prop, it)
                try:
                    alpha = math.exp(ll_p + lp_p - ll - lp)
                except OverflowError:
                    alpha = math.inf
                if math.isfinite(alpha) and u[2 * n] < alpha:
                    ll, lp, th, accept = ll_p, lp_p, prop, 1.0
        rows.append([ll + lp, ll, lp, accept] + list(th))
    return np.array(rows)


def _cols(id, event, time, node, dest):
    return [np.ascontiguousarray(x, dtype=np.int32) for x in (id, event, time, node, dest)]


def individual_events(id, event, time, node, dest, threads=1):
    """The restated cleaning of individual events (oracle_individual.c) on
    sorted, de-duplicated columns (dest NA = INT_MIN).  Returns (keep, bad):
    keep an int32 0/1 array, bad the zero-based index of the first invalid
    event type or -1."""
    cols = _cols(id, event, time, node, dest)
    n = len(cols[0])
    keep = np.zeros(n, dtype=np.int32)
    bad = C.c_longlong(-1)
    f = lib().oracle_individual_events
    f.restype = C.c_int
    f.argtypes = [C.c_longlong] + [C.c_void_p] * 6 + [C.c_int, C.POINTER(C.c_longlong)]
    code = f(n, *[c.ctypes.data for c in cols], keep.ctypes.data, int(threads), C.byref(bad))
    if code not in (0, -1):
        raise MemoryError("oracle_individual_events")
    return keep, bad.value


def ref_individual_events(id, event, time, node, dest, threads=1):
    """SimInf_individual_events compiled unmodified (oracle/_ref); returns
    (keep, message): message is the reference's error text, or None."""
    cols = _cols(id, event, time, node, dest)
    n = len(cols[0])
    keep = np.zeros(n, dtype=np.int32)
    msg = C.create_string_buffer(256)
    f = ref_lib().ref_individual_events
    f.restype = C.c_int
    f.argtypes = [C.c_longlong] + [C.c_void_p] * 6 + [C.c_int, C.c_char_p, C.c_int]
    code = f(n, *[c.ctypes.data for c in cols], keep.ctypes.data, int(threads), msg, 256)
    if code == -2:
        raise MemoryError("ref_individual_events")
    return keep, (msg.value.decode() if code == -1 else None)
