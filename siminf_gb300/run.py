"""The user-facing run(): the counterpart of R's run(model, ...) (R/run.R:
178-283) for the GPU solver.

run() fills the solver argument struct from a SimInfModel, calls
siminf_gpu_run_solver_ssm (one replicate) or siminf_gpu_run_solver_mssm
(replicates > 1) -- the same dispatch as src/SimInf.c:382-399 -- and returns
U and V in the reference's column-major layout: U is (Nn*Nc) x (Nrep*tlen),
column r*tlen + k holding replicate r at tspan[k].
"""
import ctypes as C

import numpy as np

from . import abi, native


class Result:
    def __init__(self, model, holder, stats):
        self.model = model
        m = model
        tlen = len(m.tspan)
        ncol = m.replicates * tlen
        self.U = None if holder.U is None else holder.U.reshape((m.Nn * m.Nc, ncol), order="F")
        self.V = None
        if holder.V is not None and m.Nd > 0:
            self.V = holder.V[:m.Nn * m.Nd * ncol].reshape((m.Nn * m.Nd, ncol), order="F")
        self.prU = holder.prU
        self.prV = holder.prV
        self.stats = stats

    def trajectory(self, compartment, replicate=0):
        """Matrix (Nn, tlen) of one compartment (index) of one replicate."""
        m = self.model
        tlen = len(m.tspan)
        cols = self.U[:, replicate * tlen:(replicate + 1) * tlen]
        return cols[compartment::m.Nc, :]


SOLVERS = {"ssm": 0, "aem": 1}


def run(model, seed=42, U_sparse=None, V_sparse=None, cap_transfers=False, solver="ssm"):
    """Simulate ``model`` on the GPU.  ``U_sparse``/``V_sparse`` are optional
    (ir, jc) CSC patterns over (Nn*Nc) x (Nrep*tlen) selecting which entries
    to record, as a punchcard does (R/punchcard.R:139-253).
    ``cap_transfers`` enables the siminf_gpu_options extension of that name.
    ``solver`` is "ssm" (the direct method) or "aem" (the all-events method,
    one replicate), as in R's run(model, solver) (R/run.R:128-145)."""
    if solver not in SOLVERS:
        raise ValueError("Invalid 'solver' value.")
    holder = abi.build_args(model, seed, U_sparse=U_sparse, V_sparse=V_sparse,
                            solver=SOLVERS[solver])
    dm = native.device_model(model.name)
    if cap_transfers:
        opt = abi.Options(cap_transfers=1)
        code = native.lib().siminf_gpu_run_solver_ex(C.cast(holder.ref(), C.c_void_p),
                                                     dm.handle, C.byref(opt))
        native.check(code)
        return Result(model, holder, native.last_stats())
    fn = (native.lib().siminf_gpu_run_solver_mssm if model.replicates > 1
          else native.lib().siminf_gpu_run_solver_ssm)
    code = fn(C.cast(holder.ref(), C.c_void_p), dm.handle)
    native.check(code)
    return Result(model, holder, native.last_stats())


class PfilterResult:
    def __init__(self, loglik, ess, ancestors, ms):
        self.loglik = loglik
        self.ess = ess
        self.ancestors = ancestors
        self.ms = ms


def pfilter(model, n_particles, obs_time, obs, obs_compartment, detect_p, seed=42,
            gdata=None):
    """Bootstrap particle filter on the GPU (pfilter_internal, R/pfilter.R:
    315-499) with a Binomial(x, detect_p) observation of one compartment in
    every node.  ``model`` is one particle's model (no events); ``gdata``, if
    given, is an (n_particles, ngdata) array with one parameter row per
    particle.  Returns log-likelihood, ESS per observation and one-based
    ancestors (n_obs, n_particles)."""
    m = model
    obs = np.ascontiguousarray(obs, dtype=np.int32)
    obs_time = np.ascontiguousarray(obs_time, dtype=np.int32)
    n_obs = len(obs_time)
    if gdata is not None:
        g = np.ascontiguousarray(gdata, dtype=np.float64)
        m = type(m).__new__(type(m))
        m.__dict__.update(model.__dict__)
        m.gdata = g.reshape(-1)
    holder = abi.build_args(m, seed)
    ll = np.zeros(1)
    ess = np.zeros(n_obs)
    anc = np.zeros((n_obs, n_particles), dtype=np.int32)
    pa = abi.PfilterArgs(
        n_particles=n_particles, gdata_per_particle=int(gdata is not None), n_obs=n_obs,
        obs_time=obs_time.ctypes.data_as(C.POINTER(C.c_int)),
        obs=obs.ctypes.data_as(C.POINTER(C.c_int)), obs_compartment=obs_compartment,
        detect_p=detect_p, seed=seed,
        loglik=ll.ctypes.data_as(C.POINTER(C.c_double)),
        ess=ess.ctypes.data_as(C.POINTER(C.c_double)),
        ancestors=anc.ctypes.data_as(C.POINTER(C.c_int)))
    native.check(native.lib().siminf_gpu_pfilter(C.cast(holder.ref(), C.c_void_p),
                                                 native.device_model(m.name).handle,
                                                 C.byref(pa)))
    return PfilterResult(float(ll[0]), ess, anc, pa.ms_total)


class Pmcmc:
    """A particle-marginal Metropolis-Hastings chain resident on the GPU
    (siminf_gpu_pmcmc_*), the counterpart of R's pmcmc() and
    continue_pmcmc() (R/pmcmc.R:470-600) for gdata parameters with uniform
    priors and a fixed Gaussian random-walk proposal.  run(n) continues the
    chain by n iterations and returns their rows (logPost, logLik,
    logPrior, accept, theta...); chain holds every row so far."""

    COLUMNS = ("logPost", "logLik", "logPrior", "accept")

    def __init__(self, model, n_particles, obs_time, obs, obs_compartment, detect_p, pars,
                 theta, prior_lo, prior_hi, covmat, seed=42):
        self.model = model
        self.pars = [int(k) for k in pars]
        self._holder = abi.build_args(model, seed)
        self._obs = np.ascontiguousarray(obs, dtype=np.int32)
        self._obs_time = np.ascontiguousarray(obs_time, dtype=np.int32)
        self._pf = abi.PfilterArgs(
            n_particles=n_particles, gdata_per_particle=0, n_obs=len(self._obs_time),
            obs_time=self._obs_time.ctypes.data_as(C.POINTER(C.c_int)),
            obs=self._obs.ctypes.data_as(C.POINTER(C.c_int)), obs_compartment=obs_compartment,
            detect_p=detect_p, seed=seed)
        n = len(self.pars)
        chol = np.linalg.cholesky(np.asarray(covmat, dtype=np.float64)).T   # upper: covmat = Q'Q
        self._keep = [np.ascontiguousarray(x, dtype=dt) for x, dt in (
            (self.pars, np.int32), (theta, np.float64), (prior_lo, np.float64),
            (prior_hi, np.float64), (chol, np.float64))]
        k = self._keep
        self._args = abi.PmcmcArgs(
            n_pars=n, gdata_index=k[0].ctypes.data_as(C.POINTER(C.c_int)),
            theta=k[1].ctypes.data_as(C.POINTER(C.c_double)),
            prior_lo=k[2].ctypes.data_as(C.POINTER(C.c_double)),
            prior_hi=k[3].ctypes.data_as(C.POINTER(C.c_double)),
            chol=k[4].ctypes.data_as(C.POINTER(C.c_double)), seed=seed)
        h = C.c_void_p()
        native.check(native.lib().siminf_gpu_pmcmc_create(
            C.cast(self._holder.ref(), C.c_void_p), native.device_model(model.name).handle,
            C.byref(self._pf), C.byref(self._args), C.byref(h)))
        self.handle = h
        self.chain = np.zeros((0, 4 + n))

    def run(self, n_iterations):
        rows = np.zeros((n_iterations, 4 + len(self.pars)))
        native.check(native.lib().siminf_gpu_pmcmc_run(self.handle, int(n_iterations),
                                                       rows.ctypes.data_as(C.c_void_p)))
        self.chain = np.vstack([self.chain, rows])
        return rows

    def close(self):
        if getattr(self, "handle", None):
            native.lib().siminf_gpu_pmcmc_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def compartment_mask(model, names_or_indices):
    """Bit mask of compartments given by index or by u0 row position."""
    mask = 0
    for c in names_or_indices:
        mask |= 1 << int(c)
    return mask


def run_batch(models, seeds, targets=None, numerator=(2,), denominator=None,
              cap_transfers=False):
    """Many independent models of one device model in one run
    (siminf_gpu_run_batch): returns (prevalence series, distances).

    Prevalence at tspan point k of model j is the sum over its nodes of the
    compartments in ``numerator`` over the sum of those in ``denominator``
    (default: all); the distance is the L2 norm of prevalence - target.
    Each model's trajectory is the one run(model, seed) gives it alone; this
    replaces the one-run-per-proposal loop of R/abc.R:589-628 / :675-729.
    """
    n = len(models)
    name = models[0].name
    holders = [abi.build_args(m, int(s)) for m, s in zip(models, seeds)]
    prevs = [np.zeros(len(m.tspan)) for m in models]
    dists = np.zeros(n)
    tgts = [None] * n
    jobs = (abi.BatchJob * n)()
    dptr = C.POINTER(C.c_double)
    for j in range(n):
        jobs[j].args = C.cast(holders[j].ref(), C.c_void_p)
        if targets is not None and targets[j] is not None:
            tgts[j] = np.ascontiguousarray(targets[j], dtype=np.float64)
            if len(tgts[j]) != len(models[j].tspan):
                raise ValueError("target %d needs %d values" % (j, len(models[j].tspan)))
            jobs[j].target = tgts[j].ctypes.data_as(dptr)
        jobs[j].prevalence = prevs[j].ctypes.data_as(dptr)
        jobs[j].distance = C.cast(C.c_void_p(dists.ctypes.data + 8 * j), dptr)
    den = range(models[0].Nc) if denominator is None else denominator
    opt = abi.BatchOptions(prevalence_num_mask=compartment_mask(models[0], numerator),
                           prevalence_den_mask=compartment_mask(models[0], den),
                           cap_transfers=int(bool(cap_transfers)))
    code = native.lib().siminf_gpu_run_batch(jobs, n, native.device_model(name).handle,
                                             C.byref(opt))
    native.check(code)
    return prevs, dists
