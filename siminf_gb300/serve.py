"""The serving request loop (siminf_gpu_server_*): runs, particle filters
and re-runs of device-resident plans submitted as they arrive, several on
the GPU at once under an HBM admission budget.

    srv = Server(slots=8)
    t = srv.run(model, seed=1)            # returns at once
    srv.wait(t); t.U                      # the run's U, as run() gives it
    srv.close()

Results are those of the same call made alone (run(), pfilter(),
Plan.run()); the server only decides when and beside what they run.
"""
import ctypes as C

import numpy as np

from . import abi, native


class Ticket:
    """One submitted request and the buffers it writes."""

    def __init__(self, kind, model=None, holder=None, plan=None):
        self.req = abi.Request()
        self.req.kind = kind
        self.model = model
        self.holder = holder
        self.plan = plan
        self.keep = []
        self.loglik = None
        self.ess = None
        self.ancestors = None

    @property
    def finished(self):
        return bool(self.req.finished)

    @property
    def status(self):
        return self.req.status

    @property
    def latency_ms(self):
        """Submission to completion: admission wait plus time on a slot."""
        return self.req.ms_wait + self.req.ms_run

    @property
    def U(self):
        m = self.model
        return self.holder.U.reshape((m.Nn * m.Nc, m.replicates * len(m.tspan)), order="F")


class Server:
    def __init__(self, slots=8, hbm_budget_bytes=0):
        h = C.c_void_p()
        opt = abi.ServerOptions(slots=slots, hbm_budget_bytes=int(hbm_budget_bytes))
        native.check(native.lib().siminf_gpu_server_create(C.byref(opt), C.byref(h)))
        self.handle = h

    def _submit(self, t):
        native.check(native.lib().siminf_gpu_server_submit(self.handle, C.byref(t.req)))
        return t

    def run(self, model, seed=42, cap_transfers=False, solver="ssm"):
        """A simulation run (siminf_gpu_run_solver_ex); solver "ssm" or "aem"."""
        from .run import SOLVERS
        holder = abi.build_args(model, seed, solver=SOLVERS[solver])
        t = Ticket(abi.REQUEST_RUN, model, holder)
        t.req.args = C.cast(holder.ref(), C.c_void_p)
        t.req.model = native.device_model(model.name).handle
        t.req.options = abi.Options(cap_transfers=int(bool(cap_transfers)))
        return self._submit(t)

    def pfilter(self, model, n_particles, obs_time, obs, obs_compartment, detect_p, seed=42,
                gdata=None):
        """A particle filter (siminf_gpu_pfilter)."""
        m = model
        if gdata is not None:
            m = type(model).__new__(type(model))
            m.__dict__.update(model.__dict__)
            m.gdata = np.ascontiguousarray(gdata, dtype=np.float64).reshape(-1)
        holder = abi.build_args(m, seed)
        t = Ticket(abi.REQUEST_PFILTER, m, holder)
        obs = np.ascontiguousarray(obs, dtype=np.int32)
        obs_time = np.ascontiguousarray(obs_time, dtype=np.int32)
        n_obs = len(obs_time)
        t.loglik = np.zeros(1)
        t.ess = np.zeros(n_obs)
        t.ancestors = np.zeros((n_obs, n_particles), dtype=np.int32)
        pa = abi.PfilterArgs(
            n_particles=n_particles, gdata_per_particle=int(gdata is not None), n_obs=n_obs,
            obs_time=obs_time.ctypes.data_as(C.POINTER(C.c_int)),
            obs=obs.ctypes.data_as(C.POINTER(C.c_int)), obs_compartment=obs_compartment,
            detect_p=detect_p, seed=seed,
            loglik=t.loglik.ctypes.data_as(C.POINTER(C.c_double)),
            ess=t.ess.ctypes.data_as(C.POINTER(C.c_double)),
            ancestors=t.ancestors.ctypes.data_as(C.POINTER(C.c_int)))
        t.keep += [obs, obs_time, pa]
        t.req.args = C.cast(holder.ref(), C.c_void_p)
        t.req.model = native.device_model(m.name).handle
        t.req.pfilter = C.cast(C.pointer(pa), C.c_void_p)
        return self._submit(t)

    def plan(self, plan):
        """A re-run of a device-resident native.Plan (results stay on the
        device until plan.download())."""
        t = Ticket(abi.REQUEST_PLAN, plan=plan)
        t.req.plan = plan.handle
        return self._submit(t)

    def pmcmc(self, chain, n_iterations):
        """A continuation of a resident run.Pmcmc chain by n_iterations
        (continue_pmcmc, R/pmcmc.R:474-600): its filter session stays on
        the device between requests; the rows arrive in ticket.rows and are
        appended to chain.chain once the ticket is waited for."""
        t = Ticket(abi.REQUEST_PMCMC)
        t.rows = np.zeros((n_iterations, 4 + len(chain.pars)))
        t.chain = chain
        t.req.pmcmc = chain.handle
        t.req.pmcmc_iterations = int(n_iterations)
        t.req.pmcmc_rows = t.rows.ctypes.data_as(C.c_void_p)
        return self._submit(t)

    def wait(self, ticket, timeout_ms=-1.0):
        """True when the request has finished; raises on its error."""
        done = native.lib().siminf_gpu_server_wait(self.handle, C.byref(ticket.req),
                                                   float(timeout_ms))
        if done and ticket.req.status:
            raise abi.SimInfError(ticket.req.status, ticket.req.message.decode(errors="replace"))
        if done and getattr(ticket, "chain", None) is not None:
            ticket.chain.chain = np.vstack([ticket.chain.chain, ticket.rows])
            ticket.chain = None
        return bool(done)

    def load(self):
        p, r, b = C.c_int(), C.c_int(), C.c_longlong()
        native.lib().siminf_gpu_server_load(self.handle, C.byref(p), C.byref(r), C.byref(b))
        return p.value, r.value, b.value

    def close(self):
        if getattr(self, "handle", None):
            native.lib().siminf_gpu_server_free(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
