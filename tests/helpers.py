"""Shared helpers of the test suite: model builders for the golden fixtures
and the synthetic parity cases, and runners for oracle, reference and GPU."""
import json
import os

import numpy as np

from siminf_gb300 import abi, model as M

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def golden(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)


def events_from(d):
    if not d:
        return None
    return M.make_events(**{k: np.asarray(v) for k, v in d.items()})


def model_from_fixture(fx):
    p = fx["params"]
    name = fx["model"]
    ev = events_from(fx.get("events"))
    if name == "SISe":
        phi = fx.get("phi", p.get("phi"))
        m = M.SISe(fx["u0"], fx["tspan"], phi=phi, upsilon=p["upsilon"], gamma=p["gamma"],
                   alpha=p["alpha"], beta_t1=p["beta_t1"], beta_t2=p["beta_t2"],
                   beta_t3=p["beta_t3"], beta_t4=p["beta_t4"], end_t1=p["end_t1"],
                   end_t2=p["end_t2"], end_t3=p["end_t3"], end_t4=p["end_t4"],
                   epsilon=p["epsilon"], events=ev)
    elif name == "SIR":
        m = M.SIR(fx["u0"], fx["tspan"], beta=p["beta"], gamma=p["gamma"], events=ev)
    elif name == "SISe3":
        m = M.SISe3(fx["u0"], fx["tspan"], phi=fx["phi"], events=ev, **p)
        for r, c in fx.get("E_extra", []):
            m.E[r, c] = 1
    else:
        raise ValueError(name)
    if fx.get("replicates", 1) > 1:
        nn = fx["Nn"]
        m = M.SimInfModel(m.name, m.G, m.S, m.u0, m.tspan, v0=m.v0, ldata=m.ldata[:, :nn],
                          gdata=m.gdata, E=m.E, N=m.N, events=m.events,
                          replicates=fx["replicates"])
    return m


def sparse_pattern(i, j, nrow, ncol):
    """(ir, jc) CSC pattern from one-based (i, j) pairs."""
    i = np.asarray(i, dtype=np.int64) - 1
    j = np.asarray(j, dtype=np.int64) - 1
    order = np.lexsort((i, j))
    i, j = i[order], j[order]
    jc = np.zeros(ncol + 1, dtype=np.int32)
    np.add.at(jc, j + 1, 1)
    jc = np.cumsum(jc).astype(np.int32)
    return i.astype(np.int32), jc


def run_oracle(m, seed=42, threads=1, U_sparse=None, V_sparse=None):
    from oracle import oracle
    h = abi.build_args(m, seed, U_sparse=U_sparse, V_sparse=V_sparse)
    code, res = oracle.run(h, m.name, threads)
    return code, res, h


def run_ref(m, seed=42, threads=1, U_sparse=None, V_sparse=None):
    from oracle import oracle
    h = abi.build_args(m, seed, U_sparse=U_sparse, V_sparse=V_sparse)
    code = oracle.run_ref(h, m.name, threads)
    return code, h


def run_gpu(m, seed=42, U_sparse=None, V_sparse=None):
    """(code, holder, stats) through the C ABI: ssm for one replicate,
    mssm otherwise."""
    import ctypes as C
    from siminf_gb300 import native
    h = abi.build_args(m, seed, U_sparse=U_sparse, V_sparse=V_sparse)
    dm = native.device_model(m.name)
    fn = (native.lib().siminf_gpu_run_solver_mssm if m.replicates > 1
          else native.lib().siminf_gpu_run_solver_ssm)
    code = fn(C.cast(h.ref(), C.c_void_p), dm.handle)
    return code, h, native.last_stats()


def pin_inputs_outputs(h, m, torch):
    """Move the holder's inputs (u0, ldata, the event columns) and its U
    into pinned host memory, as an end-to-end caller with pinned buffers
    passes them."""
    import ctypes as C
    a = h.args

    def pinned(src):
        t = torch.from_numpy(np.ascontiguousarray(src)).pin_memory()
        h.keep.append(t)
        return t.numpy()

    def repoint(field, n, dtype, ctype):
        if n <= 0 or not getattr(a, field):
            return
        arr = pinned(np.ctypeslib.as_array(getattr(a, field), shape=(n,)).view(dtype))
        setattr(a, field, arr.ctypes.data_as(C.POINTER(ctype)))

    for k in ("event", "time", "node", "dest", "n", "select", "shift"):
        repoint(k, a.len, np.int32, C.c_int)
    repoint("proportion", a.len, np.float64, C.c_double)
    repoint("u0", m.Nn * m.Nc * m.replicates, np.int32, C.c_int)
    repoint("ldata", m.Nld * m.Nn, np.float64, C.c_double)
    h.U = pinned(h.U)
    a.U = h.U.ctypes.data_as(C.POINTER(C.c_int))


def U_matrix(m, h):
    return h.U.reshape((m.Nn * m.Nc, m.replicates * len(m.tspan)), order="F")


def random_events(rng, Nn, days, t0=1, p_enter=0.01, p_exit=0.01, p_exit_prop=0.003,
                  n_e2=40, n_e2_prop=3, enter_select=1, exit_select=2, e2_select=2):
    ev = {k: [] for k in M.EVENT_FIELDS}

    def add(*vals):
        for key, val in zip(M.EVENT_FIELDS, vals):
            ev[key].append(val)

    for t in range(t0, t0 + days):
        for node in np.nonzero(rng.random(Nn) < p_enter)[0]:
            add(1, t, node + 1, 0, 1, 0.0, enter_select, 0)
        for node in np.nonzero(rng.random(Nn) < p_exit)[0]:
            add(0, t, node + 1, 0, 1, 0.0, exit_select, 0)
        for node in np.nonzero(rng.random(Nn) < p_exit_prop)[0]:
            add(0, t, node + 1, 0, 0, 0.05, exit_select, 0)
        src = rng.integers(1, Nn + 1, n_e2)
        dst = rng.integers(1, Nn + 1, n_e2)
        for s_, d_ in zip(src, dst):
            if s_ != d_:
                add(3, t, s_, d_, 1 + rng.poisson(3), 0.0, e2_select, 0)
        for s_, d_ in zip(src[:n_e2_prop], dst[:n_e2_prop]):
            if s_ != d_:
                add(3, t, s_, d_, 0, 0.1, e2_select, 0)
    return M.make_events(**{k: np.array(v) for k, v in ev.items()})


def parity_cases():
    """Synthetic cases shared by the oracle-vs-reference and GPU-vs-oracle
    parity tests: (label, model)."""
    rng = np.random.default_rng(1)
    cases = []
    u0 = {"S": np.full(1000, 99), "I": np.full(1000, 5), "R": np.zeros(1000)}
    cases.append(("sir_mparse_1000x150", M.SIR_mparse(u0, np.arange(1, 151), 0.16, 0.077)))
    u0 = {"S": rng.poisson(300, 500), "E": 0,
          "I": rng.poisson(3, 500) * (rng.random(500) < 0.3), "R": 0}
    cases.append(("seir_500x100", M.SEIR(u0, np.arange(1, 101), 0.16, 0.25, 0.077)))
    u0 = {"S": rng.poisson(40, 64), "I": rng.poisson(3, 64), "R": rng.poisson(2, 64)}
    cases.append(("sir_builtin_odd_tspan", M.SIR(u0, np.array([0.5, 3.0, 3.5, 10.0, 40.25]),
                                                 0.3, 0.05)))
    u0 = {"S": rng.poisson(60, 100), "I": rng.poisson(4, 100)}
    cases.append(("sis_100x80", M.SIS(u0, np.arange(0, 80), 0.2, 0.1)))
    u0 = {"S": rng.poisson(100, 200), "I": rng.poisson(2, 200)}
    cases.append(("sise_200x199", M.SISe(u0, np.arange(1, 200), phi=0.0, upsilon=0.017,
                                         gamma=0.1, alpha=1, beta_t1=0.19, beta_t2=0.085,
                                         beta_t3=0.075, beta_t4=0.185, end_t1=91, end_t2=182,
                                         end_t3=273, end_t4=365, epsilon=0.000011)))
    u0 = {k: rng.poisson(20, 50) for k in ("S_1", "I_1", "S_2", "I_2", "S_3", "I_3")}
    ev3 = {k: [] for k in M.EVENT_FIELDS}
    for t in range(1, 60):
        for node in range(50):
            r = rng.random()
            row = None
            if r < 0.05:
                row = (2, t, node + 1, 0, 2, 0.0, 4, 1)      # age S_1/I_1 -> S_2/I_2
            elif r < 0.08:
                row = (1, t, node + 1, 0, 3, 0.0, 1, 0)      # enter S_1
            elif r < 0.10:
                row = (0, t, node + 1, 0, 1, 0.0, 6, 0)      # exit from age 3
            if row:
                for key, val in zip(M.EVENT_FIELDS, row):
                    ev3[key].append(val)
        for _ in range(6):
            s_, d_ = rng.integers(1, 51, 2)
            if s_ != d_:
                for key, val in zip(M.EVENT_FIELDS, (3, t, s_, d_, 2, 0.0, 5, 0)):
                    ev3[key].append(val)
    cases.append(("sise3_events", M.SISe3(
        u0, np.arange(1, 60), phi=0.1, upsilon_1=0.01, upsilon_2=0.02, upsilon_3=0.03,
        gamma_1=0.1, gamma_2=0.12, gamma_3=0.14, alpha=1.0, beta_t1=0.19, beta_t2=0.085,
        beta_t3=0.075, beta_t4=0.185, end_t1=91, end_t2=182, end_t3=273, end_t4=365,
        epsilon=1e-5, events=M.make_events(**{k: np.array(v) for k, v in ev3.items()}))))
    cases.append(("sir_mparse_rep7", M.SIR_mparse(
        {"S": np.full(50, 99), "I": np.full(50, 5), "R": 0}, np.arange(1, 60),
        0.16, 0.077).replicate(7)))
    Nn, days = 300, 120
    u0 = {"S": rng.poisson(300, Nn), "E": 0,
          "I": rng.poisson(3, Nn) * (rng.random(Nn) < 0.1), "R": 0}
    ev = random_events(rng, Nn, days)
    seir_ev = M.SEIR(u0, np.arange(1, days + 1), 0.16, 0.25, 0.077, events=ev)
    cases.append(("seir_events_300x120", seir_ev))
    cases.append(("seir_events_rep5", seir_ev.replicate(5)))
    # weighted enter (biased urn) and internal transfer with shift on SIS
    u0 = {"S": rng.poisson(50, 40), "I": rng.poisson(5, 40)}
    evs = {k: [] for k in M.EVENT_FIELDS}
    for t in range(1, 60):
        for node in range(40):
            if rng.random() < 0.1:
                for key, val in zip(M.EVENT_FIELDS, (2, t, node + 1, 0, 2, 0.0, 1, 1)):
                    evs[key].append(val)
            if rng.random() < 0.1:
                for key, val in zip(M.EVENT_FIELDS, (1, t, node + 1, 0, 3, 0.0, 2, 1)):
                    evs[key].append(val)
    sis = M.SIS(u0, np.arange(1, 60), 0.1, 0.05,
                events=M.make_events(**{k: np.array(v) for k, v in evs.items()}))
    sis.N = np.array([[1], [0]], dtype=np.int32)
    sis.E = np.array([[1, 2], [0, 1]], dtype=np.float64)
    cases.append(("sis_shift_weighted", sis))
    # spatial coupling: phi spreads between the nodes of a 12 x 12 grid
    # within distance 1.5 (up to eight neighbours), with external
    # transfers, so each post time step reads neighbours after the day's
    # transfers; replicated, so the neighbours sit in the replicate's block
    gx, gy = np.meshgrid(np.arange(12.0), np.arange(12.0))
    dist = M.distance_matrix(gx.ravel(), gy.ravel(), 1.5)
    n = 144
    u0 = {"S": rng.poisson(200, n), "I": rng.poisson(2, n) * (rng.random(n) < 0.3)}
    sp = M.SISe_sp(u0, np.arange(1, 91), phi=rng.uniform(0, 0.2, n), upsilon=0.015,
                   gamma=0.1, alpha=0.8, beta_t1=0.19, beta_t2=0.085, beta_t3=0.075,
                   beta_t4=0.185, end_t1=91, end_t2=182, end_t3=273, end_t4=365,
                   coupling=0.05, distance=dist,
                   events=random_events(rng, n, 90, n_e2=20, n_e2_prop=2))
    cases.append(("sise_sp_grid_events", sp))
    cases.append(("sise_sp_grid_rep3", sp.replicate(3)))
    u0 = {k: rng.poisson(15, n) * (1 if k.startswith("S") else (rng.random(n) < 0.3))
          for k in ("S_1", "I_1", "S_2", "I_2", "S_3", "I_3")}
    cases.append(("sise3_sp_grid", M.SISe3_sp(
        u0, np.arange(1, 61), phi=0.05, upsilon_1=0.01, upsilon_2=0.02, upsilon_3=0.03,
        gamma_1=0.1, gamma_2=0.12, gamma_3=0.14, alpha=1.0, beta_t1=0.19, beta_t2=0.085,
        beta_t3=0.075, beta_t4=0.185, end_t1=91, end_t2=182, end_t3=273, end_t4=365,
        coupling=0.02, distance=dist)))
    return cases
