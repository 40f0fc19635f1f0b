"""Model containers mirroring the reference's SimInf_model slots.

``SimInfModel`` carries exactly the slots the solver reads (R/classes.R:
112-124, 235-251): u0, v0, G, S, E, N, tspan, events, ldata, gdata and
replicates, plus the name of the device model that holds the
transition-rate and post-time-step code.  The constructors below build the
same G, S, E and ldata/gdata layouts as the reference's R constructors:

- ``SIR``   R/SIR.R:57-61 (E), :127-137 (G, S, ldata = beta, gamma)
- ``SEIR``  R/SEIR.R:57-61 (E), :136-147 (G, S, ldata = beta, epsilon, gamma)
- ``SIS``   R/SIS.R:54-59 (E), :122-130 (G, S, ldata = beta, gamma)
- ``SISe``  R/SISe.R:140-150 (G, S, ldata = end_t1..end_t4, gdata = upsilon,
  gamma, alpha, beta_t1..beta_t4, epsilon; v0 = phi)
- ``SISe3`` R/SISe3.R:56-61 (E), :158-197 (N, G, S, ldata, gdata, v0 = phi)
- ``SIR_mparse`` and ``SISe_pf``: the models mparse (R/mparse.R:477-491)
  builds from the transition strings named in their docstrings.

Events use the reference's one-based node, dest, select and shift
(shift 0 = no shift) and must be sorted by (time, event, select) as
R/SimInf_events.R:398 sorts them.
"""
import numpy as np

from .abi import ENTER_EVENT, EXIT_EVENT, EXTERNAL_TRANSFER_EVENT, INTERNAL_TRANSFER_EVENT

EVENT_FIELDS = ("event", "time", "node", "dest", "n", "proportion", "select", "shift")


def empty_events():
    return {k: np.zeros(0, dtype=np.float64 if k == "proportion" else np.int32)
            for k in EVENT_FIELDS}


def make_events(event, time, node, dest, n, proportion, select, shift, sort=True):
    """Event arrays, stably sorted by (time, event, select) like
    R/SimInf_events.R:398 when ``sort`` is true."""
    ev = {
        "event": np.asarray(event, dtype=np.int32),
        "time": np.asarray(time, dtype=np.int32),
        "node": np.asarray(node, dtype=np.int32),
        "dest": np.asarray(dest, dtype=np.int32),
        "n": np.asarray(n, dtype=np.int32),
        "proportion": np.asarray(proportion, dtype=np.float64),
        "select": np.asarray(select, dtype=np.int32),
        "shift": np.asarray(shift, dtype=np.int32),
    }
    m = max(v.size for v in ev.values())
    for k in EVENT_FIELDS:
        ev[k] = np.broadcast_to(ev[k].reshape(-1), (m,)).copy() if ev[k].size == 1 else ev[k]
    if sort and m:
        order = np.lexsort((ev["select"], ev["event"], ev["time"]))
        ev = {k: np.ascontiguousarray(v[order]) for k, v in ev.items()}
    return ev


class SimInfModel:
    """The solver-facing slots of a SimInf_model."""

    def __init__(self, name, G, S, u0, tspan, v0=None, ldata=None, gdata=None,
                 E=None, N=None, events=None, replicates=1):
        self.name = name
        self.G = np.asarray(G, dtype=np.int32)
        self.S = np.asarray(S, dtype=np.int32)
        self.u0 = np.asarray(u0, dtype=np.int32)
        if self.u0.ndim == 1:
            self.u0 = self.u0.reshape(-1, 1)
        self.tspan = np.asarray(tspan, dtype=np.float64)
        self.replicates = int(replicates)
        ncol = self.u0.shape[1]
        if ncol % self.replicates:
            raise ValueError("ncol(u0) must be a multiple of replicates")
        self.Nn = ncol // self.replicates
        self.Nc = self.S.shape[0]
        self.Nt = self.S.shape[1]
        self.v0 = np.zeros((0, ncol)) if v0 is None else np.asarray(v0, dtype=np.float64)
        if self.v0.ndim == 1:
            self.v0 = self.v0.reshape(1, -1)
        self.Nd = self.v0.shape[0]
        self.ldata = np.zeros((0, self.Nn)) if ldata is None else np.asarray(ldata, dtype=np.float64)
        if self.ldata.ndim == 1:
            self.ldata = self.ldata.reshape(-1, 1)
        self.Nld = self.ldata.shape[0]
        self.gdata = np.zeros(0) if gdata is None else np.asarray(gdata, dtype=np.float64).reshape(-1)
        self.E = None if E is None else np.asarray(E, dtype=np.float64)
        self.N = None if N is None else np.asarray(N, dtype=np.int32)
        self.events = empty_events() if events is None else events
        if self.G.shape != (self.Nt, self.Nt):
            raise ValueError("G must be Nt x Nt")
        if self.u0.shape[0] != self.Nc:
            raise ValueError("u0 must have Nc rows")

    def replicate(self, n):
        """The same model with n replicates of u0/v0 (R's replicates slot)."""
        u0 = np.tile(self.u0[:, :self.Nn], (1, n))
        v0 = np.tile(self.v0[:, :self.Nn], (1, n)) if self.Nd else None
        m = SimInfModel(self.name, self.G, self.S, u0, self.tspan, v0=v0,
                        ldata=self.ldata, gdata=self.gdata, E=self.E, N=self.N,
                        events=self.events, replicates=n)
        if hasattr(self, "C_code"):
            m.C_code = self.C_code
        return m


def _rep_ldata(n, *params):
    return np.vstack([np.broadcast_to(np.asarray(p, dtype=np.float64), (n,)) for p in params])


def SIR(u0, tspan, beta, gamma, events=None):
    """u0: array (3, Nn) or dict with S, I, R."""
    u0 = _u0(u0, ("S", "I", "R"))
    G = np.ones((2, 2), dtype=np.int32)
    S = np.array([[-1, 0], [1, -1], [0, 1]], dtype=np.int32)
    E = np.array([[1, 0, 0, 1], [0, 1, 0, 1], [0, 0, 1, 1]], dtype=np.float64)
    return SimInfModel("SIR", G, S, u0, tspan, ldata=_rep_ldata(u0.shape[1], beta, gamma),
                       E=E, events=events)


def SEIR(u0, tspan, beta, epsilon, gamma, events=None):
    """u0: array (4, Nn) or dict with S, E, I, R."""
    u0 = _u0(u0, ("S", "E", "I", "R"))
    G = np.ones((3, 3), dtype=np.int32)
    S = np.array([[-1, 0, 0], [1, -1, 0], [0, 1, -1], [0, 0, 1]], dtype=np.int32)
    E = np.array([[1, 1], [0, 1], [0, 1], [0, 1]], dtype=np.float64)
    return SimInfModel("SEIR", G, S, u0, tspan,
                       ldata=_rep_ldata(u0.shape[1], beta, epsilon, gamma), E=E, events=events)


def SIS(u0, tspan, beta, gamma, events=None):
    u0 = _u0(u0, ("S", "I"))
    G = np.ones((2, 2), dtype=np.int32)
    S = np.array([[-1, 1], [1, -1]], dtype=np.int32)
    E = np.array([[1, 1], [0, 1]], dtype=np.float64)
    return SimInfModel("SIS", G, S, u0, tspan, ldata=_rep_ldata(u0.shape[1], beta, gamma),
                       E=E, events=events)


def SISe(u0, tspan, phi, upsilon, gamma, alpha, beta_t1, beta_t2, beta_t3, beta_t4,
         end_t1, end_t2, end_t3, end_t4, epsilon, events=None):
    u0 = _u0(u0, ("S", "I"))
    n = u0.shape[1]
    G = np.ones((2, 2), dtype=np.int32)
    S = np.array([[-1, 1], [1, -1]], dtype=np.int32)
    E = np.array([[1, 1], [0, 1]], dtype=np.float64)
    ldata = _rep_ldata(n, end_t1, end_t2, end_t3, end_t4)
    gdata = np.array([upsilon, gamma, alpha, beta_t1, beta_t2, beta_t3, beta_t4, epsilon],
                     dtype=np.float64)
    v0 = np.broadcast_to(np.asarray(phi, dtype=np.float64), (n,)).reshape(1, n)
    return SimInfModel("SISe", G, S, u0, tspan, v0=v0, ldata=ldata, gdata=gdata,
                       E=E, events=events)


def SISe3(u0, tspan, phi, upsilon_1, upsilon_2, upsilon_3, gamma_1, gamma_2, gamma_3,
          alpha, beta_t1, beta_t2, beta_t3, beta_t4, end_t1, end_t2, end_t3, end_t4,
          epsilon, events=None):
    """R/SISe3.R:56-61 (E), :158-197 (N, G, S, v0, ldata, gdata)."""
    u0 = _u0(u0, ("S_1", "I_1", "S_2", "I_2", "S_3", "I_3"))
    n = u0.shape[1]
    E = np.zeros((6, 6))
    for col, rows in enumerate(([0], [2], [4], [0, 1], [2, 3], [4, 5])):
        E[rows, col] = 1
    N = np.array([[2, 0, 0], [2, 0, -1], [0, 2, 0], [0, 2, -1], [0, 0, 0], [0, 0, -1]],
                 dtype=np.int32)
    G = np.zeros((6, 6), dtype=np.int32)
    S = np.zeros((6, 6), dtype=np.int32)
    for a in range(3):
        G[2 * a:2 * a + 2, 2 * a:2 * a + 2] = 1
        S[2 * a, 2 * a], S[2 * a + 1, 2 * a] = -1, 1
        S[2 * a, 2 * a + 1], S[2 * a + 1, 2 * a + 1] = 1, -1
    ldata = _rep_ldata(n, end_t1, end_t2, end_t3, end_t4)
    gdata = np.array([upsilon_1, upsilon_2, upsilon_3, gamma_1, gamma_2, gamma_3, alpha,
                      beta_t1, beta_t2, beta_t3, beta_t4, epsilon], dtype=np.float64)
    v0 = np.broadcast_to(np.asarray(phi, dtype=np.float64), (n,)).reshape(1, n)
    return SimInfModel("SISe3", G, S, u0, tspan, v0=v0, ldata=ldata, gdata=gdata,
                       E=E, N=N, events=events)


def distance_matrix(x, y, cutoff, min_dist=None):
    """Euclidean distances between the nodes at (x, y) that are at most
    cutoff apart, as the reference's distance_matrix() builds them
    (src/misc/SimInf_distance_matrix.c:24-83): a CSC matrix (i, p, d) whose
    column j lists node j's neighbours in node order; coincident nodes get
    min_dist, which must then be given and > 0."""
    x = np.asarray(x, dtype=np.float64)
    y = np.asarray(y, dtype=np.float64)
    n = len(x)
    if n < 1 or len(y) != n:
        raise ValueError("'x' and 'y' must be numeric vectors of one length > 0.")
    if not np.isfinite(cutoff) or cutoff < 0:
        raise ValueError("'cutoff' must be > 0.")
    ii, pp, dd = [], [0], []
    for col in range(n):
        d = np.hypot(x[col] - x, y[col] - y)
        if not np.isfinite(d).all():
            raise ValueError("Invalid distance for i=%d." % col)
        rows = np.nonzero(d <= cutoff)[0]
        rows = rows[rows != col]
        dist = d[rows]
        if (dist <= 0).any():
            if min_dist is None or not np.isfinite(min_dist) or min_dist < 0:
                raise ValueError("Invalid 'min_dist' argument. Please provide 'min_dist' > 0.")
            dist = np.where(dist <= 0, min_dist, dist)
        ii.extend(rows.tolist())
        dd.extend(dist.tolist())
        pp.append(len(ii))
    return (np.array(ii, dtype=np.int32), np.array(pp, dtype=np.int32),
            np.array(dd, dtype=np.float64))


def ldata_sp(data, distance, metric=1):
    """Local data with the spatial coupling appended, as SimInf_ldata_sp
    packs it (src/misc/SimInf_ldata.c:50-135): for each node its rows of
    data, then (neighbour index, value) pairs and a (-1, 0) stop pair, zero
    padded to the longest list.  value is the neighbour's degree (metric
    0), the distance (1) or 1 / distance^2 (2)."""
    data = np.asarray(data, dtype=np.float64)
    if data.ndim == 1:
        data = data.reshape(-1, 1)
    ir, jc, d = distance
    n = data.shape[1]
    if len(jc) - 1 != n:
        raise ValueError("The number of nodes in 'data' and 'distance' are not equal.")
    degree = np.diff(jc)
    nld = data.shape[0] + (int(degree.max(initial=0)) + 1) * 2
    out = np.zeros((nld, n))
    out[:data.shape[0], :] = data
    for node in range(n):
        k = data.shape[0]
        for e in range(jc[node], jc[node + 1]):
            out[k, node] = ir[e]
            out[k + 1, node] = (degree[ir[e]] if metric == 0 else
                                d[e] if metric == 1 else 1.0 / (d[e] * d[e]))
            k += 2
        out[k, node] = -1.0
    return out


def SISe_sp(u0, tspan, phi, upsilon, gamma, alpha, beta_t1, beta_t2, beta_t3, beta_t4,
            end_t1, end_t2, end_t3, end_t4, coupling, distance, events=None):
    """R/SISe_sp.R:139-183: SISe whose environmental pressure spreads to
    proximal nodes; ldata = end_t1..end_t4 then the neighbours (distances)
    of ldata_sp(metric 1), gdata = upsilon, gamma, alpha, beta_t1..beta_t4,
    coupling.  distance is the (i, p, x) of distance_matrix()."""
    u0 = _u0(u0, ("S", "I"))
    n = u0.shape[1]
    G = np.ones((2, 2), dtype=np.int32)
    S = np.array([[-1, 1], [1, -1]], dtype=np.int32)
    E = np.array([[1, 1], [0, 1]], dtype=np.float64)
    ldata = ldata_sp(_rep_ldata(n, end_t1, end_t2, end_t3, end_t4), distance, 1)
    gdata = np.array([upsilon, gamma, alpha, beta_t1, beta_t2, beta_t3, beta_t4, coupling],
                     dtype=np.float64)
    v0 = np.broadcast_to(np.asarray(phi, dtype=np.float64), (n,)).reshape(1, n)
    return SimInfModel("SISe_sp", G, S, u0, tspan, v0=v0, ldata=ldata, gdata=gdata,
                       E=E, events=events)


def SISe3_sp(u0, tspan, phi, upsilon_1, upsilon_2, upsilon_3, gamma_1, gamma_2, gamma_3,
             alpha, beta_t1, beta_t2, beta_t3, beta_t4, end_t1, end_t2, end_t3, end_t4,
             coupling, distance, events=None):
    """R/SISe3_sp.R: SISe3 with the spatial coupling of SISe_sp; gdata =
    upsilon_1..3, gamma_1..3, alpha, beta_t1..beta_t4, coupling."""
    m = SISe3(u0, tspan, phi, upsilon_1, upsilon_2, upsilon_3, gamma_1, gamma_2, gamma_3,
              alpha, beta_t1, beta_t2, beta_t3, beta_t4, end_t1, end_t2, end_t3, end_t4,
              coupling, events=events)
    return SimInfModel("SISe3_sp", m.G, m.S, m.u0, tspan, v0=m.v0,
                       ldata=ldata_sp(m.ldata, distance, 1), gdata=m.gdata, E=m.E, N=m.N,
                       events=events)


def SIR_mparse(u0, tspan, beta, gamma, events=None):
    """mparse(transitions = c("S -> beta*S*I/N -> I", "I -> gamma*I -> R",
    "N <- S+I+R"), compartments = c("S","I","R"), gdata = c(beta, gamma)).
    G = (depends %*% abs(S)) > 0 (R/mparse.R:485-491) is all ones here."""
    u0 = _u0(u0, ("S", "I", "R"))
    G = np.ones((2, 2), dtype=np.int32)
    S = np.array([[-1, 0], [1, -1], [0, 1]], dtype=np.int32)
    E = np.array([[1, 0, 0, 1], [0, 1, 0, 1], [0, 0, 1, 1]], dtype=np.float64)
    return SimInfModel("SIR_mparse", G, S, u0, tspan, gdata=np.array([beta, gamma]),
                       E=E, events=events)


def SISe_pf(u0, tspan, upsilon, gamma, phi0=0.0, events=None):
    """mparse(transitions = c("S -> upsilon*phi*S -> I", "I -> gamma*I -> S"),
    compartments = c("S","I"), v0 = phi, gdata = c(upsilon, gamma),
    pts_fun = phi <- phi*(1-0.03) + 0.05*I/(S+I))."""
    u0 = _u0(u0, ("S", "I"))
    n = u0.shape[1]
    G = np.ones((2, 2), dtype=np.int32)
    S = np.array([[-1, 1], [1, -1]], dtype=np.int32)
    E = np.array([[1, 0, 1], [0, 1, 1]], dtype=np.float64)
    v0 = np.full((1, n), phi0, dtype=np.float64)
    return SimInfModel("SISe_pf", G, S, u0, tspan, v0=v0, gdata=np.array([upsilon, gamma]),
                       E=E, events=events)


def _u0(u0, names):
    if isinstance(u0, dict):
        cols = [np.atleast_1d(np.asarray(u0[k])) for k in names]
        n = max(len(c) for c in cols)
        return np.vstack([np.broadcast_to(c, (n,)) for c in cols]).astype(np.int32)
    a = np.asarray(u0, dtype=np.int32)
    if a.ndim == 1:
        a = a.reshape(-1, 1)
    if a.shape[0] != len(names):
        raise ValueError("u0 must have rows %s" % (names,))
    return a


__all__ = ["SimInfModel", "SIR", "SEIR", "SIS", "SISe", "SISe3", "SIR_mparse", "SISe_pf",
           "SISe_sp", "SISe3_sp", "distance_matrix", "ldata_sp",
           "make_events", "empty_events", "EXIT_EVENT", "ENTER_EVENT",
           "INTERNAL_TRANSFER_EVENT", "EXTERNAL_TRANSFER_EVENT"]
