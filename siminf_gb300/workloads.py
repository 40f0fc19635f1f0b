"""Seeded synthetic workloads of the benchmark configurations.

No dataset ships with the reference for this path (its data/*.rda files are
examples that need R), so every workload is generated here from fixed seeds.

- ``sir_plain``  -- mparse SIR, 1,000 nodes of (S=99, I=5, R=0), beta=0.16,
  gamma=0.077, tspan 1:150, no events.
- ``seir_events`` -- built-in SEIR (beta=0.16, epsilon=0.25, gamma=0.077),
  Nn nodes with S ~ Poisson(300), E = 0, I ~ Bernoulli(0.01) * Poisson(3),
  R = 0, run for `days` days.  Every node-day: an enter event with
  probability 0.002 (1 individual into S, select column 1 = {S}) and an exit
  event with probability 0.002 (1 individual from {S,E,I,R}, select column
  2, equal weights -> hypergeometric).  External transfers:
  `transfers` per day drawn uniformly from a fixed random directed graph of
  4 * transfers edges.  Edge sources are uniform.  Edge destinations are
  drawn with probability proportional to a weight from a power law with
  exponent 2.1 (Pareto shape 1.1), truncated at the structural cutoff
  sqrt(edges) of an uncorrelated scale-free graph (Boguna, Pastor-Satorras
  & Vespignani, Eur. Phys. J. B 38, 2004), so destination in-degree follows
  the power law up to that cutoff.  Without the cutoff one node collects
  most of the population within weeks and fires ~90% of all transitions,
  which turns the benchmark into a single sequential chain.  Each transfer
  moves n = 1 + Poisson(3) individuals from {S,E,I,R}.  Sizes are capped
  at what the source holds at run time (solver option cap_transfers); the
  reference would instead stop with "Unable to sample individuals for
  event."
  Seeds: 1 graph, 2 u0, 3 events.
- ``abc_models`` -- the ABC workload over uneven models: SEIR as in
  ``seir_events`` with node counts drawn from {100, 1000, 10000, 50000}
  (weights 0.4, 0.3, 0.2, 0.1), tspan 1..T with T ~ U{60, 365}, events and
  graph scaled to the node count (transfers per day = Nn / 2), parameters
  from the priors beta ~ U(0.05, 0.5), epsilon ~ U(0.1, 0.5), gamma ~
  U(0.02, 0.2).  The target is the prevalence I/N of one such model run
  with seed 7.  Generated day-vectorised from one seed per model.
- ``sise_pfilter`` -- the particle-filter workload: mparse SISe
  ("S -> upsilon*phi*S -> I", "I -> gamma*I -> S", phi <- phi*(1-0.03) +
  0.05*I/(S+I)), `nodes` nodes with S ~ Poisson(100), I ~ Bernoulli(0.05) *
  Poisson(2), phi0 = 0.  Observations: Binomial(I, 0.8) per node every 7
  days over 52 weeks from one ground-truth run (upsilon = 0.012, gamma =
  0.1, seed 7).  Particles carry their own upsilon ~ U(0.005, 0.03) and
  gamma ~ U(0.05, 0.2).
- ``livestock_register`` -- individual events of a livestock register for
  the individual-event cleaner: births on a holding, Poisson(2) moves
  (capped at 6) a month apart, 70% exits, 3% of recorded sources wrong.
"""
import numpy as np

from . import model as M


def sir_plain(nodes=1000, days=150):
    u0 = {"S": np.full(nodes, 99), "I": np.full(nodes, 5), "R": np.zeros(nodes)}
    return M.SIR_mparse(u0, np.arange(1, days + 1, dtype=float), beta=0.16, gamma=0.077)


def powerlaw_graph(nodes, edges, seed=1, exponent=2.1, cutoff=None):
    """Fixed directed graph: uniform sources, destinations drawn with
    probability proportional to power-law weights with the given exponent
    on [1, cutoff] (default cutoff sqrt(edges); np.inf: no cutoff, the
    plain power law)."""
    rng = np.random.default_rng(seed)
    a = exponent - 1.0
    K = float(cutoff if cutoff is not None else np.sqrt(edges))
    u = rng.random(nodes)
    # truncated Pareto(a) on [1, K]; K = inf gives the untruncated law
    w = (1.0 - u * (1.0 - (0.0 if np.isinf(K) else K ** -a))) ** (-1.0 / a)
    p = w / w.sum()
    src = rng.integers(0, nodes, edges).astype(np.int32)
    dst = rng.choice(nodes, size=edges, p=p).astype(np.int32)
    same = src == dst
    dst[same] = (dst[same] + 1) % nodes
    return src, dst


def seir_events(nodes=1_000_000, days=365, transfers=500_000, p_enter=0.002, p_exit=0.002,
                graph_edges=None, seeds=(1, 2, 3), transfer_n=None, cutoff=None):
    """Config 2 (see module docstring).  Events are produced in the order
    R/SimInf_events.R:398 sorts them: by time, exits, enters, transfers.
    transfer_n: a fixed transfer size instead of 1 + Poisson(3) (n = 1 is
    the balanced variant the reference runs without capping for a few
    months); cutoff: the graph's power-law cutoff (powerlaw_graph)."""
    g_seed, u_seed, e_seed = seeds
    rng_u = np.random.default_rng(u_seed)
    S = rng_u.poisson(300, nodes)
    I = rng_u.poisson(3, nodes) * (rng_u.random(nodes) < 0.01)
    u0 = np.vstack([S, np.zeros(nodes), I, np.zeros(nodes)]).astype(np.int32)

    gsrc, gdst = powerlaw_graph(nodes, graph_edges or 4 * transfers, seed=g_seed,
                                cutoff=cutoff)
    rng = np.random.default_rng(e_seed)
    chunks = {k: [] for k in ("event", "time", "node", "dest", "n", "select")}
    for t in range(1, days + 1):
        ex = np.nonzero(rng.random(nodes) < p_exit)[0].astype(np.int32)
        en = np.nonzero(rng.random(nodes) < p_enter)[0].astype(np.int32)
        pick = rng.integers(0, len(gsrc), transfers)
        n = (1 + rng.poisson(3, transfers)).astype(np.int32)
        if transfer_n is not None:
            n[:] = transfer_n
        m = len(ex) + len(en) + transfers
        chunks["event"].append(np.concatenate([np.zeros(len(ex), np.int32),
                                               np.ones(len(en), np.int32),
                                               np.full(transfers, 3, np.int32)]))
        chunks["time"].append(np.full(m, t, np.int32))
        chunks["node"].append(np.concatenate([ex + 1, en + 1, gsrc[pick] + 1]).astype(np.int32))
        chunks["dest"].append(np.concatenate([np.zeros(len(ex) + len(en), np.int32),
                                              gdst[pick] + 1]).astype(np.int32))
        chunks["n"].append(np.concatenate([np.ones(len(ex) + len(en), np.int32), n]))
        chunks["select"].append(np.concatenate([np.full(len(ex), 2, np.int32),
                                                np.ones(len(en), np.int32),
                                                np.full(transfers, 2, np.int32)]))
    ev = {k: np.concatenate(v) for k, v in chunks.items()}
    total = len(ev["event"])
    ev["proportion"] = np.zeros(total)
    ev["shift"] = np.zeros(total, np.int32)
    return M.SEIR(u0, np.arange(1, days + 1, dtype=float), beta=0.16, epsilon=0.25,
                  gamma=0.077, events=ev)


def seir_events_fast(nodes, days, transfers, rng, beta=0.16, epsilon=0.25, gamma=0.077,
                     p_enter=0.002, p_exit=0.002, tspan0=1):
    """``seir_events`` generated with whole-horizon draws instead of a loop
    over days (same distributions, different draws)."""
    S = rng.poisson(300, nodes)
    I = rng.poisson(3, nodes) * (rng.random(nodes) < 0.01)
    u0 = np.vstack([S, np.zeros(nodes), I, np.zeros(nodes)]).astype(np.int32)
    a = 1.1
    edges = 4 * transfers
    K = float(np.sqrt(edges))
    w = (1.0 - rng.random(nodes) * (1.0 - K ** -a)) ** (-1.0 / a)
    gsrc = rng.integers(0, nodes, edges).astype(np.int32)
    gdst = rng.choice(nodes, size=edges, p=w / w.sum()).astype(np.int32)
    same = gsrc == gdst
    gdst[same] = (gdst[same] + 1) % nodes
    t_days = np.arange(tspan0, tspan0 + days, dtype=np.int32)
    ex_t, ex_n = np.nonzero(rng.random((days, nodes)) < p_exit)
    en_t, en_n = np.nonzero(rng.random((days, nodes)) < p_enter)
    pick = rng.integers(0, edges, (days, transfers))
    tr_n = (1 + rng.poisson(3, (days, transfers))).astype(np.int32)
    # per day: exits, enters, transfers (the order R/SimInf_events.R:398 gives)
    kinds = [(ex_t, ex_n, 0), (en_t, en_n, 1)]
    parts = {k: [] for k in ("event", "time", "node", "dest", "n", "select")}
    order_key = []
    for tt, nn, kind in kinds:
        parts["event"].append(np.full(len(tt), kind, np.int32))
        parts["time"].append(t_days[tt])
        parts["node"].append((nn + 1).astype(np.int32))
        parts["dest"].append(np.zeros(len(tt), np.int32))
        parts["n"].append(np.ones(len(tt), np.int32))
        parts["select"].append(np.full(len(tt), 2 if kind == 0 else 1, np.int32))
        order_key.append(tt.astype(np.int64) * 3 + kind)
    td = np.repeat(np.arange(days), transfers)
    parts["event"].append(np.full(td.size, 3, np.int32))
    parts["time"].append(t_days[td])
    parts["node"].append(gsrc[pick.reshape(-1)] + 1)
    parts["dest"].append(gdst[pick.reshape(-1)] + 1)
    parts["n"].append(tr_n.reshape(-1))
    parts["select"].append(np.full(td.size, 2, np.int32))
    order_key.append(td.astype(np.int64) * 3 + 2)
    order = np.argsort(np.concatenate(order_key), kind="stable")
    ev = {k: np.concatenate(v)[order] for k, v in parts.items()}
    ev["proportion"] = np.zeros(len(order))
    ev["shift"] = np.zeros(len(order), np.int32)
    return M.SEIR(u0, np.arange(tspan0, tspan0 + days, dtype=float), beta=beta,
                  epsilon=epsilon, gamma=gamma, events=ev)


def abc_models(n, seed=11, sizes=(100, 1000, 10000, 50000), weights=(0.4, 0.3, 0.2, 0.1),
               day_range=(60, 365)):
    """n proposals of the ABC workload (see module docstring): models and
    their seeds, plus the target prevalence series (I/N of the seed-7
    model over the longest tspan) cut to each model's tspan."""
    rng = np.random.default_rng(seed)
    models, seeds = [], []
    for j in range(n):
        Nn = int(rng.choice(sizes, p=weights))
        T = int(rng.integers(day_range[0], day_range[1] + 1))
        models.append(seir_events_fast(Nn, T, max(1, Nn // 2), rng,
                                       beta=rng.uniform(0.05, 0.5),
                                       epsilon=rng.uniform(0.1, 0.5),
                                       gamma=rng.uniform(0.02, 0.2)))
        seeds.append(int(rng.integers(1, 2 ** 62)))
    return models, seeds


def sise_pfilter(nodes=500, particles=4096, weeks=52, seed=7):
    """The particle-filter workload (see module docstring).  Returns the
    model, per-particle gdata (particles x 2), observation times and the
    (weeks x nodes) observations."""
    from .run import run
    rng = np.random.default_rng(seed)
    S = rng.poisson(100, nodes)
    I = rng.poisson(2, nodes) * (rng.random(nodes) < 0.05)
    u0 = np.vstack([S, I]).astype(np.int32)
    days = 7 * weeks
    truth = M.SISe_pf(u0, np.arange(0, days + 1, dtype=float), upsilon=0.012, gamma=0.1)
    res = run(truth, seed=seed)
    obs_time = np.arange(7, days + 1, 7, dtype=np.int32)
    I_true = res.U[1::2, :][:, obs_time]
    obs = rng.binomial(I_true.T, 0.8).astype(np.int32)
    model = M.SISe_pf(u0, np.array([0.0]), upsilon=0.012, gamma=0.1)
    gdata = np.column_stack([rng.uniform(0.005, 0.03, particles),
                             rng.uniform(0.05, 0.2, particles)])
    return model, gdata, obs_time, obs


def livestock_register(n_ind, n_nodes, seed):
    """Synthetic individual events of a livestock register, as
    individual_events() hands them to its C core: n_ind animals, each born
    (enter) on one of n_nodes holdings, moved 0-6 times (Poisson(2)
    capped) between holdings about a month apart, 70% leaving by exit; 3%
    of the recorded sources are wrong, so the search has paths to reject.
    int32 columns (id, event, time, node, dest), dest NA = INT_MIN except
    for transfers, sorted by (id, time, event, node, dest), no repeats."""
    NA = np.iinfo(np.int32).min
    rng = np.random.default_rng(seed)
    moves = np.minimum(rng.poisson(2.0, size=n_ind), 6)
    has_exit = rng.random(n_ind) < 0.7
    per = 1 + moves + has_exit
    n = int(per.sum())
    id_ = np.repeat(np.arange(1, n_ind + 1, dtype=np.int64), per)
    k = np.arange(n) - np.repeat(np.cumsum(per) - per, per)   # position within the animal
    last = k == np.repeat(per - 1, per)
    event = np.where(k == 0, 1, 3)
    event[last & np.repeat(has_exit, per)] = 0
    time = np.repeat(rng.integers(0, 3000, size=n_ind), per) + 30 * k + rng.integers(0, 29, size=n)
    hold = rng.integers(1, n_nodes + 1, size=n)               # the holding after each event
    hold[event == 0] = hold[np.flatnonzero(event == 0) - 1]   # an exit leaves it where it was
    node = hold.copy()
    node[k > 0] = hold[np.flatnonzero(k > 0) - 1]             # events start where it was
    wrong = (rng.random(n) < 0.03) & (k > 0)
    node[wrong] = rng.integers(1, n_nodes + 1, size=int(wrong.sum()))
    dest = np.where(event == 3, hold, NA)
    dkey = np.where(dest == NA, np.int64(1) << 40, dest)
    o = np.lexsort((dkey, node, event, time, id_))
    return [np.ascontiguousarray(np.asarray(c)[o], dtype=np.int32)
            for c in (id_, event, time, node, dest)]
