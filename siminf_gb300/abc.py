"""ABC-SMC over the device batch: the generation loop of the reference's
abc (R/abc.R:742-843, abc_internal) and continue_abc (R/abc.R:996-1027),
with its proposal and weight kernels
(src/misc/SimInf_abc.c, SimInf_abc_proposals and SimInf_abc_weights)
restated in numpy, and every generation's simulations run as batches of
uneven models on the GPU with their prevalence distances reduced there
(siminf_gpu_run_batch, run.run_batch).

Per generation:
  * proposals: the first generation samples the priors; later ones pick
    an ancestor by its weight (inverse of the weights' running sum, as the
    C code's binary search) and perturb it with a multivariate normal of
    covariance sigma = 2 cov(x) (R/abc.R:334-338), redrawing until every
    prior density is positive (SimInf_abc.c:171-236);
  * acceptance: every distance <= the generation's tolerance
    (R/abc.R:553-560); proposals run in batches until n_particles are
    accepted, keeping the first n_particles in proposal order;
  * weights: log prior density minus log sum_j w_j N(x_i; x_j, sigma),
    then exp after subtracting the maximum and normalised
    (SimInf_abc.c:296-395); the first generation's are uniform.

The tolerances are given (the reference's `tolerance` matrix, one
statistic), or chosen as the reference's first epsilon from n_init prior
draws (R/abc.R:429-432) and then, per later generation, a quantile of the
previous generation's accepted distances (the median by default).  The
reference's adaptive rule (Simola et al. 2021, abc_adaptive_tolerance) is
not restated: the quantile rule stands in for it here.  Random numbers come from numpy's Generator
seeded by `seed`, not R's: runs are reproducible but not R's draws.
"""
import sys
import time

import numpy as np

from .run import run_batch


class Prior:
    """One parameter's prior: distribution 'uniform', 'normal',
    'lognormal' or 'gamma' (the C code's 'u', 'n', 'l', 'g') with its two
    parameters as R's (min/max, mean/sd, meanlog/sdlog, shape/rate)."""

    def __init__(self, name, distribution, p1, p2):
        if distribution not in ("uniform", "normal", "lognormal", "gamma"):
            raise ValueError("Unknown distribution.")
        self.name, self.distribution, self.p1, self.p2 = name, distribution, float(p1), float(p2)

    def sample(self, rng, n):
        d = self.distribution
        if d == "uniform":
            return rng.uniform(self.p1, self.p2, n)
        if d == "normal":
            return rng.normal(self.p1, self.p2, n)
        if d == "lognormal":
            return rng.lognormal(self.p1, self.p2, n)
        return rng.gamma(self.p1, 1.0 / self.p2, n)

    def log_density(self, x, parent):
        """The C code's log density of a proposal x; 'normal' and
        'lognormal' are centred on the particle it came from (parent), as
        SimInf_abc.c does."""
        d = self.distribution
        x = np.asarray(x, float)
        with np.errstate(divide="ignore", invalid="ignore"):
            if d == "uniform":
                inside = (x >= self.p1) & (x <= self.p2)
                return np.where(inside, -np.log(self.p2 - self.p1), -np.inf)
            if d == "normal":
                z = (x - parent) / self.p2
                return -0.5 * z * z - np.log(self.p2 * np.sqrt(2 * np.pi))
            if d == "lognormal":
                lx = np.log(np.where(x > 0, x, np.nan))
                z = (lx - parent) / self.p2
                out = -0.5 * z * z - np.log(self.p2 * np.sqrt(2 * np.pi)) - lx
                return np.where(x > 0, out, -np.inf)
            k, rate = self.p1, self.p2
            from math import lgamma
            out = k * np.log(rate) - lgamma(k) + (k - 1) * np.log(np.where(x > 0, x, np.nan)) - rate * x
            return np.where(x > 0, out, -np.inf)


def proposals(priors, n, rng, x=None, w=None, sigma=None):
    """n proposals (n x d) and their ancestors (-1 in the first
    generation), SimInf_abc_proposals."""
    d = len(priors)
    if x is None:
        return np.column_stack([p.sample(rng, n) for p in priors]), np.full(n, -1)
    if np.any(~np.isfinite(w)) or np.any(w < 0):
        raise ValueError("Invalid weight detected (non-finite or < 0.0).")
    cdf = np.cumsum(w)
    L = np.linalg.cholesky(sigma)
    out = np.empty((n, d))
    anc = np.empty(n, dtype=np.int64)
    todo = np.arange(n)
    while len(todo):
        r = rng.random(len(todo)) * cdf[-1]
        j = np.minimum(np.searchsorted(cdf, r, side="right"), len(cdf) - 1)
        prop = x[j] + rng.standard_normal((len(todo), d)) @ L.T
        ok = np.ones(len(todo), bool)
        for k, p in enumerate(priors):
            ok &= np.isfinite(p.log_density(prop[:, k], x[j, k])) & \
                (np.exp(p.log_density(prop[:, k], x[j, k])) > 0)
        out[todo[ok]] = prop[ok]
        anc[todo[ok]] = j[ok]
        todo = todo[~ok]
    return out, anc


def weights(priors, x_anc, xx, x, w, sigma):
    """Normalised importance weights of the new particles xx
    (SimInf_abc_weights): x_anc are their ancestors' values, x and w the
    previous generation's particles and weights."""
    n, d = xx.shape
    if w is None:
        return np.full(n, 1.0 / n)
    lw = np.zeros(n)
    for k, p in enumerate(priors):
        lw += p.log_density(xx[:, k], x_anc[:, k])
    if not np.all(np.isfinite(lw)):
        raise ValueError("Invalid weight detected (non-finite or < 0.0).")
    inv = np.linalg.inv(sigma)
    norm = 1.0 / np.sqrt((2 * np.pi) ** d * np.linalg.det(sigma))
    s = np.zeros(n)
    for j0 in range(0, len(x), 1024):            # pdf of every (new, old) pair, in blocks
        diff = xx[:, None, :] - x[None, j0:j0 + 1024, :]
        q = np.einsum("ijk,kl,ijl->ij", diff, inv, diff)
        s += (norm * np.exp(-0.5 * q)) @ w[j0:j0 + 1024]
    lw -= np.log(s)
    lw -= max(lw.max(), 0.0)
    ww = np.exp(lw)
    return ww / ww.sum()


class Generation:
    """One generation's result: particles, weights, distances, tolerance,
    proposals made, ESS and wall time."""

    def __init__(self, x, w, distance, tolerance, nprop, seconds, node_days):
        self.x, self.w, self.distance, self.tolerance = x, w, distance, tolerance
        self.nprop, self.seconds, self.node_days = nprop, seconds, node_days
        self.ess = 1.0 / float(np.sum(w * w))


class ABCResult(list):
    """The generations of an ABC-SMC run (a list of Generation), with what
    continue_abc needs to add generations as if the run had not stopped:
    the random generator's state and the next generation's tolerance."""

    def __init__(self, gens, priors, n_particles, batch, quantile, rng, next_eps):
        super().__init__(gens)
        self.priors, self.n_particles, self.batch = priors, n_particles, batch
        self.quantile, self.rng, self.next_eps = quantile, rng, next_eps


def abc_smc(simulate, priors, n_particles, generations, batch=2048, tolerance=None,
            n_init=None, seed=1, verbose=False, quantile=0.5):
    """ABC-SMC.  simulate(theta_batch, rng) -> (models, seeds, targets) for
    the proposals' parameter rows; their distances come from run_batch.
    tolerance: one value per generation, or None for the first epsilon
    from n_init prior draws and after it the `quantile` of the previous
    generation's accepted distances.  Returns an ABCResult (the list of
    Generation)."""
    if not 0.0 < quantile <= 1.0:
        raise ValueError("'quantile' must be in (0, 1].")
    if tolerance is None and n_init is None:
        raise ValueError("Both 'n_init' and 'tolerance' can not be NULL.")
    eps = None if tolerance is None else float(tolerance[0])
    return _generations(simulate, priors, n_particles, generations, batch, tolerance, n_init,
                        np.random.default_rng(seed), verbose, quantile, [], None, None, eps)


def continue_abc(result, simulate, generations, tolerance=None, verbose=False):
    """More generations of an ABC-SMC run (R/abc.R:996-1027, continue_abc):
    from its last generation's particles and weights, with the next
    tolerances given (one per generation) or by the run's quantile rule, and
    the run's random generator where it stopped -- so that a run continued
    for k generations equals the same run made k generations longer.
    Returns a new ABCResult holding every generation."""
    if not len(result):
        raise ValueError("The ABC run has no generation to continue from.")
    last = result[-1]
    eps = float(tolerance[0]) if tolerance is not None else result.next_eps
    rng = np.random.default_rng()
    rng.bit_generator.state = result.rng.bit_generator.state
    return _generations(simulate, result.priors, result.n_particles, generations, result.batch,
                        tolerance, None, rng, verbose, result.quantile, list(result),
                        last.x, last.w, eps)


def _generations(simulate, priors, n_particles, generations, batch, tolerance, n_init, rng,
                 verbose, quantile, out, x, w, eps):
    """The generation loop shared by abc_smc and continue_abc."""
    if tolerance is not None and len(tolerance) < generations:
        raise ValueError("'tolerance' needs one value per generation.")
    g0 = len(out)
    for g in range(g0, g0 + generations):
        t0 = time.perf_counter()
        sigma = None if x is None else 2.0 * np.atleast_2d(np.cov(x, rowvar=False))
        want = n_particles if (g > 0 or eps is not None) else int(n_init)
        acc_x, acc_d, acc_a = [], [], []
        nprop = 0
        node_days = 0
        while sum(len(a) for a in acc_x) < want:
            theta, anc = proposals(priors, batch, rng, x, w, sigma)
            models, seeds, targets = simulate(theta, rng)
            _, dist = run_batch(models, seeds, targets, cap_transfers=True)
            node_days += sum(m.Nn * len(m.tspan) for m in models)
            ok = np.ones(len(dist), bool) if eps is None else dist <= eps
            need = want - sum(len(a) for a in acc_x)
            idx = np.flatnonzero(ok)[:need]
            nprop += (int(np.flatnonzero(ok)[need - 1]) + 1) if len(idx) == need else batch
            acc_x.append(theta[idx])
            acc_d.append(dist[idx])
            acc_a.append(anc[idx])
        xx = np.concatenate(acc_x)
        dd = np.concatenate(acc_d)
        aa = np.concatenate(acc_a)
        if eps is None:
            # first epsilon: the n_particles-th smallest of the n_init draws
            order = np.argsort(dd, kind="stable")[:n_particles]
            eps = float(dd[order[-1]])
            xx, dd, aa = xx[order], dd[order], aa[order]
        w_new = weights(priors, None if x is None else x[aa], xx, x, w, sigma)
        out.append(Generation(xx, w_new, dd, eps, nprop, time.perf_counter() - t0, node_days))
        if verbose:
            print("generation %d: tolerance %.4g, %d proposals, ESS %.0f, %.1f s"
                  % (g + 1, eps, nprop, out[-1].ess, out[-1].seconds), file=sys.stderr,
                  flush=True)
        x, w = xx, w_new
        k = g - g0 + 1                  # generations of this call done
        if tolerance is not None:
            eps = float(tolerance[k]) if k < len(tolerance) else None
        else:
            eps = float(np.quantile(dd, quantile))
    return ABCResult(out, priors, n_particles, batch, quantile, rng, eps)
