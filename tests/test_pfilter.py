"""Particle filter: the oracle restatement of pfilter_internal
(R/pfilter.R:315-499) and systematic resampling
(src/misc/SimInf_particle_filter.c:33-67), and the GPU version bit for bit
against it."""
import numpy as np
import pytest

from siminf_gb300 import model as M
from oracle import oracle


def small_case(nodes=20, particles=64, weeks=8, seed=3):
    rng = np.random.default_rng(seed)
    u0 = np.vstack([rng.poisson(60, nodes), rng.poisson(3, nodes)]).astype(np.int32)
    m = M.SISe_pf(u0, np.array([0.0]), upsilon=0.02, gamma=0.1)
    obs_time = np.arange(7, 7 * weeks + 1, 7, dtype=np.int32)
    obs = rng.binomial(4, 0.5, size=(weeks, nodes)).astype(np.int32)
    gdata = np.column_stack([rng.uniform(0.005, 0.03, particles),
                             rng.uniform(0.05, 0.2, particles)])
    return m, gdata, obs_time, obs


def _resample_both(w, unif):
    import ctypes as C
    w = np.ascontiguousarray(w, dtype=np.float64)
    n = len(w)
    mine = np.zeros(n, np.int32)
    code = oracle.lib().oracle_systematic_resampling(
        w.ctypes.data_as(C.POINTER(C.c_double)), n, C.c_double(unif),
        mine.ctypes.data_as(C.POINTER(C.c_int)))
    # the reference's search may read one weight past the end: pad it
    padded = np.concatenate([w, [1e300]])
    ref = np.zeros(n, np.int32)
    msg = C.create_string_buffer(256)
    f = oracle.ref_lib().ref_systematic_resampling
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_longlong, C.c_double, C.c_void_p, C.c_char_p, C.c_int]
    code_r = f(padded.ctypes.data, n, unif, ref.ctypes.data, msg, 256)
    return code, mine, code_r, ref, msg.value.decode()


@pytest.mark.skipif(not oracle.ref_available(), reason="oracle/_ref was not built")
def test_resampling_matches_the_reference_c_file(oracle_lib):
    """The oracle's systematic resampling against SimInf_systematic_resampling
    (src/misc/SimInf_particle_filter.c:33-67) compiled unmodified: random
    weight vectors of several shapes (flat, heavy-tailed, mostly zero, one
    survivor), uniforms near both ends, and the final index clamped to n
    (`j < n ? j + 1 : n`, :60) when rounding leaves u past the last sum."""
    rng = np.random.default_rng(17)
    cases = []
    for n in (1, 2, 7, 64, 1000, 4096):
        cases.append(rng.random(n))
        cases.append(np.exp(rng.normal(0, 6, n)))
        w = rng.random(n) * (rng.random(n) < 0.1)
        w[rng.integers(0, n)] = 0.5
        cases.append(w)
        w = np.zeros(n)
        w[-1] = 1.0
        cases.append(w)
        cases.append(np.full(n, 0.1))           # 0.1 sums inexactly
    checked = clamped = 0
    for w in cases:
        for unif in (rng.random(), 1e-12, 1.0 - 2 ** -53, 1.0):
            code, mine, code_r, ref, msg = _resample_both(w, unif)
            assert code == code_r == 0, msg
            assert np.array_equal(mine, ref)
            checked += 1
            clamped += int(ref[-1] == len(w))
    assert checked == 4 * len(cases) and clamped > 0


@pytest.mark.skipif(not oracle.ref_available(), reason="oracle/_ref was not built")
def test_resampling_rejects_what_the_reference_rejects(oracle_lib):
    for w in ([0.5, -0.1, 0.6], [0.0, 0.0], [1.0, np.nan], [np.inf, 1.0]):
        code, _, code_r, _, msg = _resample_both(w, 0.5)
        assert code == code_r == -1
        assert msg in ("Invalid weight detected (non-finite or < 0.0).",
                       "Non-positive sum of weights detected.")


def test_oracle_pfilter_runs_and_is_deterministic(oracle_lib):
    m, gdata, t, obs = small_case()
    c1, ll1, ess1, a1 = oracle.pfilter(m, 64, t, obs, 1, 0.8, seed=5, gdata=gdata)
    c2, ll2, ess2, a2 = oracle.pfilter(m, 64, t, obs, 1, 0.8, seed=5, gdata=gdata, threads=4)
    assert c1 == 0 and c2 == 0
    assert np.isfinite(ll1) and ll1 == ll2
    assert np.array_equal(ess1, ess2) and np.array_equal(a1, a2)
    assert ((ess1 >= 1.0 - 1e-9) & (ess1 <= 64 + 1e-9)).all()
    assert a1.min() >= 1 and a1.max() <= 64
    # ancestors are non-decreasing: systematic resampling walks the cumsum
    assert (np.diff(a1, axis=1) >= 0).all()


def test_oracle_pfilter_shared_gdata_and_gap_one(oracle_lib):
    """Consecutive observation days use one-point intervals (R/pfilter.R:
    187-192)."""
    m, _, _, _ = small_case()
    t = np.array([3, 4, 5, 9], dtype=np.int32)
    obs = np.ones((4, m.Nn), dtype=np.int32)
    code, ll, ess, anc = oracle.pfilter(m, 32, t, obs, 1, 0.5, seed=1)
    assert code == 0 and np.isfinite(ll)


@pytest.mark.gpu
def test_gpu_pfilter_matches_oracle(gpu, oracle_lib):
    from siminf_gb300.run import pfilter
    m, gdata, t, obs = small_case()
    code, ll, ess, anc = oracle.pfilter(m, 64, t, obs, 1, 0.8, seed=5, gdata=gdata, threads=4)
    r = pfilter(m, 64, t, obs, 1, 0.8, seed=5, gdata=gdata)
    assert code == 0
    assert r.loglik == ll
    assert np.array_equal(r.ess, ess)
    assert np.array_equal(r.ancestors, anc)


@pytest.mark.gpu
def test_gpu_pfilter_workload_small(gpu, oracle_lib):
    """The particle-filter workload generator at 2% of its size."""
    from siminf_gb300 import workloads
    from siminf_gb300.run import pfilter
    m, gdata, t, obs = workloads.sise_pfilter(nodes=50, particles=128, weeks=12)
    code, ll, ess, anc = oracle.pfilter(m, 128, t, obs, 1, 0.8, seed=11, gdata=gdata, threads=4)
    r = pfilter(m, 128, t, obs, 1, 0.8, seed=11, gdata=gdata)
    assert code == 0 and r.loglik == ll and np.array_equal(r.ancestors, anc)
