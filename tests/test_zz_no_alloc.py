"""siminf_gpu_run_solver_ssm_noalloc through the C ABI: the U and V of
siminf_gpu_run_solver_ssm on the same arguments, on calls in a row that
share the entry point's static scratch, plus its size limit and error
codes.  The file name puts it last in a session; it passes alone too."""
import ctypes as C

import numpy as np
import pytest

from siminf_gb300 import abi, native
from siminf_gb300 import model as M

pytestmark = pytest.mark.gpu


def _sir(nodes, days, seed, beta=0.16):
    rng = np.random.default_rng(seed)
    u0 = {"S": rng.poisson(150, nodes), "I": rng.poisson(4, nodes), "R": np.zeros(nodes, np.int64)}
    return M.SIR(u0, np.arange(0.0, days + 1), beta=beta, gamma=0.077)


def _sise(nodes, days, seed):
    rng = np.random.default_rng(seed)
    u0 = {"S": rng.poisson(90, nodes), "I": rng.poisson(3, nodes)}
    return M.SISe(u0, np.arange(0.0, days + 1, 2.0), phi=rng.uniform(0, 1, nodes),
                  upsilon=0.02, gamma=0.1, alpha=1.0, beta_t1=0.19, beta_t2=0.085,
                  beta_t3=0.075, beta_t4=0.185, end_t1=91, end_t2=182, end_t3=273,
                  end_t4=365, epsilon=0.000011)


def _existing(m, seed):
    h = abi.build_args(m, seed)
    code = native.lib().siminf_gpu_run_solver_ssm(C.cast(h.ref(), C.c_void_p),
                                                  native.device_model(m.name).handle)
    return code, h


def _noalloc(m, seed):
    h = abi.build_args(m, seed)
    # poison the outputs so that a column the call does not write shows up
    h.U[:] = -7
    if h.V is not None and h.V.size:
        h.V[:] = np.nan
    code = native.lib().siminf_gpu_run_solver_ssm_noalloc(
        C.cast(h.ref(), C.c_void_p), native.device_model(m.name).handle, None)
    return code, h


def _same(m, seed):
    code_e, he = _existing(m, seed)
    code_n, hn = _noalloc(m, seed)
    assert code_e == 0 and code_n == 0, native.last_status().message
    assert np.array_equal(hn.U, he.U)
    if m.Nd:
        assert np.array_equal(hn.V, he.V)


def test_noalloc_matches_solver_on_calls_in_a_row(gpu):
    a, b = _sise(300, 120, 3), _sir(120, 60, 5)
    # a larger run, then a smaller one over the scratch it left, then both again
    _same(a, 11)
    _same(b, 12)
    _same(b, 12)
    _same(a, 13)


def test_noalloc_same_bits_twice(gpu):
    m = _sir(257, 90, 8)
    c1, h1 = _noalloc(m, 99)
    c2, h2 = _noalloc(m, 99)
    assert c1 == 0 and c2 == 0
    assert np.array_equal(h1.U, h2.U)
    # every column written, and S + I + R of each node kept
    U = h1.U.reshape((m.Nc, m.Nn, len(m.tspan)), order="F")
    assert (U >= 0).all()
    assert np.array_equal(U.sum(axis=0), np.repeat(m.u0.sum(axis=0)[:, None], len(m.tspan), 1))


def test_noalloc_rejects_runs_beyond_scratch(gpu):
    m = _sir(200_000, 100, 1)        # U alone is 240 MB
    code, _ = _noalloc(m, 1)
    assert code == -35
    st = native.last_status()
    assert st.error == -35 and b"scratch" in st.message
    _same(_sir(64, 30, 2), 3)        # the next call runs normally


def _status():
    st = native.last_status()
    return st.error, st.node, st.transition, st.rate


def test_noalloc_reports_the_solver_error(gpu):
    m = _sir(50, 20, 4, beta=-0.5)   # negative rates: invalid rate at start
    code_e, _ = _existing(m, 1)
    st_e = _status()
    code_n, _ = _noalloc(m, 1)
    assert code_e == code_n == -11
    assert _status() == st_e
    _same(_sir(64, 30, 2), 3)


def test_noalloc_reports_the_last_invalid_rate_of_a_node(gpu):
    """Three invalid rates of every node at the first day's end (negative
    upsilons once phi leaves 0): both entry points report the highest
    node's last transition, the status the reference's refresh loop leaves
    behind."""
    rng = np.random.default_rng(2)
    u0 = {k: (rng.poisson(20, 30) if k.startswith("S") else np.zeros(30, np.int64))
          for k in ("S_1", "I_1", "S_2", "I_2", "S_3", "I_3")}
    m = M.SISe3(u0, np.arange(1.0, 10.0), phi=0.0, upsilon_1=-0.01, upsilon_2=-0.02,
                upsilon_3=-0.03, gamma_1=0.1, gamma_2=0.12, gamma_3=0.14, alpha=1.0,
                beta_t1=0.19, beta_t2=0.085, beta_t3=0.075, beta_t4=0.185, end_t1=91,
                end_t2=182, end_t3=273, end_t4=365, epsilon=1e-5)
    code_e, _ = _existing(m, 1)
    st_e = _status()
    code_n, _ = _noalloc(m, 1)
    st_n = _status()
    assert code_e == code_n == -11
    assert st_n == st_e
    assert st_e[1] == m.Nn - 1 and st_e[2] == 4
    _same(_sir(64, 30, 2), 3)


def test_noalloc_refuses_what_it_does_not_run(gpu):
    m = _sir(10, 5, 1)
    m2 = M.SIR(m.u0, m.tspan, beta=0.16, gamma=0.077,
               events=M.make_events(event=[1], time=[2], node=[1], dest=[0], n=[1],
                                    proportion=[0.0], select=[1], shift=[0]))
    code, _ = _noalloc(m2, 1)
    assert code == -9
