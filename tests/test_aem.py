"""The all-events method (aem, src/solvers/SimInf_solver_aem.c) on the GPU
against the oracle's restatement, bit for bit, through the same C ABI
entry points (args.solver = 1).  The oracle's aem is itself checked in
distribution against the reference's unmodified aem (test_ks.py)."""
import ctypes as C

import numpy as np
import pytest

from helpers import parity_cases
from siminf_gb300 import abi

ONE_REPLICATE = [c for c in parity_cases() if c[1].replicates == 1]


def run_oracle_aem(m, seed=42):
    from oracle import oracle
    h = abi.build_args(m, seed, solver=1)
    code, res = oracle.run(h, m.name, 4)
    return code, h, res


def test_oracle_aem_rejects_replicates(oracle_lib):
    m = dict(parity_cases())["seir_events_rep5"]
    code, _, _ = run_oracle_aem(m)
    assert code == -19


def test_oracle_aem_conserves_population(oracle_lib):
    """SIR without events: every column of every node holds its initial
    population, and transitions fired."""
    m = dict(parity_cases())["sir_mparse_1000x150"]
    code, h, res = run_oracle_aem(m)
    assert code == 0 and res.transitions > 0
    U = h.U.reshape((m.Nc, m.Nn, -1), order="F")          # [compartment, node, column]
    assert (U.sum(axis=0) == m.u0.sum(axis=0)[:, None]).all()


@pytest.mark.gpu
@pytest.mark.parametrize("heavy_rate", [0, 1, -1])
@pytest.mark.parametrize("label,m", ONE_REPLICATE, ids=[c[0] for c in ONE_REPLICATE])
def test_gpu_aem_matches_oracle(gpu, label, m, heavy_rate):
    """heavy_rate 1: every node with a rate sum >= 1 goes to the heavy
    warps first; -1: no heavy part; 0: the default threshold."""
    from siminf_gb300 import native
    code_o, ho, res = run_oracle_aem(m)
    h = abi.build_args(m, 42, solver=1)
    opt = abi.Options(heavy_rate=heavy_rate)
    code = native.lib().siminf_gpu_run_solver_ex(C.cast(h.ref(), C.c_void_p),
                                                 native.device_model(m.name).handle,
                                                 C.byref(opt))
    assert code == code_o == 0, label
    assert np.array_equal(h.U, ho.U), label
    if m.Nd:
        assert np.array_equal(h.V, ho.V), label
    assert native.last_stats().transitions == res.transitions


@pytest.mark.gpu
def test_gpu_aem_rejects_replicates(gpu):
    from siminf_gb300 import native
    m = dict(parity_cases())["seir_events_rep5"]
    h = abi.build_args(m, 42, solver=1)
    code = native.lib().siminf_gpu_run_solver_mssm(C.cast(h.ref(), C.c_void_p),
                                                   native.device_model(m.name).handle)
    assert code == -19
    assert b"aem" in native.last_status().message


@pytest.mark.gpu
def test_gpu_aem_plan_reruns(gpu):
    """A resident aem plan run three times (the later runs from one CUDA
    graph) gives the oracle's trajectories every time."""
    from siminf_gb300 import native
    m = dict(parity_cases())["seir_events_300x120"]
    _, ho, _ = run_oracle_aem(m)
    h = abi.build_args(m, 42, solver=1)
    p = native.Plan(h, m.name)
    for _ in range(3):
        h.U[:] = -1
        p.run()
        p.download()
        assert np.array_equal(h.U, ho.U)
    p.close()


@pytest.mark.gpu
def test_gpu_aem_error_codes(gpu):
    """The error cases of the ssm tests that run one replicate, under aem:
    the code the oracle's aem returns."""
    from oracle import oracle
    from siminf_gb300 import native
    from test_oracle import error_cases
    n = 0
    for label, m, _ in error_cases():
        if m.replicates != 1:
            continue
        ho = abi.build_args(m, 42, solver=1)
        want, _ = oracle.run(ho, m.name, 1)
        h = abi.build_args(m, 42, solver=1)
        got = native.lib().siminf_gpu_run_solver_ssm(C.cast(h.ref(), C.c_void_p),
                                                     native.device_model(m.name).handle)
        assert got == want, label
        n += 1
    assert n > 0
