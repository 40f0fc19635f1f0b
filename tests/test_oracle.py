"""The oracle (oracle/siminf_oracle.c) against the reference's own solver
sources compiled unmodified (oracle/_ref), and against the RNG-free golden
vectors of the reference's R tests (tests/golden/*.json)."""
import numpy as np
import pytest

from siminf_gb300 import model as M
from helpers import (U_matrix, golden, model_from_fixture, parity_cases, run_oracle, run_ref,
                     sparse_pattern)
from oracle import oracle

needs_ref = pytest.mark.skipif(not oracle.ref_available(),
                               reason="reference sources were not available to build oracle/_ref")


@needs_ref
@pytest.mark.parametrize("label,m", parity_cases(), ids=[c[0] for c in parity_cases()])
@pytest.mark.parametrize("threads", [1, 3])
def test_oracle_matches_reference(oracle_lib, label, m, threads):
    code_o, res, ho = run_oracle(m, threads=threads)
    code_r, hr = run_ref(m, threads=threads)
    assert code_o == code_r == 0
    assert np.array_equal(ho.U, hr.U)
    assert np.array_equal(ho.V, hr.V)
    assert res.transitions > 0 or label.startswith("sis_shift")


@needs_ref
def test_oracle_matches_reference_on_balanced_headline_sample(oracle_lib):
    """The benchmark workload's generator at 5% scale (50,000 nodes, 25,000
    transfers a day) for 120 days with transfers of one individual: the
    variant the reference runs without capping.  The oracle, with every
    host thread, equals the reference's unmodified solver bit for bit."""
    import os
    from siminf_gb300 import abi, workloads
    m = workloads.seir_events(nodes=50_000, days=120, transfers=25_000, transfer_n=1)
    threads = os.cpu_count() or 1
    ho = abi.build_args(m, 42)
    code_o, res = oracle.run(ho, m.name, threads)
    hr = abi.build_args(m, 42)
    code_r = oracle.run_ref(hr, m.name, threads)
    assert code_o == code_r == 0
    assert np.array_equal(ho.U, hr.U)
    assert res.transitions > 100_000 and res.e2_events == 120 * 25_000


@needs_ref
@pytest.mark.parametrize("name", ["sir_mparse_rep7", "seir_events_rep5"])
def test_oracle_crn_matches_reference(oracle_lib, name):
    """crn = 1 on a replicated model runs the reference's mssm_crn solver
    (src/solvers/SimInf_solver_mssm_crn.c): the SSA draws come from a
    generator per (replicate, node), the events from the node's stream.
    The oracle equals it bit for bit, and differs from crn = 0."""
    from siminf_gb300 import abi
    m = dict(parity_cases())[name]
    out = {}
    for crn in (0, 1):
        ho = abi.build_args(m, 42)
        ho.args.crn = crn
        code_o, res = oracle.run(ho, m.name, 3)
        hr = abi.build_args(m, 42)
        hr.args.crn = crn
        code_r = oracle.run_ref(hr, m.name, 3)
        assert code_o == code_r == 0
        assert np.array_equal(ho.U, hr.U)
        out[crn] = ho.U.copy()
    assert not np.array_equal(out[0], out[1])


def test_oracle_thread_count_invariance(oracle_lib):
    for label, m in parity_cases()[:4]:
        _, _, h1 = run_oracle(m, threads=1)
        _, _, h8 = run_oracle(m, threads=8)
        assert np.array_equal(h1.U, h8.U), label


def test_golden_sise_phi(oracle_lib):
    fx = golden("sise_phi.json")
    m = model_from_fixture(fx)
    code, res, h = run_oracle(m)
    assert code == 0 and res.transitions == 0
    phi = h.V[:len(m.tspan)]
    assert np.all(np.abs(phi - np.array(fx["phi_expected"])) < fx["tol"])


def test_golden_sir_zero_rates(oracle_lib):
    fx = golden("sir_zero_rates.json")
    m = model_from_fixture(fx)
    code, _, h = run_oracle(m)
    assert code == 0
    U = U_matrix(m, h)
    shape = tuple(fx["dim"])
    for c, key in enumerate(("S_expected", "I_expected", "R_expected")):
        want = np.array(fx[key]).reshape(shape, order="F")
        assert np.array_equal(U[c::3, :], want), key


def test_golden_sise3_transfer_one(oracle_lib):
    fx = golden("sise3_transfer_one.json")
    m = model_from_fixture(fx)
    code, _, h = run_oracle(m)
    assert code == 0
    want = np.array(fx["U_expected"]).reshape(tuple(fx["dim"]), order="F")
    assert np.array_equal(U_matrix(m, h), want)


def test_golden_sise3_transfer_three(oracle_lib):
    fx = golden("sise3_transfer_three.json")
    m = model_from_fixture(fx)
    code, _, h = run_oracle(m)
    assert code == 0
    U = U_matrix(m, h)
    s_node1 = U[0, :] + U[2, :] + U[4, :]
    assert np.array_equal(s_node1, np.array(fx["S_sum_node1_expected"]))


def _punchcard_patterns(fx, m):
    tlen = len(m.tspan)
    ncol = m.replicates * tlen
    U_sp = sparse_pattern(fx["U_i"], fx["U_j"], m.Nn * m.Nc, ncol)
    V_sp = sparse_pattern(fx["V_i"], fx["V_j"], m.Nn * m.Nd, ncol)
    return U_sp, V_sp


def test_golden_punchcard_replicates(oracle_lib):
    fx = golden("sise_punchcard_rep.json")
    m = model_from_fixture(fx)
    U_sp, V_sp = _punchcard_patterns(fx, m)
    code, _, h = run_oracle(m, U_sparse=U_sp, V_sparse=V_sp)
    assert code == 0
    assert np.array_equal(h.prU, np.array(fx["U_x_expected"], dtype=float))
    assert np.all(np.abs(h.prV - np.array(fx["V_x_expected"])) < fx["tol"])


# Error paths of the reference's tests (codes of inst/include/SimInf.h:66-89).
def error_cases():
    cases = []
    # tests/SIR.R:483-490: gamma < 0 -> invalid rate at initialisation
    cases.append(("init_invalid_rate", M.SIR({"S": [99, 99], "I": [1, 1], "R": [0, 0]},
                                             np.arange(1, 101), 0.16, -0.077), -11))
    # tests/SIR.R:552-567: S column entry -1000 -> negative state
    m = M.SIR({"S": [99], "I": [1], "R": [0]}, np.arange(1, 101), 0.16, 0.0)
    m.S = m.S.copy()
    m.S[0, 0] = -1000
    cases.append(("negative_state", m, -1))
    # tests/SEIR.R:494-502: epsilon < 0 -> invalid rate during the run
    cases.append(("seir_invalid_rate", M.SEIR({"S": [100, 100], "E": [0, 0], "I": [10, 10],
                                               "R": [0, 0]}, np.arange(1, 101), 0.16, -0.3,
                                              0.077), -11))
    # tests/sample_select.R:32-87: transfer of 2 from a node holding 1
    ev = M.make_events(3, 1, 2, 1, 2, 1.0, 4, 0)
    cases.append(("unable_to_sample", M.SISe3(
        {"S_1": [0, 1], "I_1": [0, 0], "S_2": [0, 0], "I_2": [0, 0], "S_3": [0, 0],
         "I_3": [0, 0]}, np.arange(0, 11), phi=[0.0, 0.0], upsilon_1=0, upsilon_2=0,
        upsilon_3=0, gamma_1=1, gamma_2=1, gamma_3=1, alpha=0, beta_t1=1, beta_t2=1,
        beta_t3=1, beta_t4=1, end_t1=91, end_t2=182, end_t3=273, end_t4=365, epsilon=0,
        events=ev), -8))

    # tests/sample_select.R:858-941: select column with no state, bad proportion, N, shift
    def sir1(event=0, n=1, proportion=0.0, select=4, shift=0, E=None, N=None):
        mm = M.SIR({"S": [1], "I": [1], "R": [1]}, [1], 0.0, 0.0,
                   events=M.make_events(event, 1, 1, 0, n, proportion, select, shift))
        if E is not None:
            mm.E = np.asarray(E, dtype=float)
        if N is not None:
            mm.N = np.asarray(N, dtype=np.int32)
        return mm

    E_no4 = [[1, 0, 0, 0], [0, 1, 0, 0], [0, 0, 1, 0]]
    cases.append(("exit_empty_select", sir1(E=E_no4), -8))
    cases.append(("enter_empty_select", sir1(event=1, E=E_no4), -8))
    cases.append(("enter_negative_n", sir1(event=1, n=-1, E=E_no4), -8))
    cases.append(("enter_proportion_low", sir1(event=1, n=0, proportion=-1.0), -18))
    cases.append(("enter_proportion_high", sir1(event=1, n=0, proportion=1.1), -18))
    cases.append(("enter_shift_without_N", sir1(event=1, n=1, select=1, shift=1), -15))
    cases.append(("enter_shift_oob_high", sir1(event=1, n=1, select=1, shift=1,
                                               N=[[3], [0], [0]]), -17))
    cases.append(("enter_shift_oob_low", sir1(event=1, n=1, select=1, shift=1,
                                              N=[[-1], [0], [0]]), -17))
    # node / dest out of bounds and an internal transfer without shift
    cases.append(("node_oob", M.SIR({"S": [5], "I": [0], "R": [0]}, [1, 2], 0.0, 0.0,
                                    events=M.make_events(0, 1, 2, 0, 1, 0.0, 1, 0)), -14))
    cases.append(("dest_oob", M.SIR({"S": [5], "I": [0], "R": [0]}, [1, 2], 0.0, 0.0,
                                    events=M.make_events(3, 1, 1, 7, 1, 0.0, 1, 0)), -13))
    mm = M.SIR({"S": [5], "I": [0], "R": [0]}, [1, 2], 0.0, 0.0,
               events=M.make_events(2, 1, 1, 0, 1, 0.0, 1, 0))
    mm.N = np.array([[1], [0], [0]], dtype=np.int32)
    cases.append(("internal_without_shift", mm, -16))
    return cases


@pytest.mark.parametrize("label,m,code", error_cases(), ids=[c[0] for c in error_cases()])
def test_error_codes_oracle(oracle_lib, label, m, code):
    got, _, _ = run_oracle(m)
    assert got == code


@needs_ref
@pytest.mark.parametrize("label,m,code", error_cases(), ids=[c[0] for c in error_cases()])
def test_error_codes_reference(oracle_lib, label, m, code):
    got, _ = run_ref(m)
    assert got == code


def test_deterministic_shift_enter(oracle_lib):
    """tests/sample_select.R:937-941: enter of 1 into S shifted to I."""
    m = M.SIR({"S": [1], "I": [1], "R": [1]}, [1], 0.0, 0.0,
              events=M.make_events(1, 1, 1, 0, 1, 0.0, 1, 1))
    m.N = np.array([[1], [0], [0]], dtype=np.int32)
    code, _, h = run_oracle(m)
    assert code == 0
    assert h.U.tolist() == [1, 2, 1]
