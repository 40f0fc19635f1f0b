"""The GPU path at the sizes only the benchmark reaches, bit for bit against
the oracle (src/solvers/SimInf_solver_ssm.c:144-373 restated, which equals
the reference's solver compiled unmodified), plus the bound on one node's
transitions per unit of time.

The headline case is the whole benchmark workload: 10^6 SEIR nodes x 365
days with 1.83e8 scheduled events, transfers capped at the source's size.
It takes the paths smaller cases never do: two-pass days, more heavy nodes
than a heavy list holds, the pinned staging ring wrapping many times, 64-bit
offsets into the external-transfer records, the whole-run graph replay and
the U columns copied back during the run."""
import ctypes as C
import os

import numpy as np
import pytest

from helpers import pin_inputs_outputs, run_oracle
from siminf_gb300 import abi, native, workloads
from siminf_gb300 import model as M

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def headline(oracle_lib):
    """The benchmark workload and the oracle's run of it on every host core."""
    from oracle import oracle
    m = workloads.seir_events()
    h = abi.build_args(m, 42)
    code, res = oracle.run(h, m.name, os.cpu_count() or 1, cap_transfers=True)
    assert code == 0
    return m, h, res


def test_gpu_headline_end_to_end_bit_exact(gpu, headline):
    """siminf_gpu_run_solver_ex with inputs and U in pinned host memory, as
    the end-to-end benchmark calls it: waves planned into the staging ring
    beside the GPU, U copied back during the run."""
    torch = pytest.importorskip("torch")
    m, ho, res = headline
    h = abi.build_args(m, 42)
    pin_inputs_outputs(h, m, torch)
    h.U[:] = -1
    opt = abi.Options(cap_transfers=1)
    for _ in range(2):              # the second run reuses the kept staging ring
        code = native.lib().siminf_gpu_run_solver_ex(C.cast(h.ref(), C.c_void_p),
                                                     native.device_model(m.name).handle,
                                                     C.byref(opt))
        assert code == 0, native.last_status().message
        st = native.last_stats()
        assert np.array_equal(h.U, ho.U)
        assert st.transitions == res.transitions
        assert st.e1_events == res.e1_events and st.e2_events == res.e2_events
    native.lib().siminf_gpu_release_cached()


@pytest.mark.parametrize("heavy_rate,two_pass", [(32, 1), (1, -1)])
def test_gpu_headline_resident_plan_bit_exact(gpu, headline, heavy_rate, two_pass):
    """The resident plan of the benchmark's `value`, in the layout the
    autotuner picks at this size (two-pass days, heavy threshold 32) and
    with every node of rate sum >= 1 in the heavy lists (far more than
    the 32,768 a list holds); run twice, the second time from the
    whole-run graph."""
    m, ho, res = headline
    h = abi.build_args(m, 42)
    p = native.Plan(h, m.name, cap_transfers=True, heavy_rate=heavy_rate, two_pass=two_pass)
    for _ in range(2):
        h.U[:] = -1
        p.run()
        p.download()
        assert np.array_equal(h.U, ho.U)
        assert p.stats().transitions == res.transitions
    p.close()


def test_gpu_heavy_list_overflow_matches_oracle(gpu, oracle_lib):
    """200,000 nodes that all start heavy (I ~ Poisson(20) everywhere) with
    heavy threshold 1: each heavy class gets far more than MAX_HEAVY nodes,
    the overflow goes to the ordinary queue, and the trajectories stay the
    oracle's."""
    from oracle import oracle
    m = workloads.seir_events(nodes=200_000, days=40, transfers=50_000)
    rng = np.random.default_rng(5)
    m.u0[2, :] = rng.poisson(20, m.Nn)
    h = abi.build_args(m, 9)
    code, res = oracle.run(h, m.name, os.cpu_count() or 1, cap_transfers=True)
    assert code == 0
    for two_pass in (-1, 1):
        hg = abi.build_args(m, 9)
        p = native.Plan(hg, m.name, cap_transfers=True, heavy_rate=1, two_pass=two_pass)
        p.run()
        p.download()
        assert np.array_equal(hg.U, h.U)
        assert p.stats().transitions == res.transitions
        p.close()


def _busy_sir(events):
    """One node that fires far more than 1,000 transitions on its first day."""
    u0 = {"S": [100_000, 50], "I": [1000, 0], "R": [0, 0]}
    ev = None
    if events:
        ev = M.make_events(event=[3], time=[2], node=[2], dest=[1], n=[1], proportion=[0.0],
                           select=[1], shift=[0])
    return M.SIR(u0, np.arange(1.0, 4.0), beta=5.0, gamma=0.5, events=ev)


@pytest.mark.parametrize("events,solver", [(False, 0), (True, 0), (False, 1)],
                         ids=["horizon", "work_queue", "aem"])
def test_gpu_node_day_bound_times_out(gpu, events, solver):
    """siminf_gpu_options.max_node_day_transitions = 1000: the busy node
    stops the run with SIMINF_GPU_ERR_TIMEOUT (-33) on every kernel that
    steps nodes (whole-horizon, work queue, all-events), and the same run
    without the bound completes."""
    m = _busy_sir(events)
    for bound, want in ((1000, -33), (0, 0)):
        h = abi.build_args(m, 3, solver=solver)
        opt = abi.Options(max_node_day_transitions=bound)
        code = native.lib().siminf_gpu_run_solver_ex(C.cast(h.ref(), C.c_void_p),
                                                     native.device_model(m.name).handle,
                                                     C.byref(opt))
        assert code == want, native.last_status().message
        if want:
            st = native.last_status()
            assert st.node == 0
