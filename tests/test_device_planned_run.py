"""Streamed runs whose scheduled events are planned while the run goes:
on the device (siminf_schedule.cu; SIMINF_DEVICE_PLANNER=1, the device
planning the levels too, and =2, the levels from host threads), and on host
threads without a scan of the whole table first (SIMINF_SCAN_FREE=1, the
default for large tables): the trajectories, counts and error codes equal
those of the oracle and of host planning, for every parity case, with
pinned outputs streamed back, with E and N growing chunk by chunk, and for
a plan re-run after its first run."""
import ctypes as C

import numpy as np
import pytest

from helpers import parity_cases, run_gpu, run_oracle
from test_oracle import error_cases

pytestmark = pytest.mark.gpu


@pytest.fixture(params=["1", "2", "scan_free"], ids=["device_levels", "host_levels", "scan_free"])
def device_planner(monkeypatch, request):
    if request.param == "scan_free":
        monkeypatch.setenv("SIMINF_DEVICE_PLANNER", "0")
        monkeypatch.setenv("SIMINF_SCAN_FREE", "1")
    else:
        monkeypatch.setenv("SIMINF_DEVICE_PLANNER", request.param)
        monkeypatch.setenv("SIMINF_SCAN_FREE", "0")


CASES = [c for c in parity_cases() if len(c[1].events["event"])]


@pytest.mark.parametrize("label,m", CASES, ids=[c[0] for c in CASES])
def test_device_planned_run_matches_oracle(gpu, oracle_lib, device_planner, label, m):
    code_o, res, ho = run_oracle(m, threads=4)
    code_g, hg, st = run_gpu(m)
    assert code_o == 0 and code_g == 0
    assert np.array_equal(hg.U, ho.U), label
    assert np.array_equal(hg.V, ho.V), label
    assert st.transitions == res.transitions
    assert st.e1_events == res.e1_events and st.e2_events == res.e2_events


@pytest.mark.parametrize("label,m,code", error_cases(), ids=[c[0] for c in error_cases()])
def test_device_planned_error_codes(gpu, device_planner, label, m, code):
    got, _, _ = run_gpu(m)
    assert got == code


def test_device_planned_unsorted_rejected(gpu, device_planner):
    from siminf_gb300 import model as M
    m = M.SIR({"S": [5, 5], "I": [0, 0], "R": [0, 0]}, [1, 2, 3], 0.0, 0.0,
              events=M.make_events([0, 0], [2, 1], [1, 2], 0, 1, 0.0, 1, 0, sort=False))
    got, _, _ = run_gpu(m)
    assert got == -31


def test_device_planned_e2_before_e1_rejected(gpu, device_planner):
    """Times in order but an external transfer before an E1 event of the
    same time: the order (time, E1 before E2) is broken inside a day, which
    only the day's own check sees."""
    from siminf_gb300 import model as M
    m = M.SIR({"S": [5, 5], "I": [0, 0], "R": [0, 0]}, [1, 2, 3], 0.0, 0.0,
              events=M.make_events([3, 0], [2, 2], [1, 2], [2, 0], 1, 0.0, 1, 0, sort=False))
    got, _, _ = run_gpu(m)
    assert got == -31


def test_device_planned_capped_workload(gpu, oracle_lib, device_planner):
    """The headline generator at 0.2% scale over 365 days (46 chunks of
    days, cap_transfers on): bit-exact with the oracle."""
    from siminf_gb300 import abi, workloads
    from siminf_gb300.run import run
    from oracle import oracle
    m = workloads.seir_events(nodes=2000, days=365, transfers=1000)
    h = abi.build_args(m, 42)
    code, res = oracle.run(h, m.name, 4, cap_transfers=True)
    assert code == 0
    r = run(m, seed=42, cap_transfers=True)
    assert np.array_equal(r.U, h.U.reshape(r.U.shape, order="F"))
    assert r.stats.transitions == res.transitions
    assert r.stats.e1_events == res.e1_events and r.stats.e2_events == res.e2_events


@pytest.mark.parametrize("name", ["seir_events_300x120", "seir_events_rep5", "sise3_events"])
def test_device_planned_pinned_outputs(gpu, oracle_lib, device_planner, name):
    from siminf_gb300 import abi, native
    from test_gpu_parity import _pin_outputs
    torch = pytest.importorskip("torch")
    m = dict(parity_cases())[name]
    _, _, ho = run_oracle(m, threads=4)
    h = abi.build_args(m, 42)
    _pin_outputs(h, torch)
    h.U[:] = -1
    code = native.lib().siminf_gpu_run_solver_ex(C.cast(h.ref(), C.c_void_p),
                                                 native.device_model(m.name).handle, None)
    assert code == 0
    assert np.array_equal(h.U, ho.U), name
    if m.Nd:
        assert np.array_equal(h.V, ho.V), name


def test_device_planned_plan_reruns(gpu, oracle_lib, device_planner):
    """A plan created with the streamed option plans its events on the
    device during its first run; the runs after it read the merged per-node
    E1 lists and the kept waves (and replay the run's graph): every run
    gives the oracle's trajectory."""
    from siminf_gb300 import abi, native
    m = dict(parity_cases())["seir_events_300x120"]
    _, _, ho = run_oracle(m, threads=4)
    h = abi.build_args(m, 42)
    plan = C.c_void_p()
    dm = native.device_model(m.name)
    lib = native.lib()
    opt = abi.Options(streamed=1)
    native.check(lib.siminf_gpu_plan_create_ex(C.cast(h.ref(), C.c_void_p), dm.handle,
                                               C.byref(opt), C.byref(plan)))
    try:
        for _ in range(3):
            h.U[:] = -1
            native.check(lib.siminf_gpu_plan_run(plan, None))
            native.check(lib.siminf_gpu_plan_download(plan, C.cast(h.ref(), C.c_void_p)))
            assert np.array_equal(h.U, ho.U)
    finally:
        lib.siminf_gpu_plan_free(plan)


@pytest.mark.parametrize("name", ["seir_events_300x120", "sise3_events"])
def test_device_planned_pinned_inputs(gpu, oracle_lib, device_planner, name):
    """Inputs and outputs in pinned host memory: the transfer records are
    gathered on the device from the columns copied by DMA."""
    from helpers import pin_inputs_outputs
    from siminf_gb300 import abi, native
    torch = pytest.importorskip("torch")
    m = dict(parity_cases())[name]
    _, _, ho = run_oracle(m, threads=4)
    h = abi.build_args(m, 42)
    pin_inputs_outputs(h, m, torch)
    h.U[:] = -1
    code = native.lib().siminf_gpu_run_solver_ex(C.cast(h.ref(), C.c_void_p),
                                                 native.device_model(m.name).handle, None)
    assert code == 0
    assert np.array_equal(h.U, ho.U), name
