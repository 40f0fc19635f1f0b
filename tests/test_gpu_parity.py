"""GPU trajectories against the oracle, bit for bit, through the C ABI
(siminf_gpu_run_solver_ssm / _mssm), plus the golden vectors of the
reference's R tests and the reference's error codes."""
import numpy as np
import pytest

from helpers import (U_matrix, golden, model_from_fixture, parity_cases, run_gpu, run_oracle,
                     sparse_pattern)
from test_oracle import error_cases

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("label,m", parity_cases(), ids=[c[0] for c in parity_cases()])
def test_gpu_matches_oracle(gpu, oracle_lib, label, m):
    code_o, res, ho = run_oracle(m, threads=4)
    code_g, hg, st = run_gpu(m)
    assert code_o == 0 and code_g == 0
    assert np.array_equal(hg.U, ho.U), label
    assert np.array_equal(hg.V, ho.V), label
    assert st.transitions == res.transitions
    assert st.e1_events == res.e1_events and st.e2_events == res.e2_events


@pytest.mark.parametrize("seed", [1, 2, 3, 1234567, 2 ** 40 + 5])
def test_gpu_seeds(gpu, oracle_lib, seed):
    m = dict(parity_cases())["seir_events_300x120"]     # SEIR with all event kinds
    _, _, ho = run_oracle(m, seed=seed, threads=4)
    code, hg, _ = run_gpu(m, seed=seed)
    assert code == 0 and np.array_equal(hg.U, ho.U)


def test_gpu_golden_sise_phi(gpu):
    fx = golden("sise_phi.json")
    m = model_from_fixture(fx)
    code, h, st = run_gpu(m)
    assert code == 0 and st.transitions == 0
    assert np.all(np.abs(h.V[:len(m.tspan)] - np.array(fx["phi_expected"])) < fx["tol"])


def test_gpu_golden_sir_zero_rates(gpu):
    fx = golden("sir_zero_rates.json")
    m = model_from_fixture(fx)
    code, h, _ = run_gpu(m)
    assert code == 0
    U = U_matrix(m, h)
    for c, key in enumerate(("S_expected", "I_expected", "R_expected")):
        assert np.array_equal(U[c::3, :], np.array(fx[key]).reshape(tuple(fx["dim"]), order="F"))


def test_gpu_golden_sise3_transfers(gpu):
    fx = golden("sise3_transfer_one.json")
    m = model_from_fixture(fx)
    code, h, _ = run_gpu(m)
    assert code == 0
    assert np.array_equal(U_matrix(m, h),
                          np.array(fx["U_expected"]).reshape(tuple(fx["dim"]), order="F"))
    fx = golden("sise3_transfer_three.json")
    m = model_from_fixture(fx)
    code, h, _ = run_gpu(m)
    U = U_matrix(m, h)
    assert code == 0
    assert np.array_equal(U[0] + U[2] + U[4], np.array(fx["S_sum_node1_expected"]))


def test_gpu_golden_punchcard_replicates(gpu):
    fx = golden("sise_punchcard_rep.json")
    m = model_from_fixture(fx)
    ncol = m.replicates * len(m.tspan)
    U_sp = sparse_pattern(fx["U_i"], fx["U_j"], m.Nn * m.Nc, ncol)
    V_sp = sparse_pattern(fx["V_i"], fx["V_j"], m.Nn * m.Nd, ncol)
    code, h, _ = run_gpu(m, U_sparse=U_sp, V_sparse=V_sp)
    assert code == 0
    assert np.array_equal(h.prU, np.array(fx["U_x_expected"], dtype=float))
    assert np.all(np.abs(h.prV - np.array(fx["V_x_expected"])) < fx["tol"])


def test_gpu_sparse_matches_dense(gpu, oracle_lib):
    label, m = parity_cases()[4]           # SISe with V
    rng = np.random.default_rng(3)
    nrow_u, nrow_v, ncol = m.Nn * m.Nc, m.Nn * m.Nd, len(m.tspan)
    mask_u = rng.random((nrow_u, ncol)) < 0.1
    mask_v = rng.random((nrow_v, ncol)) < 0.1
    iu, ju = np.nonzero(mask_u)
    iv, jv = np.nonzero(mask_v)
    U_sp = sparse_pattern(iu + 1, ju + 1, nrow_u, ncol)
    V_sp = sparse_pattern(iv + 1, jv + 1, nrow_v, ncol)
    code, hs, _ = run_gpu(m, U_sparse=U_sp, V_sparse=V_sp)
    _, _, ho = run_oracle(m, U_sparse=U_sp, V_sparse=V_sp)
    code_d, hd, _ = run_gpu(m)
    assert code == 0 and code_d == 0
    assert np.array_equal(hs.prU, ho.prU) and np.array_equal(hs.prV, ho.prV)
    Ud = U_matrix(m, hd)
    ir, jc = U_sp
    for j in range(ncol):
        rows = ir[jc[j]:jc[j + 1]]
        assert np.array_equal(hs.prU[jc[j]:jc[j + 1]], Ud[rows, j].astype(float))


@pytest.mark.parametrize("label,m,code", error_cases(), ids=[c[0] for c in error_cases()])
def test_gpu_error_codes(gpu, label, m, code):
    got, _, _ = run_gpu(m)
    assert got == code


@pytest.mark.parametrize("label,m,code", error_cases(), ids=[c[0] for c in error_cases()])
def test_gpu_error_codes_two_pass(gpu, label, m, code):
    """The reference's error codes when quiet node-days finish in the first
    pass of a two-pass day."""
    import ctypes as C
    from siminf_gb300 import abi, native
    h = abi.build_args(m, 42)
    opt = abi.Options(two_pass=1)
    got = native.lib().siminf_gpu_run_solver_ex(C.cast(h.ref(), C.c_void_p),
                                                native.device_model(m.name).handle,
                                                C.byref(opt))
    assert got == code


def test_gpu_unsorted_events_rejected(gpu):
    from siminf_gb300 import model as M
    m = M.SIR({"S": [5, 5], "I": [0, 0], "R": [0, 0]}, [1, 2, 3], 0.0, 0.0,
              events=M.make_events([0, 0], [2, 1], [1, 2], 0, 1, 0.0, 1, 0, sort=False))
    got, _, _ = run_gpu(m)
    assert got == -31


def test_gpu_capped_seir_workload(gpu, oracle_lib):
    """The headline workload's generator at 0.2% scale (2,000 nodes, 1,000
    transfers/day, 365 days, cap_transfers on): bit-exact with the oracle."""
    from siminf_gb300 import workloads
    from siminf_gb300.run import run
    from siminf_gb300 import abi
    from oracle import oracle
    m = workloads.seir_events(nodes=2000, days=365, transfers=1000)
    h = abi.build_args(m, 42)
    code, res = oracle.run(h, m.name, 4, cap_transfers=True)
    assert code == 0
    r = run(m, seed=42, cap_transfers=True)
    assert np.array_equal(r.U, h.U.reshape(r.U.shape, order="F"))
    assert r.stats.transitions == res.transitions
    assert r.stats.e2_events == res.e2_events
    # without the cap the reference semantics stop the run
    with pytest.raises(Exception) as e:
        run(m, seed=42)
    assert getattr(e.value, "code", None) == -8


def test_gpu_conservation_full_scale_properties(gpu):
    """At 10% of the headline size: population changes only by the enter and
    exit events (transfers conserve it), and no state is negative."""
    from siminf_gb300 import workloads
    from siminf_gb300.run import run
    m = workloads.seir_events(nodes=100_000, days=60, transfers=50_000)
    r = run(m, seed=7, cap_transfers=True)
    U = r.U
    assert (U >= 0).all()
    tot = U.reshape(m.Nn, m.Nc, -1).sum(axis=(0, 1)).astype(np.int64)
    ev = m.events
    d_enter = np.bincount(ev["time"][ev["event"] == 1], minlength=62)[1:61]
    # exits may be capped at empty nodes, so the population can only drop by
    # at most the number of exit events of a day
    d_exit = np.bincount(ev["time"][ev["event"] == 0], minlength=62)[1:61]
    start = m.u0.sum()
    for k in range(60):
        prev = start if k == 0 else tot[k - 1]
        change = tot[k] - prev
        assert change <= d_enter[k]
        assert change >= d_enter[k] - d_exit[k]


@pytest.mark.parametrize("two_pass", [-1, 1])
@pytest.mark.parametrize("heavy_rate", [1, -1])
@pytest.mark.parametrize("label,m", parity_cases(), ids=[c[0] for c in parity_cases()])
def test_gpu_heavy_queue_matches_oracle(gpu, oracle_lib, label, m, heavy_rate, two_pass):
    """heavy_rate = 1 queues every node with a rate sum >= 1 for the heavy
    warps (32 nodes to a warp, first in the day); -1 turns the queue off.
    two_pass = 1 finishes the quiet node-days in a first pass and queues
    only the others; -1 queues every node.  All stay bit-exact."""
    import ctypes as C
    from siminf_gb300 import abi, native
    _, _, ho = run_oracle(m, threads=4)
    h = abi.build_args(m, 42)
    opt = abi.Options(cap_transfers=0, heavy_rate=heavy_rate, two_pass=two_pass)
    code = native.lib().siminf_gpu_run_solver_ex(C.cast(h.ref(), C.c_void_p),
                                                 native.device_model(m.name).handle,
                                                 C.byref(opt))
    assert code == 0
    assert np.array_equal(h.U, ho.U), label
    assert np.array_equal(h.V, ho.V), label


@pytest.mark.parametrize("name", ["sir_mparse_rep7", "seir_events_rep5"])
@pytest.mark.parametrize("heavy_rate,two_pass", [(-1, -1), (1, 1), (1, -1)])
def test_gpu_crn_matches_oracle(gpu, oracle_lib, name, heavy_rate, two_pass):
    """crn = 1 on a replicated model (SimInf_run_solver_mssm_crn,
    src/solvers/SimInf_solver_mssm_crn.c:185,196): the SSA draws from a
    stream per (replicate, node) of its own, the events from the node's
    stream.  Bit-exact with the oracle, which equals the reference's
    mssm_crn compiled unmodified, on the whole-horizon kernel (no external
    transfers) and the work queue in every layout; different from crn = 0."""
    import ctypes as C
    from oracle import oracle
    from siminf_gb300 import abi, native
    m = dict(parity_cases())[name]
    ho = abi.build_args(m, 42)
    ho.args.crn = 1
    assert oracle.run(ho, m.name, 4)[0] == 0
    h = abi.build_args(m, 42)
    h.args.crn = 1
    opt = abi.Options(heavy_rate=heavy_rate, two_pass=two_pass)
    code = native.lib().siminf_gpu_run_solver_ex(C.cast(h.ref(), C.c_void_p),
                                                 native.device_model(m.name).handle,
                                                 C.byref(opt))
    assert code == 0
    assert np.array_equal(h.U, ho.U)
    h0 = abi.build_args(m, 42)
    assert native.lib().siminf_gpu_run_solver_mssm(C.cast(h0.ref(), C.c_void_p),
                                                   native.device_model(m.name).handle) == 0
    assert not np.array_equal(h0.U, h.U)


def test_gpu_autotune_keeps_results(gpu):
    """siminf_gpu_plan_tune searches its candidate layouts -- heavy
    threshold x one- or two-pass days, then the SSA kernel's other register
    budget, then the wavefront block -- keeps the fastest, caches it for
    plans of the same model and size class, and the tuned plan's
    trajectories are the untuned plan's."""
    from siminf_gb300 import abi, native
    label, m = [c for c in parity_cases() if c[0] == "seir_events_300x120"][0]
    h1 = abi.build_args(m, 42)
    p1 = native.Plan(h1, m.name)
    p1.run()
    p1.download()
    h2 = abi.build_args(m, 42)
    p2 = native.Plan(h2, m.name)
    r = p2.tune(probe_days=-10)             # a new search
    # 8 queue layouts, the other register budget, 8 heavy lanes (when the
    # best layout so far has a heavy part), two wavefront blocks
    n = r.n_candidates
    assert n in (11, 12) and 0 <= r.chosen < n and r.probe_days == 10
    assert not r.cached
    assert list(r.heavy_rate[:8]) == [0.0, 2.0, 8.0, 32.0] * 2
    assert list(r.two_pass[:8]) == [0] * 4 + [1] * 4
    assert r.ssa_variant[8] == 1 and list(r.wave_block[n - 2:n]) == [128, 512]
    if n == 12:
        assert r.heavy_lanes[9] == 8 and r.heavy_rate[9] > 0
    assert all(r.heavy_lanes[k] == 0 for k in range(9))
    p2.run()
    p2.download()
    assert np.array_equal(h1.U, h2.U)
    # a plan of the same class takes the cached choice without probing
    h3 = abi.build_args(m, 42)
    p3 = native.Plan(h3, m.name)
    r3 = p3.tune(probe_days=10)
    assert r3.cached and r3.chosen == r.chosen
    p3.run()
    p3.download()
    assert np.array_equal(h1.U, h3.U)
    # every candidate layout gives the same trajectory
    for k in range(r.n_candidates):
        h4 = abi.build_args(m, 42)
        p4 = native.Plan(h4, m.name, heavy_rate=int(r.heavy_rate[k]) or -1,
                         two_pass=1 if r.two_pass[k] else -1, ssa_variant=r.ssa_variant[k],
                         wave_block=r.wave_block[k], heavy_lanes=r.heavy_lanes[k])
        p4.run()
        p4.download()
        assert np.array_equal(h1.U, h4.U), k
        p4.close()
    for p in (p1, p2, p3):
        p.close()


@pytest.mark.parametrize("name", ["seir_events_rep5", "sise_200x199"])
def test_gpu_plan_rerun_graph(gpu, oracle_lib, name):
    """A plan run again unchanged replays its run from a CUDA graph; every
    run gives the oracle's trajectories."""
    from siminf_gb300 import abi, native
    m = dict(parity_cases())[name]
    _, _, ho = run_oracle(m, threads=4)
    h = abi.build_args(m, 42)
    p = native.Plan(h, m.name)
    for _ in range(3):
        h.U[:] = -1
        p.run()
        p.download()
        assert np.array_equal(h.U, ho.U)
        if m.Nd:
            assert np.array_equal(h.V, ho.V)
    p.close()


def _pin_outputs(h, torch):
    """Move the holder's output arrays into pinned host memory."""
    import ctypes as C
    for name, ctype in (("U", C.c_int), ("V", C.c_double), ("prU", C.c_double),
                        ("prV", C.c_double)):
        arr = getattr(h, name)
        if arr is None:
            continue
        t = torch.from_numpy(arr).pin_memory()
        h.keep.append(t)
        pinned = t.numpy()
        setattr(h, name, pinned)
        setattr(h.args, name, pinned.ctypes.data_as(C.POINTER(ctype)))


@pytest.mark.parametrize("name", ["seir_events_300x120", "seir_events_rep5", "sise3_events"])
def test_gpu_pinned_outputs_streamed_back(gpu, oracle_lib, name):
    """With pinned U/V a run with external transfers copies each chunk of
    finished columns back while later days run (a third stream); the
    arrays hold the oracle's trajectories, for every replicate."""
    import ctypes as C
    from siminf_gb300 import abi, native
    torch = pytest.importorskip("torch")
    m = dict(parity_cases())[name]
    _, _, ho = run_oracle(m, threads=4)
    for _ in range(2):                      # the second run reuses the kept staging buffer
        h = abi.build_args(m, 42)
        _pin_outputs(h, torch)
        h.U[:] = -1
        code = native.lib().siminf_gpu_run_solver_ex(C.cast(h.ref(), C.c_void_p),
                                                     native.device_model(m.name).handle, None)
        assert code == 0
        assert np.array_equal(h.U, ho.U), name
        if m.Nd:
            assert np.array_equal(h.V, ho.V), name
    native.lib().siminf_gpu_release_cached()


def test_gpu_pinned_sparse_outputs_streamed_back(gpu, oracle_lib):
    """The same with sparse U over a random pattern of 5 replicates."""
    import ctypes as C
    from siminf_gb300 import abi, native
    torch = pytest.importorskip("torch")
    m = dict(parity_cases())["seir_events_rep5"]
    rng = np.random.default_rng(11)
    nrow, ncol = m.Nn * m.Nc, m.replicates * len(m.tspan)
    iu, ju = np.nonzero(rng.random((nrow, ncol)) < 0.05)
    U_sp = sparse_pattern(iu + 1, ju + 1, nrow, ncol)
    _, _, ho = run_oracle(m, U_sparse=U_sp)
    h = abi.build_args(m, 42, U_sparse=U_sp)
    _pin_outputs(h, torch)
    h.prU[:] = -1
    code = native.lib().siminf_gpu_run_solver_ex(C.cast(h.ref(), C.c_void_p),
                                                 native.device_model(m.name).handle, None)
    assert code == 0
    assert np.array_equal(h.prU, ho.prU)


def test_gpu_two_pass_and_reductions_at_scale(gpu, monkeypatch):
    """At 10% of the headline size, 4 replicates: two-pass days give the
    trajectories of one-pass days, and the device prevalence and trajectory
    of the resident U equal numpy's on the downloaded U."""
    from oracle import trajectory as ref
    from siminf_gb300 import abi, native, workloads
    from siminf_gb300.trajectory import prevalence, trajectory
    m = workloads.seir_events(nodes=100_000, days=60, transfers=50_000).replicate(4)
    out = []
    for tp in ("-1", "1"):
        monkeypatch.setenv("SIMINF_TWO_PASS", tp)
        h = abi.build_args(m, 11)
        p = native.Plan(h, m.name, cap_transfers=True)
        p.run()
        p.download()
        out.append(h.U.copy())
        if tp == "1":
            ncol = m.replicates * len(m.tspan)
            for level in (1, 2):
                got = prevalence(p, "I ~ . | S > 250", level=level)
                want = ref.prevalence(h.U, m.Nn, m.Nc, ncol, 0b0100, 0b1111, level,
                                      lambda S, E, I, R: S > 250, None, ["S", "E", "I", "R"])
                assert np.array_equal(got, want)
            tr = trajectory(p, ["E"])
            assert np.array_equal(tr["E"], ref.trajectory(h.U, m.Nn, m.Nc, ncol, [2])[0])
        p.close()
    assert np.array_equal(out[0], out[1])


def test_gpu_day_max_matches_oracle(gpu, oracle_lib):
    """The per-day busiest node's transition count (the run's critical
    path), recorded on the GPU, equals the oracle's count of the same run."""
    from oracle import oracle
    from siminf_gb300 import abi, native
    m = dict(parity_cases())["seir_events_300x120"]
    h = abi.build_args(m, 42)
    p = native.Plan(h, m.name)
    got = p.day_max()
    p.close()
    want = np.zeros(len(got), dtype=np.uint64)
    oracle.lib().oracle_set_day_max(want.ctypes.data)
    try:
        code, _ = oracle.run(abi.build_args(m, 42), m.name, 2)
    finally:
        oracle.lib().oracle_set_day_max(None)
    assert code == 0
    assert np.array_equal(got.astype(np.uint64), want)
    assert want.sum() > 0
