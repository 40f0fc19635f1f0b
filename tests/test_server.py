"""The serving loop (siminf_gpu_server_*): requests of different kinds and
sizes submitted together and run side by side give, each, the results of
the same call made alone; the admission budget only changes when they run.
Also the C layout of every argument struct against its ctypes mirror."""
import os
import subprocess
import tempfile

import numpy as np
import pytest

from helpers import parity_cases
from siminf_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STRUCTS = [("siminf_gpu_request", abi.Request), ("siminf_gpu_server_options", abi.ServerOptions),
           ("siminf_gpu_batch_job", abi.BatchJob), ("siminf_gpu_batch_options", abi.BatchOptions),
           ("siminf_gpu_pfilter_args", abi.PfilterArgs), ("siminf_gpu_options", abi.Options),
           ("siminf_gpu_stats", abi.Stats), ("siminf_gpu_solver_args", abi.SolverArgs),
           ("siminf_gpu_tune_result", abi.TuneResult),
           ("siminf_gpu_reduce_stats", abi.ReduceStats), ("siminf_gpu_pmcmc_args", abi.PmcmcArgs),
           ("siminf_gpu_prevalence_spec", abi.PrevalenceSpec)]


def test_struct_layouts_match_the_header():
    src = '#include <stdio.h>\n#include <stddef.h>\n#include "siminf_gb300.h"\nint main(void){\n'
    for name, cls in STRUCTS:
        src += '  printf("%%zu\\n", sizeof(%s));\n' % name
        for f in cls._fields_:
            src += '  printf("%%zu\\n", offsetof(%s, %s));\n' % (name, f[0])
    src += "  return 0;\n}\n"
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "layout.c")
        exe = os.path.join(d, "layout")
        open(c, "w").write(src)
        subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe])
        got = [int(x) for x in subprocess.check_output([exe]).split()]
    want = []
    for name, cls in STRUCTS:
        want.append(C_sizeof(cls))
        want += [getattr(cls, f[0]).offset for f in cls._fields_]
    assert got == want


def C_sizeof(cls):
    import ctypes
    return ctypes.sizeof(cls)


def _cases():
    cases = dict(parity_cases())
    return [cases["seir_events_300x120"], cases["sir_mparse_1000x150"], cases["sise_200x199"],
            cases["seir_events_rep5"], cases["sis_shift_weighted"]]


@pytest.mark.gpu
@pytest.mark.parametrize("budget", [0, 1])
def test_server_results_equal_alone(gpu, budget):
    from siminf_gb300.run import run, pfilter
    from siminf_gb300.serve import Server
    from siminf_gb300 import workloads
    models = _cases()
    seeds = [5, 6, 7, 8, 9]
    alone = [run(m, seed=s) for m, s in zip(models, seeds)]
    pm, gdata, t_obs, obs = workloads.sise_pfilter(nodes=60, particles=64, weeks=6)
    pf_alone = pfilter(pm, 64, t_obs, obs, 1, 0.8, seed=3, gdata=gdata)

    # budget 1 byte: one request at a time, in submission order or passing
    srv = Server(slots=4, hbm_budget_bytes=budget)
    tickets = [srv.run(m, seed=s) for m, s in zip(models, seeds)]
    tp = srv.pfilter(pm, 64, t_obs, obs, 1, 0.8, seed=3, gdata=gdata)
    tickets2 = [srv.run(m, seed=s) for m, s in zip(models, seeds)]
    for t in tickets + [tp] + tickets2:
        assert srv.wait(t)
    for t, a in zip(tickets, alone):
        assert np.array_equal(t.U, a.U)
        if a.V is not None:
            assert np.array_equal(t.holder.V[:a.V.size], a.V.reshape(-1, order="F"))
    for t, a in zip(tickets2, alone):
        assert np.array_equal(t.U, a.U)
    assert float(tp.loglik[0]) == pf_alone.loglik
    assert np.array_equal(tp.ess, pf_alone.ess)
    assert np.array_equal(tp.ancestors, pf_alone.ancestors)
    assert srv.load() == (0, 0, 0)
    assert all(t.latency_ms > 0 for t in tickets)
    srv.close()


@pytest.mark.gpu
def test_server_plan_continuation(gpu):
    from siminf_gb300 import native
    from siminf_gb300.serve import Server
    m = _cases()[0]
    ref = abi.build_args(m, 21)
    p = native.Plan(ref, m.name)
    p.run()
    p.download()
    want = ref.U.copy()
    srv = Server(slots=2)
    t = srv.plan(p)
    assert srv.wait(t)
    ref.U[:] = 0
    p.download()
    assert np.array_equal(ref.U, want)
    srv.close()
    p.close()


@pytest.mark.gpu
def test_server_aem_requests_equal_alone(gpu):
    """aem runs served beside ssm runs give what they give alone."""
    from siminf_gb300.run import run
    from siminf_gb300.serve import Server
    cases = dict(parity_cases())
    ms = [cases["seir_events_300x120"], cases["sise_200x199"], cases["sis_shift_weighted"]]
    alone = [run(m, seed=21, solver="aem") for m in ms]
    srv = Server(slots=3)
    tickets = [srv.run(m, seed=21, solver="aem") for m in ms]
    tickets += [srv.run(m, seed=21) for m in ms]
    for t in tickets:
        assert srv.wait(t)
    for t, a in zip(tickets[:3], alone):
        assert np.array_equal(t.U, a.U)
    for t, m in zip(tickets[3:], ms):
        assert np.array_equal(t.U, run(m, seed=21).U)
    srv.close()
