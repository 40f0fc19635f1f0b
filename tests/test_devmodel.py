"""Model C code compiled for the device (siminf_gb300/devmodel.py) from the
output of mparse (siminf_gb300/mparse.py, a restatement of R/mparse.R and
R/C-generator.R): the generated models equal the hand-written device
models of the same transitions bit for bit, and a model that is not built
in runs bit-exact against the oracle running the same C code built on the
host (which equals the reference's solver running it)."""
import os

import numpy as np
import pytest

from helpers import random_events
from oracle import oracle
from siminf_gb300 import abi, devmodel, mparse
from siminf_gb300 import model as M

needs_ref = pytest.mark.skipif(not oracle.ref_available(),
                               reason="reference sources were not available to build oracle/_ref")

SIR_TRANSITIONS = ["S -> beta*S*I/N -> I", "I -> gamma*I -> R", "N <- S+I+R"]
PF_PTS = """    const double S_n = u[0];
    const double I_n = u[1];
    const double n = S_n + I_n;
    v_new[0] = v[0] * (1.0 - 0.03);
    if (n > 0.0)
        v_new[0] += 0.05 * I_n / n;
    return v[0] != v_new[0];"""


# A hand-written model file in the layout of the reference's src/models:
# enums, helpers from SimInf.h, and a run function that calls SimInf_run.
SPATIAL_MODEL_FILE = r'''
#include "SimInf.h"
#include <R_ext/Visibility.h>
enum { S, I };
enum { PHI };
enum { END_T1, END_T2, END_T3, END_T4, NEIGHBOR };
enum { UPSILON, GAMMA, ALPHA, BETA_T1, BETA_T2, BETA_T3, BETA_T4, COUPLING };
static double to_i(const int *u, const double *v, const double *ldata,
                   const double *gdata, double t)
{
    SIMINF_UNUSED(ldata);
    SIMINF_UNUSED(t);
    return gdata[UPSILON] * v[PHI] * u[S];
}
static double to_s(const int *u, const double *v, const double *ldata,
                   const double *gdata, double t)
{
    return gdata[GAMMA] * u[I];
}
static int pts(double *v_new, const int *u, const double *v, const double *ldata,
               const double *gdata, int node, double t)
{
    const int day = (int) t % 365;
    const double I_i = u[I];
    const double N_i = u[S] + I_i;
    const double phi = v[PHI];
    v_new[PHI] = SimInf_forward_euler_linear_decay(phi, day, ldata[END_T1], ldata[END_T2],
                                                   ldata[END_T3], ldata[END_T4],
                                                   gdata[BETA_T1], gdata[BETA_T2],
                                                   gdata[BETA_T3], gdata[BETA_T4]);
    if (N_i > 0.0)
        v_new[PHI] += gdata[ALPHA] * I_i / N_i +
            SimInf_local_spread(&ldata[NEIGHBOR], &v[-node], &u[-2 * node], N_i, phi, 2,
                                gdata[COUPLING]);
    if (!R_FINITE(v_new[PHI]))
        return SIMINF_ERR_V_IS_NOT_FINITE;
    if (v_new[PHI] < 0.0)
        return SIMINF_ERR_V_IS_NEGATIVE;
    return phi != v_new[PHI];
}
attribute_hidden SEXP my_model_run(SEXP model, SEXP options)
{
    TRFun tr_fun[] = { &to_i, &to_s };
    return SimInf_run(model, options, tr_fun, &pts);
}
'''


def sir_generated(nodes=200, days=120, seed=1):
    rng = np.random.default_rng(seed)
    u0 = {"S": rng.poisson(100, nodes), "I": rng.poisson(4, nodes), "R": np.zeros(nodes)}
    tspan = np.arange(1.0, days + 1)
    gen = mparse.mparse(SIR_TRANSITIONS, ["S", "I", "R"], u0, tspan,
                        gdata={"beta": 0.16, "gamma": 0.077})
    return gen, M.SIR_mparse(u0, tspan, 0.16, 0.077)


def sise_pf_generated(nodes=150, days=90, seed=2):
    rng = np.random.default_rng(seed)
    u0 = {"S": rng.poisson(100, nodes), "I": rng.poisson(2, nodes) * (rng.random(nodes) < .3)}
    tspan = np.arange(0.0, days)
    gen = mparse.mparse(["S -> upsilon*phi*S -> I", "I -> gamma*I -> S"], ["S", "I"], u0,
                        tspan, gdata={"upsilon": 0.02, "gamma": 0.1}, v0={"phi": 0.0},
                        pts_fun=PF_PTS)
    return gen, M.SISe_pf(u0, tspan, upsilon=0.02, gamma=0.1)


def seirs_custom(nodes=300, days=100, seed=3, use_enum=False, events=True):
    """A model no device model is written for: SEIRS with a waning
    transition, a local (per-node) beta, an (int) variable, a helper
    function from pre_code, and a continuous state v driven by the post
    time step; with exit, enter and external-transfer events."""
    rng = np.random.default_rng(seed)
    u0 = {"S": rng.poisson(200, nodes), "E": np.zeros(nodes),
          "I": rng.poisson(3, nodes) * (rng.random(nodes) < 0.2), "R": np.zeros(nodes)}
    ev = random_events(rng, nodes, days) if events else None
    pts = ("    v_new[0] = v[0] * 0.9 + 0.1 * (double) u[2] / (1.0 + u[0] + u[1] + u[2] + u[3]);"
           if not use_enum else
           "    v_new[PRESSURE] = v[PRESSURE] * 0.9 + 0.1 * (double) u[I] / "
           "(1.0 + u[S] + u[E] + u[I] + u[R]);")
    pts += "\n    return v_new[0] != v[0];"
    return mparse.mparse(
        ["S -> beta*S*I/N + pressure*S -> E", "E -> epsilon*E -> I",
         "I -> gamma*I + half(gamma)*I*0.0 -> R", "R -> omega*R -> S",
         "N <- Ntot", "(int) Ntot <- S+E+I+R"],
        ["S", "E", "I", "R"], u0, np.arange(1.0, days + 1),
        gdata={"epsilon": 0.25, "gamma": 0.077, "omega": 0.01},
        ldata={"beta": rng.uniform(0.1, 0.3, nodes)}, v0={"pressure": 0.0},
        pts_fun=pts, use_enum=use_enum, events=ev,
        E=np.array([[1, 1], [0, 1], [0, 1], [0, 1]], dtype=float),
        pre_code="static double half(double x)\n{\n    return 0.5 * x;\n}")


def test_mparse_emits_the_reference_layout():
    gen, _ = sir_generated(nodes=3, days=5)
    code = gen.C_code
    assert "static double trFun1(" in code and "static double trFun2(" in code
    assert "    const double N = u[0]+u[1]+u[2];\n\n    return gdata[0]*u[0]*u[1]/N;" in code
    assert "    return gdata[1]*u[1];" in code
    assert "TRFun tr_fun[] = {&trFun1, &trFun2};" in code
    assert "return SimInf_run(model, options, tr_fun, &ptsFun);" in code
    assert gen.G.tolist() == [[1, 1], [1, 1]]
    assert gen.S.tolist() == [[-1, 0], [1, -1], [0, 1]]


def test_mparse_dependency_graph_and_variables():
    m = seirs_custom(nodes=4, days=3, events=False)
    # rate 1 reads S, E, I, R (through N and Ntot): every transition changes
    # one of them; rate 2 reads E (changed by S -> E, E -> I); rate 3 reads
    # I (E -> I, I -> R); rate 4 reads R (I -> R, R -> S)
    assert m.G.tolist() == [[1, 1, 1, 1], [1, 1, 0, 0], [0, 1, 1, 0], [0, 0, 1, 1]]
    code = m.C_code
    i1 = code.index("static double trFun1(")
    body = code[i1:code.index("}", i1)]
    # variables in dependency order: Ntot before N
    assert body.index("const int Ntot = u[0]+u[1]+u[2]+u[3];") < \
        body.index("const double N = Ntot;")
    assert "return ldata[0]*u[0]*u[2]/N+v[0]*u[0];" in body
    e = seirs_custom(nodes=4, days=3, events=False, use_enum=True)
    assert "return ldata[BETA]*u[S]*u[I]/N+v[PRESSURE]*u[S];" in e.C_code
    assert "    S = 0,\n    E = 1,\n    I = 2,\n    R = 3,\n    N_COMPARTMENTS_U = 4" in e.C_code


def test_mparse_rejects_bad_transitions():
    with pytest.raises(ValueError, match="Unknown compartment"):
        mparse.c_code(["S -> b*S -> X"], ["S", "I"], gdata_names=["b"])
    with pytest.raises(ValueError, match="Invalid transition"):
        mparse.c_code(["S -> I"], ["S", "I"])
    with pytest.raises(ValueError, match="empty set"):
        mparse.c_code(["@ + S -> b -> I"], ["S", "I"], gdata_names=["b"])


def test_device_source_keeps_the_signatures_and_drops_the_r_glue():
    m = seirs_custom(nodes=4, days=3, events=False)
    src = devmodel.device_source(m.C_code, m.Nc, m.Nt, m.Nd, 3)
    assert "__device__ static double trFun1(\n    const int *u," in src
    assert "__device__ static int ptsFun(" in src
    assert "__device__ static double half(double x)" in src
    assert "SEXP" not in src and "R_init" not in src and "Rdynload" not in src
    assert "static constexpr bool PTS_LOCAL = true;" in src
    assert "case 3" not in src and "default: return ::trFun4(" in src


def test_device_source_of_a_reference_style_model_file():
    """A hand-written model file in the layout of the reference's
    src/models (enums, attribute_hidden run function calling SimInf_run
    directly, helpers from SimInf.h): the run function's tr_fun order and
    post-time-step function are found, and a post time step that reaches
    other nodes through `node` is marked non-local."""
    code = SPATIAL_MODEL_FILE
    pc = devmodel.parse_model_code(code)
    assert pc.tr_names == ["to_i", "to_s"] and pc.pts_name == "pts"
    src = devmodel.device_source(code, 2, 2, 1, 8)
    assert "static constexpr bool PTS_LOCAL = false;" in src
    assert "my_model_run" not in src and "__device__ static int pts(" in src


def test_generated_model_compiles_for_the_device():
    """nvcc builds the device model library (no GPU needed to compile)."""
    gen, _ = sir_generated(nodes=4, days=5)
    path = devmodel.compile(gen.C_code, gen.Nc, gen.Nt, gen.Nd, 2)
    assert os.path.exists(path) and path.endswith(".so")
    assert devmodel.compile(gen.C_code, gen.Nc, gen.Nt, gen.Nd, 2) == path   # cached


def test_model_libraries_keep_their_own_tables():
    """Several model libraries in one process each hand out their own
    launcher table (their instantiations must not be shared through
    process-wide symbols); no GPU is needed to load them."""
    import ctypes as C
    from siminf_gb300 import native
    native.lib()
    dims = []
    for gen, ngd in ((sir_generated()[0], 2), (sise_pf_generated()[0], 2),
                     (seirs_custom(nodes=4, days=3, events=False), 3)):
        lib = C.CDLL(devmodel.compile(gen.C_code, gen.Nc, gen.Nt, gen.Nd, ngd))
        lib.siminf_model_launchers.restype = C.POINTER(C.c_int * 4)
        dims.append(list(lib.siminf_model_launchers().contents))
    assert dims == [[3, 2, 0, 2], [2, 2, 1, 2], [4, 4, 1, 3]]


@pytest.mark.parametrize("factory", [sir_generated, sise_pf_generated])
def test_oracle_generated_equals_hand_written(oracle_lib, factory):
    """The host build of the generated code gives the hand-written host
    model's trajectories (the oracle's SIR_mparse and SISe_pf)."""
    gen, hand = factory()
    oracle.register_c_model(gen.name, gen.C_code, gen.Nc, gen.Nt, gen.Nd)
    hg = abi.build_args(gen, 42)
    hh = abi.build_args(hand, 42)
    assert oracle.run(hg, gen.name, 2)[0] == 0
    assert oracle.run(hh, hand.name, 2)[0] == 0
    assert np.array_equal(hg.U, hh.U) and np.array_equal(hg.V, hh.V)


@needs_ref
@pytest.mark.parametrize("use_enum", [False, True])
def test_oracle_custom_model_matches_reference(oracle_lib, use_enum):
    m = seirs_custom(use_enum=use_enum)
    oracle.register_c_model(m.name, m.C_code, m.Nc, m.Nt, m.Nd)
    ho = abi.build_args(m, 42)
    code_o, res = oracle.run(ho, m.name, 3)
    hr = abi.build_args(m, 42)
    code_r = oracle.run_ref(hr, m.name, 3)
    assert code_o == code_r == 0
    assert np.array_equal(ho.U, hr.U) and np.array_equal(ho.V, hr.V)
    assert res.transitions > 1000


@pytest.mark.gpu
@pytest.mark.parametrize("factory", [sir_generated, sise_pf_generated])
def test_gpu_generated_equals_hand_written(gpu, factory):
    """The generated model on the device, through the C ABI, gives the
    built-in device model's trajectories bit for bit."""
    from helpers import run_gpu
    gen, hand = factory()
    code_g, hg, sg = run_gpu(gen)
    code_h, hh, sh = run_gpu(hand)
    assert code_g == code_h == 0
    assert np.array_equal(hg.U, hh.U) and np.array_equal(hg.V, hh.V)
    assert sg.transitions == sh.transitions


@pytest.mark.gpu
@pytest.mark.parametrize("use_enum", [False, True])
@pytest.mark.parametrize("heavy_rate,two_pass", [(-1, -1), (1, 1)])
def test_gpu_custom_model_matches_oracle(gpu, oracle_lib, use_enum, heavy_rate, two_pass):
    import ctypes as C
    from siminf_gb300 import native
    m = seirs_custom(use_enum=use_enum)
    oracle.register_c_model(m.name, m.C_code, m.Nc, m.Nt, m.Nd)
    ho = abi.build_args(m, 42)
    code_o, res = oracle.run(ho, m.name, 4)
    assert code_o == 0
    h = abi.build_args(m, 42)
    opt = abi.Options(heavy_rate=heavy_rate, two_pass=two_pass)
    code = native.lib().siminf_gpu_run_solver_ex(C.cast(h.ref(), C.c_void_p),
                                                 native.device_model(m.name).handle,
                                                 C.byref(opt))
    assert code == 0, native.last_status().message
    assert np.array_equal(h.U, ho.U) and np.array_equal(h.V, ho.V)
    assert native.last_stats().transitions == res.transitions


@pytest.mark.gpu
def test_gpu_custom_model_replicates_and_aem(gpu, oracle_lib):
    """The compiled model under the other solver paths: replicates with
    the whole-horizon kernel (no external transfers) and the aem solver."""
    from helpers import run_gpu
    from siminf_gb300.run import run
    m = seirs_custom(events=False, nodes=120, days=60).replicate(3)
    oracle.register_c_model(m.name, m.C_code, m.Nc, m.Nt, m.Nd)
    ho = abi.build_args(m, 5)
    assert oracle.run(ho, m.name, 3)[0] == 0
    code, hg, _ = run_gpu(m, seed=5)
    assert code == 0 and np.array_equal(hg.U, ho.U)
    one = seirs_custom(nodes=120, days=60)
    ha = abi.build_args(one, 7, solver=1)
    assert oracle.run(ha, one.name, 3)[0] == 0
    r = run(one, seed=7, solver="aem")
    assert np.array_equal(r.U, ha.U.reshape(r.U.shape, order="F"))


@pytest.mark.gpu
def test_gpu_spatial_model_file_equals_built_in(gpu):
    """The reference-style spatial model file above, compiled for the
    device, gives the built-in SISe_sp's trajectories on the spatial parity
    case (its post time step reads the neighbours after the day's
    transfers)."""
    from helpers import parity_cases, run_gpu
    from siminf_gb300 import native
    m = dict(parity_cases())["sise_sp_grid_events"]
    gen = M.SimInfModel("spatial_model_file", m.G, m.S, m.u0, m.tspan, v0=m.v0,
                        ldata=m.ldata, gdata=m.gdata, E=m.E, N=m.N, events=m.events)
    native.register_model_code(gen.name, SPATIAL_MODEL_FILE, 2, 2, 1, 8)
    code_g, hg, _ = run_gpu(gen)
    code_h, hh, _ = run_gpu(m)
    assert code_g == code_h == 0
    assert np.array_equal(hg.U, hh.U) and np.array_equal(hg.V, hh.V)
