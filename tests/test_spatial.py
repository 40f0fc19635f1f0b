"""Spatial coupling (SISe_sp, SISe3_sp): the post time step of every node
reads its neighbours' compartments and phi (src/models/SISe_sp.c:108-160,
src/misc/SimInf_local_spread.c:43-71).  The neighbour lists are packed into
ldata as SimInf_ldata_sp does (src/misc/SimInf_ldata.c:50-135), checked
against the reference's own test vectors (tests/ldata_sp.R, lifted into
tests/golden/ldata_sp.json); the trajectories are checked in the shared
parity cases (oracle vs the reference's model files, GPU vs oracle)."""
import numpy as np
import pytest

from helpers import golden, run_gpu, run_oracle, run_ref
from oracle import oracle
from siminf_gb300 import model as M

needs_ref = pytest.mark.skipif(not oracle.ref_available(),
                               reason="reference sources were not available to build oracle/_ref")


def test_distance_matrix_and_ldata_sp_golden():
    fx = golden("ldata_sp.json")
    i, p, d = M.distance_matrix(fx["x"], fx["y"], fx["cutoff"])
    assert i.tolist() == fx["d_i"] and p.tolist() == fx["d_p"]
    assert np.all(np.abs(d - np.array(fx["d_x"])) < fx["tol"])
    data = np.repeat(np.array(fx["end_t"], dtype=float)[:, None], 10, axis=1)
    shape = tuple(fx["dim"])
    for metric, key in ((0, "ldata_degree"), (1, "ldata_distance"),
                        (2, "ldata_inverse_square")):
        got = M.ldata_sp(data, (i, p, d), metric)
        want = np.array(fx[key]).reshape(shape, order="F")
        assert got.shape == want.shape
        assert np.all(np.abs(got - want) < fx["tol"]), key


def test_distance_matrix_rejects_coincident_nodes_without_min_dist():
    with pytest.raises(ValueError, match="min_dist"):
        M.distance_matrix([1, 10, 1], [1, 10, 1], 20)
    i, p, d = M.distance_matrix([1, 10, 1], [1, 10, 1], 20, min_dist=0.5)
    assert d.min() == 0.5


def _sise_sp_errors():
    """tests/SISe_sp.R:1051-1099: infinite betas make phi non-finite (-7),
    a negative alpha makes it negative (-10)."""
    gx, gy = np.meshgrid(np.arange(3.0), np.arange(3.0))
    dist = M.distance_matrix(gx.ravel(), gy.ravel(), 2)
    base = dict(tspan=np.arange(0, 10), phi=np.ones(9), upsilon=0.0357, gamma=0.1,
                alpha=1.0, beta_t1=0.19, beta_t2=0.085, beta_t3=0.075, beta_t4=0.185,
                end_t1=91, end_t2=182, end_t3=273, end_t4=365, coupling=0.0005,
                distance=dist)
    inf = M.SISe_sp({"S": np.arange(9), "I": np.zeros(9)}, **base)
    inf.gdata[3:7] = np.inf
    neg = M.SISe_sp({"S": np.arange(9), "I": np.full(9, 10)},
                    **dict(base, upsilon=0.0, gamma=0.0, alpha=-1.0))
    return [("v_not_finite", inf, -7), ("v_negative", neg, -10)]


@needs_ref
@pytest.mark.parametrize("label,m,code", _sise_sp_errors(), ids=[c[0] for c in _sise_sp_errors()])
def test_oracle_spatial_errors_match_reference(oracle_lib, label, m, code):
    code_o, _, _ = run_oracle(m)
    code_r, _ = run_ref(m)
    assert code_o == code_r == code


@pytest.mark.gpu
@pytest.mark.parametrize("label,m,code", _sise_sp_errors(), ids=[c[0] for c in _sise_sp_errors()])
def test_gpu_spatial_errors(gpu, label, m, code):
    got, _, _ = run_gpu(m)
    assert got == code


@pytest.mark.gpu
def test_gpu_spatial_batch_rejected(gpu):
    """A batch numbers nodes across its models; a post time step that reads
    neighbours by their index in its own model cannot run there."""
    from helpers import parity_cases
    from siminf_gb300.run import run_batch
    m = dict(parity_cases())["sise_sp_grid_events"]
    with pytest.raises(Exception) as e:
        run_batch([m, m], [1, 2], numerator=(1,))
    assert getattr(e.value, "code", None) == -9
