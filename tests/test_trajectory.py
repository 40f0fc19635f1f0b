"""Trajectory and prevalence on the device (siminf_gpu_trajectory_u/_v,
siminf_gpu_prevalence) against the oracle's numpy restatement, which is
pinned to the reference's own test vectors: tests/prevalence.R:41-85 and
tests/trajectory.R:28-70."""
import numpy as np
import pytest

from helpers import parity_cases
from oracle import trajectory as ref
from siminf_gb300.trajectory import FormulaError, parse_formula

NAMES = ["S", "I", "R"]


def prevalence_fixture():
    """The 3-node SIR trajectory of tests/prevalence.R:41-55 (rows S, I, R
    of nodes 1-3, five time points), flattened column-major."""
    rows = np.array([[8, 8, 8, 8, 8], [0, 0, 0, 0, 0], [0, 0, 0, 0, 0],
                     [5, 4, 3, 2, 1], [1, 2, 3, 3, 3], [0, 0, 0, 1, 2],
                     [0, 0, 0, 0, 0], [0, 0, 0, 0, 0], [4, 4, 4, 4, 4]], dtype=np.int32)
    return np.ascontiguousarray(rows.T).reshape(-1)


def q(a, b):
    with np.errstate(invalid="ignore"):
        return np.array(a, dtype=np.float64) / np.array(b, dtype=np.float64)


# (formula, condition as a function of the compartments, index, expected):
# the level-1 cases of tests/prevalence.R:60-85.
GOLDEN = [
    ("I ~ .", None, None, q([1, 2, 3, 3, 3], [18] * 5)),
    ("I ~ . | R == 0", lambda S, I, R: R == 0, None, q([1, 2, 3, 0, 0], [14, 14, 14, 8, 8])),
    ("I ~ . | R > 0", lambda S, I, R: R > 0, None, q([0, 0, 0, 3, 3], [4, 4, 4, 10, 10])),
    ("I ~ . | (I + R) < 4", lambda S, I, R: (I + R) < 4, None,
     q([1, 2, 3, 0, 0], [14, 14, 14, 8, 8])),
    ("I ~ . | R == 5", lambda S, I, R: R == 5, None, q([0] * 5, [0] * 5)),
    ("I ~ . | S == 0 | R == 0", lambda S, I, R: (S == 0) | (R == 0), None,
     q([1, 2, 3, 0, 0], [18, 18, 18, 12, 12])),
    ("I ~ . | S == 0 | R == 0", lambda S, I, R: (S == 0) | (R == 0), [2],
     q([1, 2, 3, 0, 0], [6, 6, 6, 0, 0])),
]


def same(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return a.shape == b.shape and np.array_equal(np.isnan(a), np.isnan(b)) and \
        np.array_equal(a[~np.isnan(a)], b[~np.isnan(b)])


def eval_program(prog, cols):
    """A direct postfix evaluator of compile_condition's output, for the
    parser tests."""
    from siminf_gb300.abi import COND_OPS
    inv = {v: k for k, v in COND_OPS.items()}
    st = []
    for op, arg in prog:
        name = inv[op]
        if name == "compartment":
            st.append(cols[arg].astype(np.int64))
        elif name == "const":
            st.append(np.int64(arg))
        elif name == "neg":
            st.append(-st.pop())
        elif name == "!":
            st.append((st.pop() == 0).astype(np.int64))
        else:
            b, a = st.pop(), st.pop()
            r = {"+": a + b, "-": a - b, "*": a * b, "==": a == b, "!=": a != b, "<": a < b,
                 "<=": a <= b, ">": a > b, ">=": a >= b, "&": (a != 0) & (b != 0),
                 "|": (a != 0) | (b != 0)}[name]
            st.append(np.asarray(r).astype(np.int64))
    assert len(st) == 1
    return st[0] != 0


def test_oracle_prevalence_golden():
    U = prevalence_fixture()
    for formula, cond, index, want in GOLDEN:
        got = ref.prevalence(U, 3, 3, 5, 0b010, 0b111, 1, cond, index, NAMES)
        assert same(got, want), formula


def test_oracle_trajectory_golden():
    # tests/trajectory.R:28-47 (one replicate) and :52-70 (two replicates)
    for ncol in (10, 20):
        U = np.arange(1, 18 * ncol + 1, dtype=np.int32)
        got = ref.trajectory(U, 6, 3, ncol, [1, 2, 3])
        for k in range(3):
            assert np.array_equal(got[k], np.arange(k + 1, 18 * ncol + 1, 3))
    # nodes 2 and 5 (tests/trajectory.R's identifier subsets)
    got = ref.trajectory(np.arange(1, 181, dtype=np.int32), 6, 3, 10, [1, 3], id=[2, 5])
    assert np.array_equal(got[0], (np.array([4, 13]) + 18 * np.arange(10)[:, None]).ravel())
    assert np.array_equal(got[1], (np.array([6, 15]) + 18 * np.arange(10)[:, None]).ravel())


@pytest.mark.parametrize("text,fn", [
    ("S == 0 | R == 0", lambda S, I, R: (S == 0) | (R == 0)),
    ("(I + R) < 4", lambda S, I, R: (I + R) < 4),
    ("!(S > 2) & R <= 1 | -I < -3", lambda S, I, R: (~(S > 2) & (R <= 1)) | (-I < -3)),
    ("S * 2 == I + R * 3 - 1", lambda S, I, R: S * 2 == I + R * 3 - 1),
    ("S != I && I >= R || !(R == 1)", lambda S, I, R: ((S != I) & (I >= R)) | ~(R == 1)),
])
def test_condition_parser_follows_r_precedence(text, fn):
    rng = np.random.default_rng(3)
    cols = [rng.integers(0, 5, 200) for _ in range(3)]
    cases, pop, prog = parse_formula("I ~ . | " + text, NAMES)
    assert cases == 0b010 and pop == 0b111
    assert np.array_equal(eval_program(prog, cols), fn(*cols))


def test_formula_errors():
    with pytest.raises(FormulaError):
        parse_formula("~I", NAMES)
    with pytest.raises(FormulaError):
        parse_formula("I ~ Q", NAMES)
    with pytest.raises(FormulaError):
        parse_formula("I ~ . | R ==", NAMES)
    assert parse_formula("I ~ S + I", NAMES)[:2] == (0b010, 0b011)


# ---------------------------------------------------------------- GPU

def _device(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.gpu
def test_gpu_prevalence_golden(gpu):
    import ctypes as C
    from siminf_gb300.trajectory import prevalence_device
    dU = _device(prevalence_fixture())
    for formula, _, index, want in GOLDEN:
        cases, pop, prog = parse_formula(formula, NAMES)
        flat = [x for pair in prog for x in pair]
        got, st = prevalence_device(C.c_void_p(dU.data_ptr()), 3, 3, 5, cases, pop, 1, flat, index)
        assert same(got, want), formula
        assert st.bytes_read == 5 * (3 if index is None else len(index)) * 3 * 4


@pytest.mark.gpu
def test_gpu_trajectory_golden(gpu):
    import ctypes as C
    from siminf_gb300.trajectory import trajectory_device
    for ncol in (10, 20):
        U = np.arange(1, 18 * ncol + 1, dtype=np.int32)
        dU = _device(U)
        got, _ = trajectory_device(C.c_void_p(dU.data_ptr()), 6, 3, ncol, [1, 2, 3])
        assert np.array_equal(got, ref.trajectory(U, 6, 3, ncol, [1, 2, 3]))
        got, _ = trajectory_device(C.c_void_p(dU.data_ptr()), 6, 3, ncol, [3, 1], index=[5, 2, 6])
        assert np.array_equal(got, ref.trajectory(U, 6, 3, ncol, [3, 1], id=[5, 2, 6]))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["seir_events_rep5", "sise_200x199", "sise3_events"])
def test_gpu_reductions_of_a_run_match_the_oracle(gpu, name):
    from siminf_gb300 import abi, native
    from siminf_gb300.trajectory import COMPARTMENTS, prevalence, trajectory
    m = dict(parity_cases())[name]
    names = list(COMPARTMENTS[m.name])
    h = abi.build_args(m, 42)
    p = native.Plan(h, m.name)
    p.run()
    p.download()
    ncol = m.replicates * len(m.tspan)
    rng = np.random.default_rng(4)
    index = sorted(rng.choice(m.Nn, size=min(m.Nn, 17), replace=False) + 1)
    first, second = names[0], names[1]
    conds = [(None, None),
             ("%s > 3" % second, lambda **k: k[second] > 3),
             ("%s < 40 & %s + %s >= 2" % (first, second, first),
              lambda **k: (k[first] < 40) & (k[second] + k[first] >= 2))]
    for level in (1, 2, 3):
        for text, fn in conds:
            for idx in (None, index):
                formula = "%s ~ ." % second + (" | " + text if text else "")
                got = prevalence(p, formula, level=level, index=idx)
                cases, pop, _ = parse_formula(formula, names)
                want = ref.prevalence(h.U, m.Nn, m.Nc, ncol, cases, pop, level, fn, idx,
                                      names)
                assert same(got, want), (level, formula, idx is None)
    tr = trajectory(p, names[::-1], index=index)
    want = ref.trajectory(h.U, m.Nn, m.Nc, ncol, list(range(m.Nc, 0, -1)), id=index)
    for k, nm in enumerate(names[::-1]):
        assert np.array_equal(tr[nm], want[k])
    assert np.array_equal(tr["node"], np.tile(index, ncol))
    if m.Nd:
        import ctypes as C
        from siminf_gb300.trajectory import _outputs, trajectory_device
        _, dV, _ = _outputs(p)
        got, _ = trajectory_device(dV, m.Nn, m.Nd, ncol, [1], index=index, continuous=True)
        assert np.array_equal(got, ref.trajectory(h.V, m.Nn, m.Nd, ncol, [1], id=index))
    p.close()


@pytest.mark.gpu
def test_gpu_prevalence_errors(gpu):
    import ctypes as C
    from siminf_gb300 import abi, native
    from siminf_gb300.trajectory import prevalence, prevalence_device
    m = dict(parity_cases())["sir_builtin_odd_tspan"]
    h = abi.build_args(m, 42)
    p = native.Plan(h, m.name)
    with pytest.raises(abi.SimInfError, match="Please run the model first"):
        prevalence(p, "I ~ .")
    p.run()
    with pytest.raises(abi.SimInfError, match="'level' must be an integer"):
        prevalence(p, "I ~ .", level=4)
    dU = _device(prevalence_fixture())
    const = [abi.COND_OPS["const"], 1, abi.COND_OPS["const"], 0, abi.COND_OPS["=="], 0]
    with pytest.raises(abi.SimInfError, match="TRUE' or 'FALSE' for every node"):
        prevalence_device(C.c_void_p(dU.data_ptr()), 3, 3, 5, 2, 7, 1, const)
    with pytest.raises(abi.SimInfError, match="node index out of range"):
        prevalence_device(C.c_void_p(dU.data_ptr()), 3, 3, 5, 2, 7, 1, (), index=[4])
    p.close()
