"""Trajectory and prevalence of a run, computed where the run left U and V
in HBM: the counterparts of SimInf's trajectory() (the long format built by
src/misc/SimInf_trajectory.c) and prevalence() (R/prevalence.R), through
siminf_gpu_trajectory_u/_v and siminf_gpu_prevalence.

    plan.run()
    p = prevalence(plan, "I ~ S + I + R", level=1)
    p = prevalence(plan, "I ~ . | R == 0", level=2, index=[1, 5, 9])
    df = trajectory(plan, ["S", "I"], index=[1, 2, 3])

Formulas follow prevalence(): cases on the left of `~`, the population at
risk on the right (`.` for every compartment), compartments joined by `+`,
and an optional condition after `|` in R's syntax and precedence
(`|`/`||` below `&`/`&&` below `!` below comparisons below `+ -` below
`*` below unary minus), over compartments and integer constants.
"""
import ctypes as C
import re

import numpy as np

from . import abi, native

# Compartment names of the shipped device models, in U's row order.
COMPARTMENTS = {
    "SIR": ("S", "I", "R"), "SIR_mparse": ("S", "I", "R"), "SEIR": ("S", "E", "I", "R"),
    "SIS": ("S", "I"), "SISe": ("S", "I"), "SISe_pf": ("S", "I"),
    "SISe3": ("S_1", "I_1", "S_2", "I_2", "S_3", "I_3"),
}


class FormulaError(ValueError):
    pass


_TOKEN = re.compile(r"\s*(\|\||&&|==|!=|<=|>=|[A-Za-z_.][A-Za-z0-9_.]*|\d+|[()+\-*<>!&|])")


def _tokens(text):
    pos, out = 0, []
    text = text.strip()
    while pos < len(text):
        m = _TOKEN.match(text, pos)
        if not m:
            raise FormulaError("Invalid 'formula' specification.")
        out.append(m.group(1))
        pos = m.end()
    return out


def compile_condition(text, names):
    """The postfix program (pairs of SIMINF_GPU_COND_* operator, argument)
    of an R condition over the compartments `names`."""
    toks = _tokens(text)
    ops = abi.COND_OPS
    prog = []
    i = 0

    def peek():
        return toks[i] if i < len(toks) else None

    def take():
        nonlocal i
        i += 1
        return toks[i - 1]

    def expr_or():
        expr_and()
        while peek() in ("|", "||"):
            take()
            expr_and()
            prog.append((ops["|"], 0))

    def expr_and():
        expr_not()
        while peek() in ("&", "&&"):
            take()
            expr_not()
            prog.append((ops["&"], 0))

    def expr_not():
        if peek() == "!":
            take()
            expr_not()
            prog.append((ops["!"], 0))
        else:
            expr_cmp()

    def expr_cmp():
        expr_add()
        while peek() in ("==", "!=", "<", "<=", ">", ">="):
            op = take()
            expr_add()
            prog.append((ops[op], 0))

    def expr_add():
        expr_mul()
        while peek() in ("+", "-"):
            op = take()
            expr_mul()
            prog.append((ops[op], 0))

    def expr_mul():
        expr_unary()
        while peek() == "*":
            take()
            expr_unary()
            prog.append((ops["*"], 0))

    def expr_unary():
        if peek() == "-":
            take()
            expr_unary()
            prog.append((ops["neg"], 0))
        elif peek() == "+":
            take()
            expr_unary()
        else:
            atom()

    def atom():
        t = take() if peek() is not None else None
        if t is None:
            raise FormulaError("Invalid 'formula' specification.")
        if t == "(":
            expr_or()
            if take() != ")":
                raise FormulaError("Invalid 'formula' specification.")
        elif t.isdigit():
            if int(t) > 2 ** 31 - 1:
                raise FormulaError("constant out of range")
            prog.append((ops["const"], int(t)))
        elif t in names:
            prog.append((ops["compartment"], names.index(t)))
        elif t in ("TRUE", "FALSE"):
            prog.append((ops["const"], 1 if t == "TRUE" else 0))
        else:
            raise FormulaError("Non-existing compartment(s) in model: '%s'." % t)

    try:
        expr_or()
    except IndexError:
        raise FormulaError("Invalid 'formula' specification.")
    if i != len(toks):
        raise FormulaError("Invalid 'formula' specification.")
    return prog


def parse_formula(formula, names):
    """(cases mask, population mask, condition program) of a prevalence
    formula such as 'I ~ S + I + R | R == 0'."""
    if "~" not in formula:
        raise FormulaError("Invalid 'formula' specification.")
    lhs, rhs = formula.split("~", 1)
    cond = None
    if "|" in rhs:
        j = rhs.index("|")
        rhs, cond = rhs[:j], rhs[j + 1:]

    def mask(side):
        side = side.strip()
        if not side:
            raise FormulaError("Invalid 'formula' specification.")
        if side == ".":
            return (1 << len(names)) - 1
        m = 0
        for part in side.split("+"):
            part = part.strip()
            if part == ".":
                return (1 << len(names)) - 1
            if part not in names:
                raise FormulaError("Non-existing compartment(s) in model: '%s'." % part)
            m |= 1 << names.index(part)
        return m

    return mask(lhs), mask(rhs), (compile_condition(cond, names) if cond else [])


def _names(plan, compartments):
    if compartments is not None:
        return list(compartments)
    name = plan.model.name if hasattr(plan.model, "name") else None
    if name not in COMPARTMENTS:
        raise ValueError("compartment names unknown for this model; pass compartments=")
    return list(COMPARTMENTS[name])


def _outputs(plan):
    dU, dV, ncol = C.c_void_p(), C.c_void_p(), C.c_int()
    native.check(native.lib().siminf_gpu_plan_outputs(plan.handle, C.byref(dU), C.byref(dV),
                                                      C.byref(ncol)))
    return dU, dV, ncol.value


def _ids(index):
    if index is None:
        return None, 0
    ids = np.ascontiguousarray(np.asarray(index, dtype=np.int32).reshape(-1))
    return ids, len(ids)


def prevalence_device(d_U, Nn, Nc, ncol, cases, population, level=1, condition=(),
                      index=None, stream=None):
    """siminf_gpu_prevalence on a device U; condition is the flat list of
    (operator, argument) pairs.  Returns (values, ReduceStats)."""
    ids, n_id = _ids(index)
    n = n_id if ids is not None else Nn
    out = np.empty(ncol * n if level == 3 else ncol, dtype=np.float64)
    prog = np.ascontiguousarray(np.asarray(condition, dtype=np.int32).reshape(-1))
    if len(prog) % 2:
        raise ValueError("condition: (operator, argument) pairs expected")
    spec = abi.PrevalenceSpec(cases=cases, population=population, level=level,
                              n_condition=len(prog) // 2,
                              condition=prog.ctypes.data_as(C.POINTER(C.c_int))
                              if len(prog) else None)
    st = abi.ReduceStats()
    native.check(native.lib().siminf_gpu_prevalence(
        d_U, Nn, Nc, ncol, C.byref(spec),
        ids.ctypes.data_as(C.POINTER(C.c_int)) if ids is not None else None, n_id,
        out.ctypes.data_as(C.POINTER(C.c_double)), stream, C.byref(st)))
    return (out.reshape(ncol, n) if level == 3 else out), st


def trajectory_device(d_M, Nn, stride, ncol, variables, index=None, stream=None, continuous=False):
    """siminf_gpu_trajectory_u (or _v) on a device U (or V); variables are
    one-based.  Returns (array [len(variables), ncol * n], ReduceStats)."""
    ids, n_id = _ids(index)
    n = n_id if ids is not None else Nn
    var = np.ascontiguousarray(np.asarray(variables, dtype=np.int32))
    out = np.empty((len(var), ncol * n), dtype=np.float64 if continuous else np.int32)
    st = abi.ReduceStats()
    fn = native.lib().siminf_gpu_trajectory_v if continuous else native.lib().siminf_gpu_trajectory_u
    ptr = out.ctypes.data_as(C.POINTER(C.c_double) if continuous else C.POINTER(C.c_int))
    native.check(fn(d_M, Nn, stride, ncol, var.ctypes.data_as(C.POINTER(C.c_int)), len(var),
                    ids.ctypes.data_as(C.POINTER(C.c_int)) if ids is not None else None, n_id,
                    ptr, stream, C.byref(st)))
    return out, st


def prevalence(plan, formula, level=1, index=None, compartments=None, stream=None):
    """prevalence(model, formula, level, index) of a plan that has run:
    one value per column of U (replicate-major, then time) for levels 1
    and 2, an array [column, node] for level 3."""
    names = _names(plan, compartments)
    cases, pop, cond = parse_formula(formula, names)
    dU, _, ncol = _outputs(plan)
    a = plan.holder.args
    flat = [x for pair in cond for x in pair]
    vals, _ = prevalence_device(dU, a.Nn, a.Nc, ncol, cases, pop, level, flat, index, stream)
    return vals


def trajectory(plan, compartments_wanted=None, index=None, compartments=None, stream=None):
    """trajectory(model, compartments, index) of a plan that has run, in
    SimInf's long format: a dict with `node`, `time` (tspan values),
    `replicate` when there are several, and one array per compartment; rows
    ordered by replicate, time, node."""
    names = _names(plan, compartments)
    wanted = names if compartments_wanted is None else list(compartments_wanted)
    for w in wanted:
        if w not in names:
            raise FormulaError("Non-existing compartment(s) in model: '%s'." % w)
    dU, _, ncol = _outputs(plan)
    a = plan.holder.args
    vals, _ = trajectory_device(dU, a.Nn, a.Nc, ncol, [names.index(w) + 1 for w in wanted],
                                index, stream)
    ids = np.arange(1, a.Nn + 1) if index is None else np.asarray(index)
    tspan = np.ctypeslib.as_array(a.tspan, shape=(a.tlen,))
    out = {"node": np.tile(ids, ncol),
           "time": np.tile(np.repeat(tspan, len(ids)), a.Nrep)}
    if a.Nrep > 1:
        out["replicate"] = np.repeat(np.arange(1, a.Nrep + 1), a.tlen * len(ids))
    for k, w in enumerate(wanted):
        out[w] = vals[k]
    return out
