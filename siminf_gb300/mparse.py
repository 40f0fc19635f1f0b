"""mparse(): a model from transition strings, with its C code.

A restatement of the reference's mparse (R/mparse.R:27-491, 647-724) and of
the C code generator behind it (R/C-generator.R): the same tokenizer (the
C operator and punctuator list, longest first), the same rewriting of
compartment, ldata, gdata and v0 names into u[..], ldata[..], gdata[..]
and v[..] (or enumeration constants with use_enum), variables ("N <-
S+I+R", optionally "(int)" or "(double)", topologically sorted with ties
broken by name), the state-change matrix S (dest - from) and the
dependency graph G = (depends %*% |S|) > 0, and C code with the layout of
C_code_mparse: enumerations, pre_code, trFun1..trFunK with the variables
each needs, ptsFun with the given body, and the run function that hands
tr_fun and ptsFun to SimInf_run.

The model it returns runs on the GPU through siminf_gb300.devmodel, which
compiles that C code for the device: its name is "mparse_" followed by a
digest of the code, and it is registered with the native layer the first
time it is built.  R-level argument checks and the model's S4 class are
not rebuilt.
"""
import hashlib
import re

import numpy as np

from . import native
from .model import SimInfModel

OPERATORS = ["<<=", ">>=", "!=", "%=", "##", "&&", "&=", "*=", "++", "+=", "--", "-=",
             "->", "/=", "<<", "<=", "==", ">=", ">>", "^=", "|=", "||", "!", "~", "%",
             "&", "(", ")", "*", "+", ",", "-", "/", ":", ";", "<", "=", ">", "?", "[",
             "]", "^", "{", "|", "}", "#"]

VARIABLE = re.compile(r"^\s*(\(double\)|\(int\))?\s*([a-zA-Z_][a-zA-Z_0-9]*)\s*<-")


def tokenize(code):
    """Split code on the operators, one operator after the other in the
    list's order, as R/mparse.R:27-85 does: a piece already split off as an
    operator is not split again; the rest are trimmed, empty ones dropped."""
    pieces = [(code, False)]
    for op in OPERATORS:
        out = []
        for text, is_op in pieces:
            if is_op or op not in text:
                out.append((text, is_op))
                continue
            parts = text.split(op)
            for k, part in enumerate(parts):
                part = part.strip()
                if part:
                    out.append((part, False))
                if k < len(parts) - 1:
                    out.append((op, True))
        pieces = out
    return [t for t, _ in pieces]


def _substitute(tokens, names, target, use_enum):
    out = []
    for t in tokens:
        if t in names:
            k = names.index(t)
            out.append("%s[%s]" % (target, t.upper() if use_enum else str(k)))
        else:
            out.append(t)
    return out


def _rewrite(tokens, compartments, ldata_names, gdata_names, v0_names, use_enum):
    tokens = _substitute(tokens, compartments, "u", use_enum)
    tokens = _substitute(tokens, ldata_names, "ldata", use_enum)
    tokens = _substitute(tokens, gdata_names, "gdata", use_enum)
    return _substitute(tokens, v0_names, "v", use_enum)


def _parse_compartments(x, compartments):
    """'2*S + I' -> counts per compartment; '@' is the empty set."""
    names = []
    for part in x.split("+"):
        part = part.replace(" ", "")
        m = re.match(r"^([0-9]+)\*", part)
        if m:
            names += [part[m.end():]] * int(m.group(1))
        else:
            names.append(part)
    if "@" in names and len(names) > 1:
        raise ValueError("Invalid usage of the empty set '@'.")
    names = [n for n in names if n != "@"]
    counts = np.zeros(len(compartments), dtype=np.int32)
    for n in names:
        if n not in compartments:
            raise ValueError("Unknown compartment: '%s'." % n)
        counts[compartments.index(n)] += 1
    return counts


def _topological_sort(names, deps):
    """Variables ordered so that each follows the ones it uses (R/mparse.R:
    372-399): lexicographic to break ties, then repeatedly the first
    variable with no unmet dependency."""
    names = sorted(names)
    remaining = {n: set(deps[n]) for n in names}
    order = []
    ready = [n for n in names if not remaining[n]]
    if not ready:
        raise ValueError("Invalid dependencies between variables.")
    while ready:
        v = ready.pop(0)
        order.append(v)
        for n in names:
            if v in remaining[n]:
                remaining[n].discard(v)
                if not remaining[n] and n not in order and n not in ready:
                    ready.append(n)
    if len(order) != len(names):
        raise ValueError("Invalid dependencies between variables.")
    return order


def _enum_block(target, labels):
    if not labels:
        return []
    lines = ["/* Enumeration constants for indicies in the '%s' vector. */" % target, "enum {"]
    for k, lbl in enumerate(labels):
        lines.append("    %s = %d%s" % (lbl.upper(), k, "," if k < len(labels) - 1 else ""))
    return lines + ["};", ""]


def c_code(transitions, compartments, ldata_names=(), gdata_names=(), v0_names=(),
           pts_fun=None, use_enum=False, pre_code=None):
    """(C code, S, G) for the transitions, laid out as C_code_mparse
    (R/C-generator.R:392-416) writes it."""
    compartments = list(compartments)
    ldata_names, gdata_names, v0_names = list(ldata_names), list(gdata_names), list(v0_names)
    args = (compartments, ldata_names, gdata_names, v0_names, use_enum)

    variables = {}
    order = []
    props = []
    for tr in transitions:
        m = VARIABLE.match(tr)
        if m:
            typ = m.group(1)[1:-1] if m.group(1) else "double"
            name = m.group(2)
            if name in compartments + ldata_names + gdata_names + v0_names:
                raise ValueError("Variable name already exists in 'u0', 'gdata', 'ldata' or "
                                 "'v0'.")
            tokens = tokenize(tr[m.end():].replace(" ", ""))
            variables[name] = {"type": typ, "tokens": tokens,
                               "compartments": [c for c in dict.fromkeys(tokens)
                                                if c in compartments]}
            order.append(name)
        else:
            props.append(tr)
    if len(set(order)) != len(order):
        raise ValueError("Variables must have non-duplicated names.")
    deps = {n: [t for t in variables[n]["tokens"] if t in variables] for n in variables}
    for n in variables:
        variables[n]["code"] = "".join(_rewrite(variables[n]["tokens"], *args))
    sorted_vars = _topological_sort(list(variables), deps) if variables else []

    S_cols, dep_rows, parsed = [], [], []
    for tr in props:
        parts = tr.split("->")
        if len(parts) < 3:
            raise ValueError("Invalid transition: '%s'." % tr)
        propensity = "->".join(p.replace(" ", "") for p in parts[1:-1])
        from_ = _parse_compartments(parts[0], compartments)
        dest = _parse_compartments(parts[-1], compartments)
        S_cols.append(dest - from_)
        tokens = tokenize(propensity)
        used = [t for t in dict.fromkeys(tokens) if t in variables]
        depends = np.zeros(len(compartments), dtype=np.int32)
        for t in tokens:
            if t in compartments:
                depends[compartments.index(t)] = 1
        todo = list(used)
        seen = set()
        while todo:
            v = todo.pop(0)
            if v in seen:
                continue
            seen.add(v)
            for c in variables[v]["compartments"]:
                depends[compartments.index(c)] = 1
            todo += deps[v]
        dep_rows.append(depends)
        # variables this propensity needs, with their own dependencies, in
        # the sorted order (R/C-generator.R:164-193)
        need = set()
        todo = list(used)
        while todo:
            v = todo.pop(0)
            if v not in need:
                need.add(v)
                todo += deps[v]
        parsed.append(("".join(_rewrite(tokens, *args)),
                       [v for v in sorted_vars if v in need]))
    S = np.column_stack(S_cols).astype(np.int32)
    G = ((np.vstack(dep_rows) @ np.abs(S)) > 0).astype(np.int32)

    lines = ["/* Generated by siminf_gb300.mparse */", "",
             "#include <R_ext/Rdynload.h>", '#include "SimInf.h"', "",
             "#if !defined(SIMINF_MODEL_RUN)",
             "#  error Definition for 'SIMINF_MODEL_RUN' is missing.", "#endif",
             "#if !defined(SIMINF_R_INIT)",
             "#  error Definition for 'SIMINF_R_INIT' is missing.", "#endif",
             "#if !defined(SIMINF_FORCE_SYMBOLS)",
             "#  error Definition for 'SIMINF_FORCE_SYMBOLS' is missing.", "#endif", ""]
    if use_enum:
        lines += _enum_block("u", compartments + ["N_COMPARTMENTS_U"])
        if v0_names:
            lines += _enum_block("v", v0_names + ["N_COMPARTMENTS_V"])
        lines += _enum_block("ldata", ldata_names) + _enum_block("gdata", gdata_names)
    if pre_code:
        lines += ["/* User defined code. */"] + pre_code.split("\n") + [""]
    for k, (code, need) in enumerate(parsed, 1):
        lines += ["static double trFun%d(" % k, "    const int *u,", "    const double *v,",
                  "    const double *ldata,", "    const double *gdata,", "    double t)", "{"]
        for v in need:
            lines.append("    const %s %s = %s;" % (variables[v]["type"], v,
                                                     variables[v]["code"]))
        if need:
            lines.append("")
        lines += ["    return %s;" % code, "}", ""]
    body = pts_fun if pts_fun is not None else "    return 0;"
    lines += ["static int ptsFun(", "    double *v_new,", "    const int *u,",
              "    const double *v,", "    const double *ldata,", "    const double *gdata,",
              "    int node,", "    double t)", "{"] + body.split("\n") + ["}", ""]
    lines += ["static SEXP SIMINF_MODEL_RUN(SEXP model, SEXP options)", "{",
              "    static SEXP(*SimInf_run)(SEXP, SEXP, TRFun*, PTSFun) = NULL;",
              "    TRFun tr_fun[] = {%s};" % ", ".join("&trFun%d" % k
                                                      for k in range(1, len(parsed) + 1)),
              "", "    if (!SimInf_run) {",
              "        SimInf_run = (SEXP(*)(SEXP, SEXP, TRFun*, PTSFun))",
              '            R_GetCCallable("SimInf", "SimInf_run");', "",
              "        if (!SimInf_run) {",
              "            Rf_error(\"Cannot find function 'SimInf_run'.\");", "        }",
              "    }", "", "    return SimInf_run(model, options, tr_fun, &ptsFun);", "}", "",
              "static const R_CallMethodDef callMethods[] =", "{",
              "    SIMINF_CALLDEF(SIMINF_MODEL_RUN, 2),", "    {NULL, NULL, 0}", "};", "",
              "void SIMINF_R_INIT(DllInfo *info)", "{",
              "    R_registerRoutines(info, NULL, callMethods, NULL, NULL);",
              "    R_useDynamicSymbols(info, FALSE);",
              "    R_forceSymbols(info, SIMINF_FORCE_SYMBOLS);", "}"]
    return "\n".join(lines) + "\n", S, G


def _names(x):
    if x is None:
        return [], None
    if isinstance(x, dict):
        return list(x), np.asarray(list(x.values()), dtype=np.float64)
    raise ValueError("named parameters are given as a dict of name -> value(s)")


def mparse(transitions, compartments, u0, tspan, gdata=None, ldata=None, v0=None,
           events=None, E=None, N=None, pts_fun=None, use_enum=False, pre_code=None,
           replicates=1):
    """The model R's mparse() builds (R/mparse.R:647-724).  gdata: dict
    name -> value; ldata and v0: dict name -> one value per node (or one
    value for all); u0: dict compartment -> counts, or an (Nc, Nn) array.
    Returns a SimInfModel whose C_code attribute holds the generated code;
    its device model is built from that code on first use."""
    compartments = list(compartments)
    if isinstance(u0, dict):
        cols = [np.atleast_1d(np.asarray(u0[c])) for c in compartments]
        n = max(len(c) for c in cols)
        u0 = np.vstack([np.broadcast_to(c, (n,)) for c in cols]).astype(np.int32)
    u0 = np.asarray(u0, dtype=np.int32)
    nn = u0.shape[1] // replicates
    gdata_names, gvals = _names(gdata)
    ldata_names, lvals = (list(ldata), None) if ldata else ([], None)
    v0_names = list(v0) if v0 else []
    if len(set(compartments + gdata_names + ldata_names + v0_names)) != \
            len(compartments) + len(gdata_names) + len(ldata_names) + len(v0_names):
        raise ValueError("'u0', 'gdata', 'ldata' and 'v0' have names in common.")
    code, S, G = c_code(transitions, compartments, ldata_names, gdata_names, v0_names,
                        pts_fun, use_enum, pre_code)
    ld = (np.vstack([np.broadcast_to(np.asarray(ldata[k], dtype=np.float64), (nn,))
                     for k in ldata_names]) if ldata_names else None)
    vv = (np.vstack([np.broadcast_to(np.asarray(v0[k], dtype=np.float64), (u0.shape[1],))
                     for k in v0_names]) if v0_names else None)
    name = "mparse_" + hashlib.sha256(code.encode()).hexdigest()[:16]
    m = SimInfModel(name, G, S, u0, tspan, v0=vv, ldata=ld, gdata=gvals, E=E, N=N,
                    events=events, replicates=replicates)
    m.C_code = code
    native.register_model_code(name, code, m.Nc, m.Nt, m.Nd, len(gdata_names))
    return m
