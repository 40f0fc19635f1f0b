"""Generate the golden fixtures in tests/golden/ from the reference's own R
test files.

The reference's tests need R, which is absent, so their RNG-free expected
values are lifted here into JSON fixtures: this script reads the literal
vectors out of the R sources (it does not run R) and pairs them with the
model inputs of the same test, transcribed below with the file:line they
come from.  Run it where the reference tree is available:

    python tests/golden/make_golden.py [/path/to/reference]

Fixtures written:
  sise_phi.json            tests/phi.R:33-108       SISe phi series (tol 1e-8)
  sir_zero_rates.json      tests/SIR.R:36-38,97-135 zero-rate SIR trajectory
  sise3_transfer_one.json  tests/sample_select.R:604-645  one E2 transfer, dense U
  sise3_transfer_three.json tests/sample_select.R:651-671 three moved, select S_1..S_3
  sise_punchcard_rep.json  tests/punchcard.R:364-410 replicates + sparse U/V
  individual_events.json   tests/individual_events.R:199-690,1222-1256 every
                           case that compares individual_events() with an
                           expected table (input and expected columns), and
                           :84-330 every literal table it must reject, with
                           the message
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def r_vector(text):
    """Parse the first R literal `c(...)` in text into a list of numbers."""
    i = text.index("c(")
    depth, j = 0, i + 1
    while True:
        ch = text[j]
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
            if depth == 0:
                break
        j += 1
    body = text[i + 2:j]
    out = []
    for tok in body.split(","):
        tok = tok.strip()
        if not tok:
            continue
        if tok.endswith("L"):
            out.append(int(tok[:-1]))
        else:
            out.append(float(tok))
    return out


def block(lines, start, end):
    return "\n".join(lines[start - 1:end])


def after(lines, start, pattern):
    """Text from the first line >= start matching pattern to the end."""
    for k in range(start - 1, len(lines)):
        if re.search(pattern, lines[k]):
            return "\n".join(lines[k:])
    raise ValueError("pattern %r not found after line %d" % (pattern, start))


def r_args(text):
    """Split the argument list of an R call (text from after its opening
    parenthesis) at top-level commas; returns (args, end index)."""
    args, depth, cur, quote, k = [], 0, "", None, 0
    while k < len(text):
        ch = text[k]
        if quote:
            cur += ch
            if ch == quote:
                quote = None
        elif ch in "\"'":
            quote = ch
            cur += ch
        elif ch == "(":
            depth += 1
            cur += ch
        elif ch == ")":
            if depth == 0:
                args.append(cur.strip())
                return [a for a in args if a], k
            depth -= 1
            cur += ch
        elif ch == "," and depth == 0:
            args.append(cur.strip())
            cur = ""
        else:
            cur += ch
        k += 1
    raise ValueError("unbalanced call")


def r_value(expr):
    """An R literal vector: c(...), a scalar, integer(0), as.Date(...).
    Returns a list of ints, floats, strings and None (NA)."""
    expr = expr.strip()
    if expr.startswith("as.Date("):
        inner, _ = r_args(expr[len("as.Date("):])
        return [{"date": v} for v in r_value(inner[0])]
    if expr == "integer(0)":
        return []
    if expr.startswith("c("):
        items, _ = r_args(expr[2:])
        return [x for it in items for x in r_value(it)]
    if expr in ("NA", "NA_integer_", "NA_character_", "NA_real_"):
        return [None]
    if expr in ("TRUE", "FALSE"):
        return [expr == "TRUE"]
    if expr[0] in "\"'":
        return [expr[1:-1]]
    if expr.endswith("L"):
        return [int(expr[:-1])]
    v = float(expr)
    return [int(v) if v == int(v) else v]


def r_data_frame(text):
    """Columns of data.frame(name = vector, ...) starting at text."""
    i = text.index("data.frame(") + len("data.frame(")
    args, _ = r_args(text[i:])
    out = {}
    for a in args:
        name, expr = a.split("=", 1)
        out[name.strip()] = r_value(expr)
    return out


def individual_event_cases(lines, first, last):
    """(line, input, expected) for each check of individual_events()
    against an expected table in lines [first, last]."""
    cases, events, expected, called = [], None, None, False
    k = first - 1
    while k < last:
        line = lines[k]
        m = re.match(r"^(events|events_exp|events_expected) <- data.frame\(", line)
        if m:
            df = r_data_frame("\n".join(lines[k:k + 40]))
            if m.group(1) == "events":
                events, expected, called = (df, None, False)
            else:
                expected = df
        elif "individual_events(events)" in line and "u0_from" not in line:
            called = True
        if events is not None and called and set(events) == {"id", "event", "time",
                                                             "node", "dest"}:
            if re.match(r"^stopifnot\(identical\((events_obs|events_observed), "
                        r"(events_exp|events_expected)\)\)", line) and expected:
                cases.append({"line": k + 1, "input": events, "expected": expected})
            elif re.match(r"^stopifnot\(identical\((events_obs, events|events, "
                          r"as.data.frame\(individual_events\(events\)\))\)\)", line):
                cases.append({"line": k + 1, "input": events, "expected": events})
        k += 1
    return cases


def individual_event_errors(lines, first, last):
    """(line, input, message) for each data.frame that individual_events()
    must reject with a message, in lines [first, last]."""
    cases, events = [], None
    k = first - 1
    while k < last:
        line = lines[k]
        if line.startswith("events <- data.frame("):
            events = r_data_frame("\n".join(lines[k:k + 40]))
        elif line.startswith("events$"):
            events = None                     # modified in place: not a literal table
        elif line.startswith("res <- assertError(individual_events(events))") and events:
            text = "\n".join(lines[k + 1:k + 6])
            m = re.search(r'check_error\(\s*res,\s*"((?:[^"\\]|\\.)*)"', text)
            if m:
                cases.append({"line": k + 1, "input": events, "message": m.group(1)})
        k += 1
    return cases


def main(ref):
    tests = os.path.join(ref, "tests")

    def read(name):
        with open(os.path.join(tests, name)) as f:
            return f.read().split("\n")

    fixtures = {}

    # tests/phi.R: SISe with no transitions; phi follows the post time step.
    phi = read("phi.R")
    fixtures["sise_phi.json"] = {
        "source": "tests/phi.R:33-108",
        "model": "SISe",
        "u0": {"S": [100], "I": [0]},
        "tspan": list(range(1, 701, 7)),
        "params": {"phi": 1.0, "upsilon": 0.0, "gamma": 0.0, "alpha": 0.0,
                   "beta_t1": 0.19, "beta_t2": 0.085, "beta_t3": 0.075, "beta_t4": 0.185,
                   "end_t1": 91, "end_t2": 182, "end_t3": 273, "end_t4": 365,
                   "epsilon": 0.000011},
        "phi_expected": r_vector(after(phi, 30, r"^phi_exp <- c\(")),
        "tol": 1e-8,
    }

    # tests/SIR.R: zero rates, u0 S = 0..5, tspan 0..9.
    sir = read("SIR.R")
    fixtures["sir_zero_rates.json"] = {
        "source": "tests/SIR.R:36-38,97-135",
        "model": "SIR",
        "u0": {"S": [0, 1, 2, 3, 4, 5], "I": [0] * 6, "R": [0] * 6},
        "tspan": list(range(0, 10)),
        "params": {"beta": 0.0, "gamma": 0.0},
        "S_expected": r_vector(after(sir, 90, r"^S_expected <- structure\(")),
        "I_expected": r_vector(after(sir, 90, r"^I_expected <- structure\(")),
        "R_expected": r_vector(after(sir, 90, r"^R_expected <- structure\(")),
        "dim": [6, 10],
    }

    ss = read("sample_select.R")
    sise3_zero = {"upsilon_1": 0, "upsilon_2": 0, "upsilon_3": 0, "gamma_1": 1,
                  "gamma_2": 1, "gamma_3": 1, "alpha": 0, "beta_t1": 1, "beta_t2": 1,
                  "beta_t3": 1, "beta_t4": 1, "end_t1": 91, "end_t2": 182, "end_t3": 273,
                  "end_t4": 365, "epsilon": 0}
    fixtures["sise3_transfer_one.json"] = {
        "source": "tests/sample_select.R:604-645",
        "model": "SISe3",
        "u0": {"S_1": [0, 2], "I_1": [0, 0], "S_2": [0, 0], "I_2": [0, 0],
               "S_3": [0, 0], "I_3": [0, 0]},
        "tspan": list(range(0, 11)),
        "phi": [0.0, 0.0],
        "params": sise3_zero,
        "events": {"event": [3], "time": [1], "node": [2], "dest": [1], "n": [1],
                   "proportion": [0.0], "select": [1], "shift": [0]},
        "U_expected": r_vector(after(ss, 620, r"^U <- structure\(")),
        "dim": [12, 11],
    }
    fixtures["sise3_transfer_three.json"] = {
        "source": "tests/sample_select.R:651-671",
        "model": "SISe3",
        "u0": {"S_1": [0, 2], "I_1": [0, 0], "S_2": [0, 2], "I_2": [0, 0],
               "S_3": [0, 2], "I_3": [0, 0]},
        "tspan": list(range(0, 11)),
        "phi": [0.0, 0.0],
        "params": sise3_zero,
        "events": {"event": [3], "time": [1], "node": [2], "dest": [1], "n": [3],
                   "proportion": [0.0], "select": [1], "shift": [0]},
        "E_extra": [[2, 0], [4, 0]],
        "S_sum_node1_expected": r_vector(after(ss, 690, r"^S_expected <- c\(")),
    }

    pc = read("punchcard.R")
    fixtures["sise_punchcard_rep.json"] = {
        "source": "tests/punchcard.R:364-410",
        "model": "SISe",
        "u0": {"S": [101, 102, 103, 104, 105, 106], "I": [1, 2, 3, 4, 5, 6]},
        "phi": [0.1, 0.2, 0.3, 0.4, 0.5, 0.6],
        "tspan": list(range(1, 11)),
        "replicates": 2,
        "Nn": 3,
        "params": {"upsilon": 0, "gamma": 0, "alpha": 0, "epsilon": 0, "beta_t1": 0,
                   "beta_t2": 0, "beta_t3": 0, "beta_t4": 0, "end_t1": 91, "end_t2": 182,
                   "end_t3": 273, "end_t4": 365},
        "U_i": r_vector(after(pc, 380, r"^i <- c\(1, 6")),
        "U_j": r_vector(after(pc, 380, r"^j <- c\(1, 1, 2")),
        "V_i": r_vector(after(pc, 380, r"^i <- c\(1, 3")),
        "V_j": r_vector(after(pc, 388, r"^j <- c\(1, 2, 3")),
        "U_x_expected": r_vector(after(pc, 395, r"stopifnot\(identical\(")),
        "V_x_expected": r_vector(after(pc, 400, r"result@V_sparse@x - c\(").replace(
            "stopifnot(all(abs(result@V_sparse@x - ", "")),
        "tol": 1e-8,
    }

    # tests/ldata_sp.R: the distance matrix of (1..10, 1..10) with cutoff 3
    # and the spatial ldata (end_t1..end_t4, then neighbour pairs) packed
    # with each metric.
    ls = read("ldata_sp.R")
    fixtures["ldata_sp.json"] = {
        "source": "tests/ldata_sp.R:34-66,147-226",
        "x": list(range(1, 11)), "y": list(range(1, 11)), "cutoff": 3,
        "end_t": [91, 182, 273, 365],
        "d_i": r_vector(after(ls, 40, r"^d <- new\(")),
        "d_p": r_vector(after(ls, 40, r"^\s+p = c\(")),
        "d_x": r_vector(after(ls, 40, r"^\s+x = c\(")),
        "ldata_degree": r_vector(after(ls, 145, r"^ldata_exp <- structure\(")),
        "ldata_distance": r_vector(after(ls, 160, r"^ldata_exp <- structure\(")),
        "ldata_inverse_square": r_vector(after(ls, 196, r"^ldata_exp <- structure\(")),
        "dim": [14, 10],
        "tol": 1e-8,
    }

    ie = read("individual_events.R")
    fixtures["individual_events.json"] = {
        "source": "tests/individual_events.R:199-690,1222-1256",
        "cases": individual_event_cases(ie, 199, 690) + individual_event_cases(ie, 1222, 1256),
        "errors": individual_event_errors(ie, 84, 330),
    }

    for name, fx in fixtures.items():
        with open(os.path.join(HERE, name), "w") as f:
            json.dump(fx, f, indent=1)
        print("wrote", name)


if __name__ == "__main__":
    if len(sys.argv) < 2 and not os.environ.get("SIMINF_REFERENCE"):
        sys.exit("usage: make_golden.py REFERENCE_TREE (or set SIMINF_REFERENCE)")
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ["SIMINF_REFERENCE"])
