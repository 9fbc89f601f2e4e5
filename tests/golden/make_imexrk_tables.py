"""Generate tests/golden/imexrk_tables.json: every IMEXRK Butcher pair of the
reference evaluated in IEEE double from its own Fortran source.

Run where the FAlCon-DNS reference tree is available, with the environment
variable FALCON_REFERENCE naming its root (the directory holding src/ and
python/).  The script reads
src/timeschemes.F90 as text (nothing of the reference is executed):

  init_time_schemes      (:37-973)    the named constants of each scheme
                                      (alpha1 = 29.0_dp/96.0_dp, ...)
  rhs_update_wts_imp     (:993-1612)  butcher_aD, butcher_bD,
                                      ars_eqn_check_D, diag_diff, diag_index
  rhs_update_wts_exp     (:1614-2388) butcher_aA, butcher_bA, ars_eqn_check_A

and the named parameters of src/constants.F90:7-27 (onethird, ...).

Expressions are evaluated with the Fortran rules that matter here: a
literal with the _dp kind is a double, one without it a default (single
precision) real, so mixed arithmetic is emulated with numpy float32/float64
(the reference's tables carry _dp on every literal; the check records any
that do not).  ars_eqn_check_* set inside the reference's
"do i=1,n; if (butcher_a(n,i)==butcher_b(i)) ... = .TRUE." loop is
evaluated the same way: true when any last-row entry equals b.

Output: {scheme: {n, aD, bD, aA, bA, check_D, check_A, diag_diff,
diag_index}} with the numbers written by repr (round-trips exactly).
"""
import json
import os
import re

import numpy as np

REF = os.environ.get("FALCON_REFERENCE")
if not REF or not os.path.isdir(os.path.join(REF, "src")):
    raise SystemExit("set FALCON_REFERENCE to the root of the FAlCon-DNS source tree")
HERE = os.path.dirname(os.path.abspath(__file__))

IDENT = re.compile(r"(?<![\w.])([A-Za-z]\w*)")
NUM = re.compile(r"(?<![\w.])(\d+\.\d*(?:[eEdD][+-]?\d+)?|\d*\.\d+(?:[eEdD][+-]?\d+)?|\d+)(_dp)?")


def logical_lines(lines):
    """Strip comments, join '&' continuations."""
    out, cur = [], ""
    for raw in lines:
        s = raw.split("!", 1)[0].rstrip()
        t = s.strip()
        if t.startswith("&"):
            t = t[1:].strip()
        if t.endswith("&"):
            cur += " " + t[:-1]
            continue
        cur += " " + t
        if cur.strip():
            out.append(cur.strip())
        cur = ""
    return out


def subroutine(src, name):
    lo = next(i for i, l in enumerate(src) if re.match(r"\s*subroutine\s+%s\b" % name, l))
    hi = next(i for i, l in enumerate(src) if re.match(r"\s*end\s+subroutine\s+%s\b" % name, l))
    return src[lo:hi + 1]


def case_blocks(lines):
    """label -> logical lines up to the next case label or end select."""
    blocks, label = {}, None
    for l in logical_lines(lines):
        m = re.match(r"case\s*\('([^']+)'\)", l, re.I)
        if m:
            label = m.group(1)
            blocks.setdefault(label, [])
            continue
        if re.match(r"(end\s*select|select\s+case)", l, re.I):
            label = None
            continue
        if label is not None:
            blocks[label].append(l)
    return blocks


class Evaluator:
    def __init__(self):
        self.env = {}
        self.single = []

    def value(self, expr):
        def lit(m):
            text, dp = m.group(1), m.group(2)
            if "." not in text and "e" not in text.lower() and "d" not in text.lower():
                return "int(%s)" % text
            text = text.lower().replace("d", "e")
            if dp:
                return "np.float64(%r)" % float(text)
            self.single.append(m.group(0))
            return "np.float32(%r)" % float(text)
        def ident(m):
            name = m.group(1).lower()
            return name if name == "sqrt" else "V[%r]" % name
        py = NUM.sub(lit, IDENT.sub(ident, expr))
        return eval(py, {"np": np, "int": int, "sqrt": np.sqrt, "V": self.env, "__builtins__": {}})

    def array(self, body):
        items, depth, cur = [], 0, ""
        for ch in body:
            if ch == "(":
                depth += 1
            elif ch == ")":
                depth -= 1
            if ch == "," and depth == 0:
                items.append(cur)
                cur = ""
            else:
                cur += ch
        items.append(cur)
        return [float(np.float64(self.value(x.strip()))) for x in items if x.strip()]


def reshape_body(stmt):
    m = re.search(r"reshape\s*\(\s*\[(.*?)\]\s*,\s*\[([\d,\s]+)\]", stmt, re.I)
    return m.group(1), [int(v) for v in m.group(2).split(",")]


def table(ev, block, a_name, b_name, check_name):
    a = b = None
    check = None
    diag_diff = diag_index = None
    loop_check = False
    for l in block:
        low = l.lower().replace(" ", "")
        if low.startswith(a_name.lower() + "="):
            body, shape = reshape_body(l)
            v = ev.array(body)
            n = shape[0]
            a = [v[i * n:(i + 1) * n] for i in range(n)]   # order=[2,1]: row-major
        elif low.startswith(b_name.lower() + "="):
            body, _ = reshape_body(l)
            b = ev.array(body)
        elif low.startswith("if(%s(" % a_name.lower()) and "==%s(" % b_name.lower() in low:
            loop_check = True
        elif low.startswith(check_name.lower() + "="):
            if not loop_check:
                check = low.endswith(".true.")
        elif low.startswith("diag_diff="):
            diag_diff = low.endswith(".true.")
        elif low.startswith("diag_index="):
            diag_index = int(low.split("=")[1])
    if loop_check:
        n = len(b)
        check = any(a[n - 1][i] == b[i] for i in range(n))
    return a, b, bool(check), diag_diff, diag_index


def main():
    src = open(os.path.join(REF, "src", "timeschemes.F90")).read().split("\n")
    init = case_blocks(subroutine(src, "init_time_schemes"))
    imp = case_blocks(subroutine(src, "rhs_update_wts_imp"))
    exp = case_blocks(subroutine(src, "rhs_update_wts_exp"))
    # the named parameters of src/constants.F90 used by the tables (onethird, ...)
    consts, cev = {}, Evaluator()
    for l in logical_lines(open(os.path.join(REF, "src", "constants.F90")).read().split("\n")):
        m = re.match(r"real\(kind=dp\),\s*parameter\s*::\s*(\w+)\s*=\s*(.+)$", l, re.I)
        if m and "atan" not in m.group(2):
            consts[m.group(1).lower()] = cev.value(m.group(2))
    out = {}
    for name, block in imp.items():
        if "butcher_aD" not in " ".join(block) or ("exp" + name) not in exp:
            continue
        ev = Evaluator()
        ev.env.update(consts)
        for l in init.get(name, []) + init.get("exp" + name, []):
            m = re.match(r"([A-Za-z]\w*)\s*=\s*(.+)$", l)
            if m and not m.group(1).lower().startswith(("n_order", "rhs_", "wt_", "butcher")) \
                    and "(" not in m.group(1):
                ev.env[m.group(1).lower()] = ev.value(m.group(2))
        aD, bD, cD, dd, di = table(ev, block, "butcher_aD", "butcher_bD", "ars_eqn_check_D")
        aA, bA, cA, _, _ = table(ev, exp["exp" + name], "butcher_aA", "butcher_bA", "ars_eqn_check_A")
        assert len(aD) == len(aA) == len(bD) == len(bA), name
        out[name] = {"n": len(bD), "aD": aD, "bD": bD, "aA": aA, "bA": bA, "check_D": cD, "check_A": cA,
                     "diag_diff": bool(dd), "diag_index": di, "single_precision_literals": ev.single}
    path = os.path.join(HERE, "imexrk_tables.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)
    print("wrote %s: %d schemes" % (path, len(out)))


if __name__ == "__main__":
    main()
