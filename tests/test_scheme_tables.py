"""IMEXRK Butcher tables (src/timeschemes.F90) shared by the library and the
oracle: every table equals, bit for bit, the reference's own expressions
evaluated in IEEE double (tests/golden/imexrk_tables.json, made by
tests/golden/make_imexrk_tables.py from the reference source), with the
reference's ars_eqn_check, diag_diff and diag_index flags; every table
satisfies the order conditions of its scheme; the namelist names map to
them; a mismatched implicit/explicit pair is refused."""
import ctypes
import json
import os

import numpy as np
import pytest

# order of the (implicit, explicit) tables; an int means both
ORDER = {"ARS443": 3, "ARS343": 3, "BPR353": 3, "ARS222": 2, "ARS232": 2, "ARS233": 3, "EUL111": 1,
         "MARS343": 3, "IJ3": 3, "PC2": 2, "SSP332": 2, "SSP543": 3, "PR433": 3, "DBM453": 3, "KC343": 3,
         "KC564": 3, "FW53": 3, "CK222": 2, "BPR442": 2, "CFN343": 3, "BHR553": 3, "CFN564": 3,
         "KC774": 4, "KC885": 5, "SMR333": (2, 3), "CB3e": 3, "CB3f": 3, "CB4": 4, "LZ3L1": 3, "LZ3A4a": 3,
         "LZ4A1": 4}
# (ars_eqn_check_D, ars_eqn_check_A): both true -> the stiffly accurate assembly
STIFFLY_ACCURATE = {"ARS443", "BPR353", "ARS222", "PC2", "SSP332", "SSP543", "FW53", "CK222", "BPR442",
                    "SMR333", "LZ3L1", "LZ3A4a", "LZ4A1"}
# the implicit diagonal varies by stage
DIAG_DIFF = {"SMR333", "CB3e", "CB3f", "CB4", "LZ3L1", "LZ3A4a", "LZ4A1"}
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "imexrk_tables.json")


def table(orc, name):
    L = orc.lib()
    L.orc_imexrk_table.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    out = (ctypes.c_double * 400)()
    sid = orc.EXP["exp" + name]
    assert L.orc_imexrk_table(sid, out) == 0
    n = int(out[0])
    v = np.array(out[1:2 * n * n + 2 * n + 4])
    aD, bD = v[:n * n].reshape(n, n), v[n * n:n * n + n]
    aA, bA = v[n * n + n:2 * n * n + n].reshape(n, n), v[2 * n * n + n:2 * n * n + 2 * n]
    flags = np.array(out[2 * n * n + 2 * n + 1:2 * n * n + 2 * n + 5])  # check_D, check_A, diag_index, diag_diff
    return aD, bD, aA, bA, flags


def order_residuals(A, b):
    """Residuals of the Butcher order conditions (rooted trees up to order 5)."""
    c = A.sum(1)
    Ac = A @ c
    return {1: [b.sum() - 1.0], 2: [b @ c - 0.5], 3: [b @ c ** 2 - 1 / 3, b @ Ac - 1 / 6],
            4: [b @ c ** 3 - 1 / 4, b @ (c * Ac) - 1 / 8, b @ (A @ c ** 2) - 1 / 12, b @ (A @ Ac) - 1 / 24],
            5: [b @ c ** 4 - 1 / 5, b @ (c ** 2 * Ac) - 1 / 10, b @ (c * (A @ c ** 2)) - 1 / 15,
                b @ (c * (A @ Ac)) - 1 / 30, b @ Ac ** 2 - 1 / 20, b @ (A @ c ** 3) - 1 / 20,
                b @ (A @ (c * Ac)) - 1 / 40, b @ (A @ (A @ c ** 2)) - 1 / 60, b @ (A @ (A @ Ac)) - 1 / 120]}


@pytest.mark.parametrize("name", sorted(ORDER))
def test_table_order_conditions(orc, name):
    aD, bD, aA, bA, flags = table(orc, name)
    pD, pA = ORDER[name] if isinstance(ORDER[name], tuple) else (ORDER[name], ORDER[name])
    for A, b, p in ((aA, bA, pA), (aD, bD, pD)):
        res = order_residuals(A, b)
        for k in range(1, p + 1):
            assert max(abs(x) for x in res[k]) < 1e-12, (k, res[k])
    assert np.allclose(np.triu(aA), 0.0)          # explicit table strictly lower triangular
    assert np.allclose(np.triu(aD, 1), 0.0)       # implicit table lower triangular
    assert (bool(flags[0]) and bool(flags[1])) == (name in STIFFLY_ACCURATE)
    assert bool(flags[3]) == (name in DIAG_DIFF)
    # FW53 and IJ3 have stage-dependent diagonals too, but the reference sets
    # diag_diff = .FALSE. for them (src/timeschemes.F90), so every stage
    # solves with the operators of stage diag_index; library and oracle
    # follow the flag.
    assert (len(set(np.diag(aD)[1:])) > 1) == (name in DIAG_DIFF | {"FW53", "IJ3"})


def test_golden_tables_cover_every_reference_pair():
    gold = json.load(open(GOLDEN))
    assert set(gold) == set(ORDER)
    assert all(not v["single_precision_literals"] for v in gold.values())


@pytest.mark.parametrize("name", sorted(ORDER))
def test_tables_equal_reference_expressions(orc, name):
    g = json.load(open(GOLDEN))[name]
    aD, bD, aA, bA, flags = table(orc, name)
    assert aD.shape == (g["n"], g["n"])
    for ours, ref in ((aD, g["aD"]), (bD, g["bD"]), (aA, g["aA"]), (bA, g["bA"])):
        assert np.array_equal(ours, np.array(ref, dtype=np.float64)), (ours, ref)  # bit for bit
    assert [bool(flags[0]), bool(flags[1]), int(flags[2]), bool(flags[3])] == \
        [g["check_D"], g["check_A"], g["diag_index"], g["diag_diff"]]


@pytest.mark.parametrize("name", sorted(ORDER))
def test_namelist_names_select_the_table(fg, name):
    p = fg.make_params(17, 8, name)
    assert p.scheme_type == 1 and p.scheme_imp == p.scheme_exp == fg.EXP["exp" + name]


@pytest.mark.parametrize("imp,exp", [("SMR333", "expKC885"), ("ARS443", "expARS343")])
def test_mismatched_pair_is_refused(fg, imp, exp):
    p = fg.default_params()
    fg.check(fg.lib().falcon_params_set_scheme(ctypes.byref(p), b"IMEXRK", imp.encode(), exp.encode()))
    h = ctypes.c_void_p()
    rc = fg.lib().falcon_create(ctypes.byref(p), ctypes.byref(h))
    assert rc == -1 and b"unsupported time scheme" in fg.lib().falcon_last_error()
