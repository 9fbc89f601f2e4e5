"""IMEXRK Butcher tables (src/timeschemes.F90) shared by the library and the
oracle: every built table satisfies the order conditions of its scheme, the
namelist names map to them, and the schemes that are not built are refused
with a clear error.  The tables were also compared entry by entry with the
reference's own expressions evaluated in IEEE double (all equal)."""
import ctypes

import numpy as np
import pytest

ORDER = {"ARS443": 3, "ARS343": 3, "BPR353": 3, "ARS222": 2, "ARS232": 2, "ARS233": 3, "EUL111": 1,
         "MARS343": 3, "IJ3": 3, "PC2": 2, "SSP332": 2, "SSP543": 3, "PR433": 3, "DBM453": 3, "KC343": 3,
         "KC564": 3, "FW53": 3, "CK222": 2, "BPR442": 2, "CFN343": 3, "BHR553": 3, "CFN564": 3}
# (ars_eqn_check_D, ars_eqn_check_A): both true -> the stiffly accurate assembly
STIFFLY_ACCURATE = {"ARS443", "BPR353", "ARS222", "PC2", "SSP332", "SSP543", "FW53", "CK222", "BPR442"}


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
    flags = v[2 * n * n + 2 * n:]
    return aD, bD, aA, bA, flags


@pytest.mark.parametrize("name", sorted(ORDER))
def test_table_order_conditions(orc, name):
    aD, bD, aA, bA, flags = table(orc, name)
    p = ORDER[name]
    for A, b in ((aA, bA), (aD, bD)):
        c = A.sum(1)
        assert abs(b.sum() - 1.0) < 1e-13
        if p >= 2:
            assert abs(b @ c - 0.5) < 1e-13
        if p >= 3:
            assert abs(b @ c ** 2 - 1.0 / 3.0) < 1e-13 and abs(b @ (A @ c) - 1.0 / 6.0) < 1e-13
    assert np.allclose(np.triu(aA), 0.0)          # explicit table strictly lower triangular
    assert np.allclose(np.triu(aD, 1), 0.0)       # implicit table lower triangular
    assert (bool(flags[0]) and bool(flags[1])) == (name in STIFFLY_ACCURATE)


@pytest.mark.parametrize("name", sorted(ORDER))
def test_namelist_names_select_the_table(fg, name):
    p = fg.make_params(17, 8, name)
    assert p.scheme_type == 1 and p.scheme_imp == p.scheme_exp == fg.EXP["exp" + name]


@pytest.mark.parametrize("name", ["SMR333", "CB3e", "CB3f", "CB4", "LZ3L1", "LZ3A4a", "LZ4A1", "KC774", "KC885"])
def test_schemes_not_built_are_refused(fg, name):
    p = fg.default_params()
    fg.check(fg.lib().falcon_params_set_scheme(ctypes.byref(p), b"IMEXRK", name.encode(), ("exp" + name).encode()))
    h = ctypes.c_void_p()
    rc = fg.lib().falcon_create(ctypes.byref(p), ctypes.byref(h))
    assert rc == -1 and b"not supported" in fg.lib().falcon_last_error()
