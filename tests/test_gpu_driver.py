"""The drop-in driver falcon_run (falcon-dns_gb300/driver/falcon_run.cpp) on
the plain reference run's configuration (Nr=33, Ntheta=128 -> Nm=42,
CNAB2, dt=1e-5, Ra=1e5, seeded noise 1e-3), 100 steps: it reads a namelist
in the reference's input.txt syntax and writes KE_<tag>, Nusselt_<tag>,
power_<tag>, upbalance_<tag> every n_KE = 10 steps and KEspec_<tag>,
Temp_spec_<tag> every n_KEspec = 50 steps (src/output.F90:30-51,122-355,
src/steptime.F90:255-293).  Every file's format (Fortran ES20.12 / I8
fields, line counts) and every number against the oracle at the same
steps."""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import PKG

pytestmark = pytest.mark.gpu

NAMELIST = """&grid
Nr_max = 33 ! radial points
Nm_max = 42  ! azimuthal modes (Ntheta = 128)
/
&physics
eta = 0.35,
Ra = 1.0e5,
Pr = 1.0,
mBC = "NS",
ampT = 0.001,
l_add_pert = .FALSE.
lagpts = 16,
n_init = 0
buo_tscheme="IMP"
/
&timecontrol
n_time_steps = 100,
dt = 0.00001
totaltime=100.0
l_vartimestep=.FALSE.
l_optimizedt=.FALSE.
time_scheme_type = "IMEX"
time_scheme_imp = "CN",
time_scheme_exp = "AB2",
l_imexrk_started = .FALSE.
dt_coef=1.0,
dt_max=1.e-2
CFL=0.1,
l_restart=.FALSE.,
n_restart=0,
n_restart_point=0,
n_snapshot_point=0
/
&output
tag="cfg1"
n_checkpoint=1000000,
n_snapshot=1000000,
n_KE=10,
n_KEspec=50
/
"""

ES = re.compile(r"^ +-?\d\.\d{12}E[+-]\d\d$")


def fields(line, widths):
    out, pos = [], 0
    for w in widths:
        out.append(line[pos:pos + w])
        pos += w
    assert pos == len(line), line
    return out


def read_es(path, ncol):
    rows = []
    for line in open(path).read().splitlines():
        f = fields(line, [20] * ncol)
        assert all(ES.match(x) for x in f), line
        rows.append([float(x) for x in f])
    return np.array(rows)


def read_spec(path):
    rows = []
    for line in open(path).read().splitlines():
        a, b, c = fields(line, [8, 8, 20])
        assert re.match(r"^ *\d+$", a) and re.match(r"^ *\d+$", b) and ES.match(c), line
        rows.append((int(a), int(b), float(c)))
    return rows


def close(a, b, tol, floor=0.0):
    return abs(a - b) <= tol * max(abs(b), floor)


@pytest.fixture(scope="module")
def run_dir(fg, tmp_path_factory):
    d = tmp_path_factory.mktemp("cfg1")
    (d / "input.txt").write_text(NAMELIST)
    exe = os.path.join(PKG, "_build", "falcon_run")
    r = subprocess.run([exe, "input.txt", "--noise", "1", "0.001"], cwd=d, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    return d, r.stdout


def test_driver_files_match_oracle(run_dir, orc):
    d, stdout = run_dir
    ke = read_es(d / "KE_cfg1", 6)
    nu = read_es(d / "Nusselt_cfg1", 3)
    pw = read_es(d / "power_cfg1", 3)
    ub = read_es(d / "upbalance_cfg1", 4)
    ks = read_spec(d / "KEspec_cfg1")
    ts = read_spec(d / "Temp_spec_cfg1")
    assert ke.shape == (10, 6) and nu.shape == (10, 3) and pw.shape == (10, 3)
    assert ub.shape == (10 * 33, 4)
    assert len(ks) == 2 * 43 and len(ts) == 2 * 43
    assert len(stdout.splitlines()) == 10
    o = orc.Sim(orc.make_params(33, 42, "CNAB2", ra=1e5, dt=1e-5, pr=1.0))
    o.init_noise(1, 1e-3)
    for j in range(10):
        o.step(10)
        dg = o.diagnostics()
        assert ke[j, 0] == 1e-5
        assert close(ke[j, 1], dg["time"], 1e-13)
        for c, k in ((2, "KE"), (3, "KE_r"), (4, "KE_phi")):
            assert close(ke[j, c], dg[k], 1e-9), (j, k)
        assert close(ke[j, 5], dg["KE_upbar"], 1e-8, floor=1e-12 * dg["KE"])
        assert close(nu[j, 1], dg["Nu_top"], 1e-10) and close(nu[j, 2], dg["Nu_bot"], 1e-10)
        assert close(pw[j, 1], dg["vis"], 1e-9) and close(pw[j, 2], dg["buo"], 1e-9)
        ref = o.upbalance()
        blk = ub[33 * j:33 * (j + 1)]
        for c in range(4):
            scale = max(np.abs(ref[:, c]).max(), 1e-300)
            assert np.abs(blk[:, c] - ref[:, c]).max() <= 1e-8 * scale, (j, c)
        if (j + 1) % 5 == 0:
            kr, tr = o.spectra()
            base = 43 * ((j + 1) // 5 - 1)
            for m in range(43):
                assert ks[base + m][:2] == (10 * (j + 1), m) and ts[base + m][:2] == (10 * (j + 1), m)
                assert close(ks[base + m][2], kr[m], 1e-9, floor=1e-12 * kr.max()), m
                assert close(ts[base + m][2], tr[m], 1e-9, floor=1e-12 * tr.max()), m
