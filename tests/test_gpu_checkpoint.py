"""Checkpoint and snapshot files from the GPU (store_checkpoint /
store_snapshot layouts, src/output.F90:359-516) against the oracle's, and
restart from a checkpoint continuing bit for bit."""
import numpy as np
import pytest

from conftest import rel
from test_checkpoint_format import parse_checkpoint, parse_snapshot

pytestmark = pytest.mark.gpu

TOL = 1e-10
FIELDS = ("T", "omg", "up", "ur", "psi")


@pytest.mark.parametrize("scheme", ["SBDF3", "CNAB2", "SBDF4", "ARS443", "RK4"])
def test_checkpoint_file_matches_oracle(orc, fg, tmp_path, scheme):
    R, Nm, nsteps = 17, 8, 20
    M = Nm + 1
    dt = 1e-6 if scheme == "RK4" else 1e-5
    g = fg.Instance(fg.make_params(R, Nm, scheme, ra=1e4, dt=dt))
    o = orc.Sim(orc.make_params(R, Nm, scheme, ra=1e4, dt=dt))
    g.init_noise(4)
    o.init_noise(4)
    g.step(nsteps)
    o.step(nsteps)
    fg_path, fo_path = tmp_path / "gpu_ckpt", tmp_path / "orc_ckpt"
    g.store_checkpoint(str(fg_path))
    o.store_checkpoint(str(fo_path))
    a, b = parse_checkpoint(str(fg_path), R, M), parse_checkpoint(str(fo_path), R, M)
    for k in ("nm", "nr", "ni", "ne", "nmax", "dt", "time"):
        assert a[k] == b[k], k
    assert np.array_equal(a["dt_array"], b["dt_array"])
    for k in ("T", "omg", "ur", "up"):
        assert rel(a[k], b[k]) < TOL, k
    multistep = scheme.startswith("SBDF") or scheme.startswith("CN")
    for k in ("imp_T", "exp_T", "imp_omg", "exp_omg", "imp_u", "exp_u"):
        assert a[k].shape == b[k].shape, k
        x, y = a[k], b[k]
        if multistep and k.startswith("imp"):
            # the oldest implicit level is not kept on the device (shifted out unused)
            assert np.all(x[..., -1] == 0)
            x, y = x[..., :-1], y[..., :-1]
        if np.linalg.norm(y) == 0:
            assert np.linalg.norm(x) == 0, k
        else:
            assert rel(x, y) < TOL, k


# variable dt: settings under which dt changes every step (operators rebuilt
# every step), so that the restored run and the uninterrupted one rebuild alike.
# Not stiffly accurate IMEXRK schemes take the CFL step from a nonlinear pass
# on the assembled state in both runs.  Stiffly accurate ones take it from
# the last nonlinear pass of the previous step, which the restored run does
# not have; like the reference (src/steptime_imexrk.F90:109-117) it runs a
# pass on the restored state instead, so those runs are not compared here.
VARDT = dict(ra=1e6, vartimestep=True, cfl=0.02, dt_coef=1.5, dt_max=1e-4)


@pytest.mark.parametrize("scheme,vardt", [("SBDF3", False), ("CNAB2", False), ("CNAB3", False), ("SBDF4", False),
                                          ("ARS443", False), ("ARS343", False), ("RK4", False),
                                          ("SBDF3", True), ("ARS343", True), ("CB4", False), ("SMR333", False),
                                          ("CB3f", True)])
def test_restart_continues_bit_for_bit(fg, tmp_path, scheme, vardt):
    R, Nm = 17, 8
    kw = dict(ra=1e5, dt=1e-6 if scheme.startswith("RK") else 1e-5)
    amp = 1e-2
    if vardt:
        kw.update(VARDT)
        amp = 1e-1
    p = fg.make_params(R, Nm, scheme, **kw)
    a = fg.Instance(p)
    a.init_noise(5, amp)
    a.step(12)
    path = tmp_path / "checkpoint_00001"
    a.store_checkpoint(str(path))
    a.step(9)
    b = fg.Instance(p)
    b.init_noise(99, amp)  # overwritten by the load
    b.load_checkpoint(str(path))
    b.step(9)
    sa, sb = a.get_state(), b.get_state()
    for f in FIELDS:
        assert np.array_equal(sa[f], sb[f]), f
    da, db = a.diagnostics(), b.diagnostics()
    assert da["time"] == db["time"] and da["dt"] == db["dt"]


def test_snapshot_file_matches_oracle(orc, fg, tmp_path):
    R, Nm = 17, 8
    g = fg.Instance(fg.make_params(R, Nm, "CNAB2", ra=3e4, pr=0.7, dt=1e-5))
    o = orc.Sim(orc.make_params(R, Nm, "CNAB2", ra=3e4, pr=0.7, dt=1e-5))
    g.init_noise(6)
    o.init_noise(6)
    g.step(15)
    o.step(15)
    g.store_snapshot(str(tmp_path / "g"))
    o.store_snapshot(str(tmp_path / "o"))
    a, b = parse_snapshot(str(tmp_path / "g"), R, Nm + 1), parse_snapshot(str(tmp_path / "o"), R, Nm + 1)
    for k in ("ra", "pr", "eta", "dt", "time", "nm", "nr"):
        assert a[k] == b[k], k
    assert np.array_equal(a["radius"], b["radius"])
    for k in ("T", "omg", "ur", "up"):
        assert rel(a[k], b[k]) < TOL, k


def test_checkpoint_of_another_grid_is_refused(fg, tmp_path):
    a = fg.Instance(fg.make_params(17, 8, "SBDF3", ra=1e4, dt=1e-5))
    a.init_noise(1)
    a.step(3)
    a.store_checkpoint(str(tmp_path / "c"))
    b = fg.Instance(fg.make_params(17, 10, "SBDF3", ra=1e4, dt=1e-5))
    with pytest.raises(fg.FalconError, match="grid"):
        b.load_checkpoint(str(tmp_path / "c"))
