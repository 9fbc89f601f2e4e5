"""The oracle's checkpoint and snapshot files follow store_checkpoint /
store_snapshot (src/output.F90:359-516): Fortran unformatted sequential
records (4-byte length, data, 4-byte length) in the reference's order and
shapes, with the multistep histories as the reference keeps them."""
import numpy as np


def read_records(path):
    data = open(path, "rb").read()
    recs, i = [], 0
    while i < len(data):
        n = int(np.frombuffer(data[i:i + 4], np.int32)[0])
        recs.append(data[i + 4:i + 4 + n])
        assert int(np.frombuffer(data[i + 4 + n:i + 8 + n], np.int32)[0]) == n
        i += 8 + n
    return recs


def parse_checkpoint(path, R, M):
    recs = read_records(path)
    assert len(recs) == 12
    dt, t = np.frombuffer(recs[0][:16], np.float64)
    nm, nr, ni, ne, nmax = np.frombuffer(recs[0][16:], np.int32)
    out = dict(dt=dt, time=t, nm=nm, nr=nr, ni=ni, ne=ne, nmax=nmax,
               dt_array=np.frombuffer(recs[1], np.float64))
    for k, name in enumerate(("T", "omg", "ur", "up")):
        out[name] = np.frombuffer(recs[2 + k], np.complex128).reshape(R, M)
    for k, name in enumerate(("imp_T", "exp_T", "imp_omg", "exp_omg")):
        a = np.frombuffer(recs[6 + k], np.complex128)
        out[name] = a.reshape(R, M, a.size // (R * M))  # (order, M, R) Fortran -> [r][m][order]
    for k, name in enumerate(("imp_u", "exp_u")):
        a = np.frombuffer(recs[10 + k], np.complex128)
        out[name] = a.reshape(R, a.size // R)
    return out


def parse_snapshot(path, R, M):
    recs = read_records(path)
    assert len(recs) == 8
    ra, pr, eta = np.frombuffer(recs[0], np.float64)
    dt, t = np.frombuffer(recs[1], np.float64)
    nm, nr = np.frombuffer(recs[2], np.int32)
    out = dict(ra=ra, pr=pr, eta=eta, dt=dt, time=t, nm=nm, nr=nr, radius=np.frombuffer(recs[3], np.float64))
    for k, name in enumerate(("T", "omg", "ur", "up")):
        out[name] = np.frombuffer(recs[4 + k], np.complex128).reshape(R, M)
    return out


def test_oracle_checkpoint_layout(orc, tmp_path):
    R, Nm = 9, 4
    M = Nm + 1
    o = orc.Sim(orc.make_params(R, Nm, "SBDF3", ra=1e4, dt=1e-4))
    o.init_noise(1, 1e-2)
    states = []
    for k in range(5):
        states.append(o.get_state())
        o.step(1)
    f = tmp_path / "checkpoint_00001"
    o.store_checkpoint(str(f))
    c = parse_checkpoint(str(f), R, M)
    assert (c["nm"], c["nr"], c["ni"], c["ne"], c["nmax"]) == (Nm, R, 3, 3, 3)
    assert c["dt"] == 1e-4 and np.all(c["dt_array"] == 1e-4)
    assert abs(c["time"] - 5e-4) < 1e-15
    s = o.get_state()
    for k in ("T", "omg", "ur", "up"):
        assert np.array_equal(c[k], s[k])
    # rhs_imp_temp(io): the temperature io steps before the current one
    # (the vorticity histories hold modes m >= 1 only: mode 0 is the uphi_bar equation)
    for io in range(3):
        assert np.allclose(c["imp_T"][:, :, io], states[4 - io]["T"], rtol=0, atol=1e-14)
        assert np.allclose(c["imp_omg"][:, 1:, io], states[4 - io]["omg"][:, 1:], rtol=0, atol=1e-14)
        assert np.all(c["imp_omg"][:, 0, io] == 0) and np.all(c["exp_omg"][:, 0, io] == 0)
    assert np.allclose(c["imp_u"][:, 0], states[4]["up"][:, 0], atol=1e-14)


def test_oracle_snapshot_layout(orc, tmp_path):
    R, Nm = 9, 4
    o = orc.Sim(orc.make_params(R, Nm, "CNAB2", ra=2e4, pr=0.7, dt=1e-4))
    o.init_noise(2, 1e-2)
    o.step(3)
    f = tmp_path / "snapshot_plot_00001"
    o.store_snapshot(str(f))
    c = parse_snapshot(str(f), R, Nm + 1)
    assert (c["ra"], c["pr"], c["eta"]) == (2e4, 0.7, 0.35)
    assert (c["nm"], c["nr"]) == (Nm, R) and abs(c["time"] - 3e-4) < 1e-15
    rmin = 0.35 / 0.65
    assert np.allclose(c["radius"], rmin + 0.5 * (1 + np.cos((R - 1 - np.arange(R)) * np.pi / (R - 1))))
    s = o.get_state()
    for k in ("T", "omg", "ur", "up"):
        assert np.array_equal(c[k], s[k])
