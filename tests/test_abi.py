"""CPU checks of the C ABI: the library builds for sm_103a, loads, exports
every entry point include/falcon_gpu.h declares, and its host-side logic
(defaults, namelist reader, argument validation) mirrors the reference."""
import ctypes
import os
import re

import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "falcon_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(falcon_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_step_boundary():
    names = declared_functions()
    for required in ("falcon_create", "falcon_step", "falcon_set_state", "falcon_get_state",
                     "falcon_diagnostics", "falcon_destroy", "falcon_batch_step",
                     "falcon_nonlin_dev", "falcon_getrs_batched_dev", "falcon_server_submit"):
        assert required in names


def test_library_exports_every_declared_symbol(fg):
    lib = fg.lib()
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(fg.EXPORTS) <= set(declared_functions())


def test_defaults_mirror_reference_namelists(fg):
    p = fg.default_params()  # src/namelists.F90:112-146
    assert (p.nr_max, p.nm_max) == (20, 20)
    assert p.eta == 0.35 and p.ra == 1000.0 and p.pr == 1.0
    assert p.mbc == 1 and p.lagpts == 14 and p.buo_imp == 1
    assert p.dt == 0.01 and p.n_time_steps == 100 and p.l_imexrk_started == 1
    assert (p.scheme_type, p.scheme_imp, p.scheme_exp) == (1, 13, 13)


def test_namelist_reader(fg, tmp_path):
    nml = tmp_path / "input.txt"
    nml.write_text("""&grid
Nr_max = 33 ! radial points
Nm_max = 42
/
&physics
eta = 0.35, Ra = 1.e5, Pr = 1.0, mBC = "NS", ampT = 0.001, lagpts = 16, n_init = 0
buo_tscheme="IMP"
/
&timecontrol
n_time_steps = 1000, dt = 0.00001, totaltime=100.0
l_vartimestep=.FALSE.
time_scheme_type = "IMEX", time_scheme_imp = "CN", time_scheme_exp = "AB2"
l_imexrk_started = .FALSE.
/
&output
tag="CNAB2", n_KE=10
/
""")
    p = fg.read_namelist(nml)
    assert (p.nr_max, p.nm_max) == (33, 42)
    assert p.ra == 1e5 and p.dt == 1e-5 and p.mbc == 0 and p.ampT == 0.001
    assert (p.scheme_type, p.scheme_imp, p.scheme_exp) == (0, 0, 0)
    assert p.l_vartimestep == 0 and p.l_imexrk_started == 0
    assert p.tag == b"CNAB2" and p.n_KE == 10


def test_namelist_errors_are_reported(fg, tmp_path):
    with pytest.raises(fg.FalconError):
        fg.read_namelist(tmp_path / "missing.txt")
    bad = tmp_path / "bad.txt"
    bad.write_text('&timecontrol\ntime_scheme_type="IMEX"\ntime_scheme_imp="XYZ"\n/\n')
    with pytest.raises(fg.FalconError, match="XYZ"):
        fg.read_namelist(bad)


def test_no_cpu_fallback_without_gpu(fg):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(fg.FalconError, match="no CPU fallback"):
        fg.Instance(fg.make_params(9, 4))


def test_process_wide_switches_round_trip(fg):
    # defaults: autotuned contraction paths, step graphs, groups of <= 128
    L = fg.lib()
    assert fg.set_gemm_mode(0) == 4 and fg.set_gemm_mode(1) == 0 and fg.set_gemm_mode(2) == 1
    assert fg.set_gemm_mode(3) == 2 and fg.set_gemm_mode(9) == 3   # unknown: autotuned
    assert fg.set_gemm_mode(4) == 4
    assert fg.set_max_group_size(64) == 128
    assert fg.set_max_group_size(-5) == 64      # negative means one group per key
    assert fg.set_max_group_size(128) == 0
    L.falcon_set_step_graphs.argtypes = [ctypes.c_int]
    assert L.falcon_set_step_graphs(0) == 1 and L.falcon_set_step_graphs(1) == 0


def test_namelist_reader_on_the_reference_input(fg):
    # the reference's own src/input.txt, copied verbatim by make_golden.py
    p = fg.read_namelist(os.path.join(ROOT, "tests", "golden", "input_reference.txt"))
    assert (p.nr_max, p.nm_max) == (32, 32)
    assert p.eta == 0.35 and p.ra == 2000.0 and p.pr == 1.0 and p.mbc == 0
    assert p.ampT == 0.01 and p.l_add_pert == 0 and p.lagpts == 16 and p.n_init == 0 and p.buo_imp == 1
    assert p.n_time_steps == 1000000 and p.dt == 1e-5 and p.totaltime == 100.0
    assert p.l_vartimestep == 1 and p.l_optimizedt == 0
    assert (p.scheme_type, p.scheme_imp, p.scheme_exp) == (1, 44, 44)   # IMEXRK BHR553 / expBHR553
    assert p.l_imexrk_started == 0
    assert p.dt_coef == 1.0 and p.dt_max == 1e-2 and p.cfl == 0.1
    assert (p.l_restart, p.n_restart, p.n_restart_point, p.n_snapshot_point) == (0, 0, 1, 0)
    assert p.tag == b"BHR553"
    assert (p.n_checkpoint, p.n_snapshot, p.n_KE, p.n_KEspec) == (10000, 100000, 10, 100000)
