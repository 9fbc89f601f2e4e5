"""The allocation-free nonlinear pass (falcon_nonlin_noalloc_dev).

Some hosts cannot let the library allocate device memory: they own every
byte through their own pre-sized pool (as the serving loop budgets HBM per
request) or step in loops where a cudaMalloc/cudaFree pair would
synchronise the device.  This entry point keeps its FFT tables in a fixed
static device array instead; it must give the same products as the
allocating entry point, call after call.  Collected last on purpose.
"""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


def _run(fg, fn, R, Nm, B, fields):
    import torch
    dev = [torch.from_numpy(np.ascontiguousarray(f).view(np.float64)).cuda() for f in fields]
    outs = [torch.empty_like(dev[0]) for _ in range(4)]
    fg.check(getattr(fg.lib(), fn)(R, Nm, B, *[d.data_ptr() for d in dev], *[o.data_ptr() for o in outs], None))
    torch.cuda.synchronize()
    return [o.cpu().numpy().view(np.complex128) for o in outs]


def test_noalloc_matches_allocating_entry_point_twice(fg):
    rng = np.random.default_rng(11)
    # two calls in a row with different sizes, so the second call's tables
    # overwrite the first call's in the shared scratch array
    for R, Nm, B in ((33, 42, 3), (65, 170, 2)):
        M = Nm + 1
        d = np.exp(-0.05 * np.arange(M))[None, :, None]
        fields = [(rng.standard_normal((R, M, B)) + 1j * rng.standard_normal((R, M, B))) * d for _ in range(4)]
        ref = _run(fg, "falcon_nonlin_dev", R, Nm, B, fields)
        got = _run(fg, "falcon_nonlin_noalloc_dev", R, Nm, B, fields)
        for g, r in zip(got, ref):
            assert rel(g, r) < 1e-13


def test_noalloc_rejects_sizes_beyond_the_scratch(fg):
    import torch
    x = torch.zeros(16, dtype=torch.float64, device="cuda")
    rc = fg.lib().falcon_nonlin_noalloc_dev(3, 1366, 1, *([x.data_ptr()] * 8), None)
    assert rc == -1
    assert b"4096" in fg.lib().falcon_last_error()
