"""The allocation-free nonlinear pass (falcon_nonlin_noalloc_dev).

Some hosts cannot let the library allocate device memory: they own every
byte through their own pre-sized pool (as the serving loop budgets HBM per
request) or step in loops where a cudaMalloc/cudaFree pair would
synchronise the device.  This entry point keeps its FFT tables in a fixed
static device array instead; it must give the same bits as the allocating
entry point, call after call, whatever size the previous call had, and
agree with the oracle.  It is asynchronous on its stream, so every call here
is followed by a synchronisation before the outputs are read.  Collected
last on purpose.
"""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


def _run(fg, fn, R, Nm, B, fields, stream=None):
    import torch
    dev = [torch.from_numpy(np.ascontiguousarray(f).view(np.float64)).cuda() for f in fields]
    outs = [torch.empty_like(dev[0]) for _ in range(4)]
    torch.cuda.synchronize()
    handle = stream.cuda_stream if stream is not None else None
    fg.check(getattr(fg.lib(), fn)(R, Nm, B, *[d.data_ptr() for d in dev], *[o.data_ptr() for o in outs], handle))
    if stream is not None:
        stream.synchronize()
    torch.cuda.synchronize()
    return [o.cpu().numpy().view(np.complex128) for o in outs]


def _fields(rng, R, Nm, B):
    M = Nm + 1
    d = np.exp(-0.05 * np.arange(M))[None, :, None]
    return [(rng.standard_normal((R, M, B)) + 1j * rng.standard_normal((R, M, B))) * d for _ in range(4)]


def test_noalloc_matches_allocating_entry_point_call_after_call(fg):
    import torch
    rng = np.random.default_rng(11)
    # a larger size after a smaller one (the second call's tables cover the
    # first's), then a smaller one after it (stale entries of the larger
    # tables stay beyond the region it uses), then the first size again on
    # a stream of its own
    cases = ((33, 42, 3, False), (65, 170, 2, False), (17, 10, 4, False), (33, 42, 3, True))
    for R, Nm, B, on_stream in cases:
        fields = _fields(rng, R, Nm, B)
        ref = _run(fg, "falcon_nonlin_dev", R, Nm, B, fields)
        got = _run(fg, "falcon_nonlin_noalloc_dev", R, Nm, B, fields,
                   stream=torch.cuda.Stream() if on_stream else None)
        for g, r in zip(got, ref):
            # same tables, same kernel: the same bits
            assert np.array_equal(g.view(np.float64), r.view(np.float64))


def test_noalloc_matches_the_oracle(fg, orc):
    rng = np.random.default_rng(12)
    R, Nm, B = 17, 10, 2
    fields = _fields(rng, R, Nm, B)
    got = _run(fg, "falcon_nonlin_noalloc_dev", R, Nm, B, fields)
    M = Nm + 1
    for b in range(B):
        ref = orc.nonlin(Nm, *[f[:, :, b] for f in fields])
        for g, r in zip(got, ref):
            assert rel(g.reshape(R, M, B)[:, :, b], r) < 1e-13


def test_noalloc_rejects_sizes_beyond_the_scratch(fg):
    import torch
    x = torch.zeros(16, dtype=torch.float64, device="cuda")
    rc = fg.lib().falcon_nonlin_noalloc_dev(3, 1366, 1, *([x.data_ptr()] * 8), None)
    assert rc == -1
    assert b"4096" in fg.lib().falcon_last_error()
