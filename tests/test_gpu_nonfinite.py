"""A non-finite value in one instance's state is reported by the batch's
diagnostics (FALCON_ENONFINITE, the reference's own guard is on KE) and does
not reach the other instances of the batch: every contraction, transform and
slice exponent works per instance column, on the tensor-core paths (Inf or
NaN columns give NaN) as on the FP64 ones."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("gemm_mode", [1, 3, 0])
def test_nonfinite_instance_is_reported_and_isolated(fg, gemm_mode):
    n, bad = 20, 7
    prev = fg.set_gemm_mode(gemm_mode)
    try:
        ps = [fg.make_params(65, 42, "SBDF3", ra=1e5 * (1 + 0.05 * k), dt=1e-5) for k in range(n)]
        b = fg.Batch(ps)
        b.init_noise(list(range(40, 40 + n)))
        b.step(2)
        s = b.get_state(bad)
        t = s["T"].copy()
        t[10, 3] = np.nan
        b.set_state(bad, t, s["omg"], s["up"], s["ur"])
        b.step(3)
        with pytest.raises(fg.FalconError, match="non-finite"):
            b.diagnostics()
        for i in range(n):
            st = b.get_state(i)
            finite = all(np.isfinite(st[f]).all() for f in ("T", "omg", "up", "ur"))
            assert finite == (i != bad), i
        b.close()
    finally:
        fg.set_gemm_mode(prev)
