"""A non-finite value in one instance's state is reported by the batch's
diagnostics (FALCON_ENONFINITE, the reference's own guard is on KE) and does
not reach the other instances of the batch: every contraction, transform and
slice exponent works per instance column, on the tensor-core paths (Inf or
NaN columns give NaN) as on the FP64 ones."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


# Nm = 42: Np = 126 (FMA butterflies); 85: Np = 255 (radix 17 on the tensor
# cores); 19: Np = 57 (radix 19, the wide tensor-core stage)
@pytest.mark.parametrize("gemm_mode,Nm", [(1, 42), (3, 42), (0, 42), (4, 85), (4, 19)])
def test_nonfinite_instance_is_reported_and_isolated(fg, gemm_mode, Nm):
    n, bad = 20, 7
    prev = fg.set_gemm_mode(gemm_mode)
    try:
        ps = [fg.make_params(65, Nm, "SBDF3", ra=1e5 * (1 + 0.05 * k), dt=1e-5) for k in range(n)]
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
