"""The tcgen05 operator contractions (falcon_set_gemm_mode(3): every
contraction with a slice view on tcgen05, narrow per-mode ones included;
TMA-staged operator slices, X sliced by producer warps in shared memory, one
FP32 accumulator per slice diagonal in tensor memory) against the mma.sync
path with the same slices (mode 1).  Every FP32 sum of slice products is
exact in both, so the states must agree bit for bit, step after step, on
every configuration: 7-bit slices with the operator resident in shared memory
(K <= 80), 7-bit slices streamed (Nr = 97, K = 112) and 6-bit slices
streamed (Nr = 129); groups whose per-mode contractions span several column
tiles and the radial contractions over all modes; IMEX, IMEXRK (with the
psi Poisson operator) and RK.  A wait that timed out inside the kernel
would make get_state fail."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("T", "omg", "up", "ur", "psi")


def run(fg, params, seeds, nsteps, mode):
    prev = fg.set_gemm_mode(mode)
    try:
        b = fg.Batch(params)
        b.init_noise(seeds)
        b.step(nsteps)
        out = [b.get_state(i) for i in range(len(params))]
        b.close()
    finally:
        fg.set_gemm_mode(prev)
    return out


@pytest.mark.parametrize("scheme,R,Nm,B,nsteps", [
    ("SBDF3", 17, 8, 3, 10),        # K = 17 (padded 32): one column tile per mode
    ("CNAB2", 33, 42, 12, 10),      # the plain reference run's grid, 12 instances
    ("SBDF3", 65, 170, 40, 5),      # the uniform batch's grid: K = 65 (padded 80), operator resident
    ("ARS343", 33, 20, 10, 10),     # psi Poisson operator with Johnston wall rows
    ("RK4", 33, 20, 8, 10),
    ("BPR353", 97, 42, 6, 5),       # K = 97 (padded 112): 7-bit slices streamed
    ("SBDF3", 129, 85, 5, 5),       # K = 129 (padded 144): 6-bit slices streamed
])
def test_tcgen05_matches_mma_sync_bitwise(fg, scheme, R, Nm, B, nsteps):
    ras = np.geomspace(1e4, 1e6, B)
    ps = [fg.make_params(R, Nm, scheme, ra=float(ra), dt=1e-5) for ra in ras]
    seeds = list(range(300, 300 + B))
    a = run(fg, ps, seeds, nsteps, 3)
    b = run(fg, ps, seeds, nsteps, 1)
    for i in range(B):
        for k in FIELDS:
            assert np.array_equal(a[i][k], b[i][k]), (i, k, float(np.abs(a[i][k] - b[i][k]).max()))
