import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "falcon-dns_gb300")
ORACLE = os.path.join(ROOT, "oracle")
for p in (PKG, ORACLE, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def orc():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def fg():
    import build as falcon_build
    falcon_build.build()
    import falcon_gpu
    falcon_gpu.lib()
    return falcon_gpu


@pytest.fixture
def fixed_paths(fg):
    """Contraction paths by the fixed rules (falcon_set_gemm_mode(2)) instead
    of the autotuner: the path of a contraction then depends only on its
    kind and on whether it has 16 columns per batch entry, and every path is
    exact per column, so an instance of a small batch steps to the same bits
    alone and in the batch.  (Under the autotuner the paths of different
    shapes may differ, and such results agree to FP64 rounding.)"""
    prev = fg.set_gemm_mode(2)
    yield
    fg.set_gemm_mode(prev)


@pytest.fixture(scope="session")
def golden():
    import numpy as np
    return np.load(os.path.join(ROOT, "tests", "golden", "golden.npz"))


def rel(a, b):
    import numpy as np
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm((a - b).ravel()) / max(np.linalg.norm(b.ravel()), 1e-300))


def _intcheb(f, eta=0.35):
    """Chebyshev quadrature of values on the Gauss-Lobatto grid over
    [rmin, rmax]: intcheb of the reference's post-processing
    (python/annulus/cheblib.py:57-85), through its chebtransform
    (:467-494), restated."""
    import numpy as np
    f = np.asarray(f, dtype=float)
    nr = f.size
    ext = np.concatenate([f[::-1], f[1:nr - 1]])
    ff = np.real(np.fft.fft(ext)) / (2 * nr - 2)
    f2 = ff[:nr].copy()
    f2[1:nr - 1] *= 2.0
    fac = np.sqrt(2.0 / (nr - 1))
    fn = f2 / fac
    fn[0] *= 2.0
    fn[nr - 1] *= 2.0
    width = 1.0 / (1.0 - eta) - eta / (1.0 - eta)
    total = 0.0
    for i in range(0, nr, 2):
        w = 0.5 if (i == 0 or i == nr - 1) else 1.0
        total -= w * width / (i * i - 1.0) * fn[i]
    return total * np.sqrt(2.0 / (nr - 1.0))


def rel_l2_reference(comp, ref, eta=0.35):
    """The reference's error norm calc_rel_L2norm (python/annulus/cheblib.py:
    251-271), restated for state arrays (R, M) (mode fastest): the ratio of
    the radial integrals of r (|d_0|^2 + 2 sum_{m>=1} |d_m|^2) for the
    difference and for the reference field."""
    import numpy as np
    comp = np.asarray(comp)
    ref = np.asarray(ref)
    nr = ref.shape[0]
    rmin = eta / (1.0 - eta)
    rr = rmin + 0.5 * (1.0 + np.cos(np.pi * (1.0 - np.arange(nr) / (nr - 1.0))))
    d = np.abs(comp - ref) ** 2
    q = np.abs(ref) ** 2
    diff = 2.0 * d[:, 1:].sum(axis=1) + d[:, 0]
    den = 2.0 * q[:, 1:].sum(axis=1) + q[:, 0]
    return float(np.sqrt(_intcheb(rr * diff, eta) / _intcheb(rr * den, eta)))
