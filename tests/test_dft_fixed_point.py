"""The fixed-point odd-prime butterfly of the tensor-core DFT stages
(dft_mma_stage / dft_mma_stage_wide, falcon-dns_gb300/csrc/falcon_fft.cuh)
restated in exact integer arithmetic on the CPU:
- every value of a butterfly as trunc(v 2^(FB - e)) at the scale 2^e of its
  largest, the pre-adds a = V_q + V_{p-q}, b = V_q - V_{p-q} and y_0 exact;
- the coefficients (63- or 64-bit fractions) and 2^UP |a|, 2^UP |b| cut
  into S slices of W bits, the pairs s + t <= D summed per diagonal: every
  diagonal sum below 2^24 in magnitude (what keeps the kernel's FP32
  accumulation exact), checked at the largest inputs;
- v_0 added in units of 2^(e - 71), each output rounded once.
Its outputs are the exact sums (with the kernels' FP64 cos/sin values)
rounded once, up to the inputs' truncation; against the exact DFT
(mpmath, 40 digits) its error is of the order of the FP64 FMA butterfly's,
on butterflies of mixed magnitudes.  CPU only."""
import math
import random
import struct
from fractions import Fraction

import pytest

mp = pytest.importorskip("mpmath")

NARROW = dict(W=9, S=7, D=6, FB=58, UP=4, MAG=63)   # p = 11, 13, 17
WIDE = dict(W=8, S=8, D=7, FB=57, UP=6, MAG=64)     # p = 19, 23, 29, 31


def bexp(x):
    return (struct.unpack("<q", struct.pack("<d", x))[0] >> 52) & 0x7FF


def fix(a, e, fb):
    if a == 0 or bexp(a) == 0:
        return 0
    t = math.floor(Fraction(abs(a)) * 2 ** (fb - e))
    return -t if a < 0 else t


def slices(T, f):
    return [(T >> (f["W"] * (f["S"] - 1 - s))) & ((1 << f["W"]) - 1) for s in range(f["S"])]


def slice_product(coef, data, f, qmax):
    """sum_q coef_q data_q from the slices, diagonals d <= D, in units of
    2^-(MAG + FB - e + UP); records the largest diagonal sum."""
    Q = [0] * (f["D"] + 1)
    for c, x in zip(coef, data):
        cs = slices(math.floor(abs(Fraction(c)) * 2 ** f["MAG"]), f)
        xs = slices(abs(x) << f["UP"], f)
        sg = (-1 if c < 0 else 1) * (-1 if x < 0 else 1)
        for s in range(f["S"]):
            for t in range(f["S"] - s):
                if s + t <= f["D"]:
                    Q[s + t] += sg * cs[s] * xs[t]
    qmax[0] = max(qmax[0], max(abs(q) for q in Q))
    return sum(Q[d] * 2 ** (f["W"] * (f["D"] - d)) for d in range(f["D"] + 1))


def fixed_point_butterfly(v, p, qmax):
    f = NARROW if p <= 17 else WIDE
    h = (p - 1) // 2
    e = max(max(bexp(z.real), bexp(z.imag)) for z in v) - 1022
    unit = Fraction(2) ** (e - 71)     # units of the slice products with V0 folded in
    shift = 71 - f["FB"]               # V0 into those units (13 or 14 bits)
    parts = {}
    for comp in (0, 1):
        X = [fix(z.imag if comp else z.real, e, f["FB"]) for z in v]
        a = [X[q] + X[p - q] for q in range(1, h + 1)]
        b = [X[q] - X[p - q] for q in range(1, h + 1)]
        y0 = X[0] + sum(a)
        assert abs(y0) < 2 ** 63
        parts[("y0", comp)] = Fraction(y0) * Fraction(2) ** (e - f["FB"])
        for j in range(1, h + 1):
            C = [math.cos(2 * math.pi * ((j * q) % p) / p) for q in range(1, h + 1)]
            Sn = [math.sin(2 * math.pi * ((j * q) % p) / p) for q in range(1, h + 1)]
            parts[("A", j, comp)] = slice_product(C, a, f, qmax) + X[0] * 2 ** shift
            parts[("B", j, comp)] = slice_product(Sn, b, f, qmax)
    y = [0j] * p
    y[0] = complex(float(parts[("y0", 0)]), float(parts[("y0", 1)]))
    for j in range(1, h + 1):
        Ar, Ai = parts[("A", j, 0)], parts[("A", j, 1)]
        Br, Bi = parts[("B", j, 0)], parts[("B", j, 1)]
        y[j] = complex(float((Ar + Bi) * unit), float((Ai - Br) * unit))
        y[p - j] = complex(float((Ar - Bi) * unit), float((Ai + Br) * unit))
    return y


def fma_butterfly(v, p):
    """The FP64 symmetric butterfly of the FMA stages (dft_odd_store)."""
    h = (p - 1) // 2
    fma = lambda x, c, acc: float(Fraction(x) * Fraction(c) + Fraction(acc))
    a = [complex(v[q].real + v[p - q].real, v[q].imag + v[p - q].imag) for q in range(1, h + 1)]
    b = [complex(v[q].real - v[p - q].real, v[q].imag - v[p - q].imag) for q in range(1, h + 1)]
    y0r, y0i = v[0].real, v[0].imag
    for q in range(h):
        y0r += a[q].real
        y0i += a[q].imag
    y = [complex(y0r, y0i)] + [0j] * (p - 1)
    for j in range(1, h + 1):
        Ar, Ai, Br, Bi = v[0].real, v[0].imag, 0.0, 0.0
        for q in range(1, h + 1):
            c = math.cos(2 * math.pi * ((j * q) % p) / p)
            s = math.sin(2 * math.pi * ((j * q) % p) / p)
            Ar, Ai = fma(a[q - 1].real, c, Ar), fma(a[q - 1].imag, c, Ai)
            Br, Bi = fma(b[q - 1].real, s, Br), fma(b[q - 1].imag, s, Bi)
        y[j] = complex(Ar + Bi, Ai - Br)
        y[p - j] = complex(Ar - Bi, Ai + Br)
    return y


def exact_dft(v, p):
    mp.mp.dps = 40
    return [complex(sum(mp.mpc(v[q].real, v[q].imag) * mp.expjpi(-2 * mp.mpf((j * q) % p) / p) for q in range(p)))
            for j in range(p)]


def max_err(y, ref, scale):
    return max(max(abs(y[i].real - ref[i].real), abs(y[i].imag - ref[i].imag)) for i in range(len(y))) / scale


def coef_dft(v, p):
    """The DFT in exact rational arithmetic with the FP64 cos/sin values the
    kernels use (symmetric form): what the fixed-point butterfly rounds."""
    h = (p - 1) // 2
    out = []
    for comp in (0, 1):
        x = [Fraction(z.imag if comp else z.real) for z in v]
        a = [x[q] + x[p - q] for q in range(1, h + 1)]
        b = [x[q] - x[p - q] for q in range(1, h + 1)]
        A = [x[0] + sum(Fraction(math.cos(2 * math.pi * ((j * q) % p) / p)) * a[q - 1] for q in range(1, h + 1))
             for j in range(1, h + 1)]
        B = [sum(Fraction(math.sin(2 * math.pi * ((j * q) % p) / p)) * b[q - 1] for q in range(1, h + 1))
             for j in range(1, h + 1)]
        out.append((x[0] + sum(a), A, B))
    (y0r, Ar, Br), (y0i, Ai, Bi) = out
    y = [(y0r, y0i)] + [None] * (p - 1)
    for j in range(1, h + 1):
        y[j] = (Ar[j - 1] + Bi[j - 1], Ai[j - 1] - Br[j - 1])
        y[p - j] = (Ar[j - 1] - Bi[j - 1], Ai[j - 1] + Br[j - 1])
    return y


@pytest.mark.parametrize("p", [11, 13, 17, 19, 31])
def test_fixed_point_butterfly_rounds_the_exact_sums_once(p):
    """Against the exact sums with the kernels' own coefficients: within half
    an ulp plus the inputs' truncation (2^(e - FB) each) and the dropped
    slice pairs; every diagonal sum exact in FP32 (below 2^24), also at the
    largest inputs."""
    f = NARROW if p <= 17 else WIDE
    rng = random.Random(100 + p)
    qmax = [0]
    for it in range(12):
        sc = 10.0 ** rng.uniform(-5, 5)
        v = [complex(rng.gauss(0, 1), rng.gauss(0, 1)) * sc * 10.0 ** rng.uniform(-3, 0) for _ in range(p)]
        if it == 0:  # every value at the top of its binade: the largest slices and diagonal sums
            v = [complex(rng.choice((-1, 1)) * (2.0 - 2.0 ** -52), rng.choice((-1, 1)) * (2.0 - 2.0 ** -52))
                 for _ in range(p)]
        e = max(max(bexp(z.real), bexp(z.imag)) for z in v) - 1022
        tol = Fraction(2) ** (e - f["FB"]) * (2 * p + 2) + Fraction(2) ** (e - 54)
        y = fixed_point_butterfly(v, p, qmax)
        for got, ref in zip(y, coef_dft(v, p)):
            for g, r in ((got.real, ref[0]), (got.imag, ref[1])):
                assert abs(Fraction(g) - r) <= Fraction(math.ulp(float(r))) / 2 + tol
    assert qmax[0] < 2 ** 24


@pytest.mark.parametrize("p", [11, 13, 17, 19, 31])
def test_fixed_point_butterfly_accuracy_against_the_exact_dft(p):
    """Against the exact DFT: the error of the FP64 FMA butterfly's order
    (both are dominated by the rounding of the cos/sin tables and of the
    largest outputs)."""
    rng = random.Random(p)
    worst_fix = worst_fma = 0.0
    for it in range(12):
        sc = 10.0 ** rng.uniform(-5, 5)
        v = [complex(rng.gauss(0, 1), rng.gauss(0, 1)) * sc * 10.0 ** rng.uniform(-3, 0) for _ in range(p)]
        ref = exact_dft(v, p)
        mx = max(max(abs(z.real), abs(z.imag)) for z in v)
        worst_fix = max(worst_fix, max_err(fixed_point_butterfly(v, p, [0]), ref, mx))
        worst_fma = max(worst_fma, max_err(fma_butterfly(v, p), ref, mx))
    assert worst_fix < p * 2.0 ** -51
    assert worst_fix <= 2 * worst_fma + 2 * 2.0 ** -53
