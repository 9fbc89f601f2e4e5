"""The integer-slice arithmetic of the tensor-core paths, restated with
Python integers and checked against exact rational sums (no GPU).

Mirrors falcon-dns_gb300/csrc/falcon_slices.cuh: an FP64 value with
|a| < 2^e is cut into S signed W-bit slices of |a| 2^(MAGB - e); products of
slice pairs s + t <= D are summed per diagonal (the FP32 sums on the GPU,
which must stay below 2^24 to be exact), then recombined as
2^kH H + 2^kL L.  Operator GEMM formats (W, S, D) = (6, 10, 9) for K <= 257
and (7, 9, 8) for K <= 112; the odd-prime DFT stages (9, 7, 6) with at
most 8 products per output (p <= 17) and (8, 8, 7) with at most 15
(p = 19 .. 31)."""
import math
import random
import struct
from fractions import Fraction

import pytest

FORMATS = {6: dict(S=10, D=9, HD=4, MAGB=60), 7: dict(S=9, D=8, HD=3, MAGB=63), 9: dict(S=7, D=6, HD=2, MAGB=63),
           8: dict(S=8, D=7, HD=3, MAGB=64)}


def bexp(x):
    return (struct.unpack("<q", struct.pack("<d", x))[0] >> 52) & 0x7FF


def mag(a, e, magb):
    bits = struct.unpack("<q", struct.pack("<d", a))[0]
    eb = (bits >> 52) & 0x7FF
    if eb == 0:
        return 0
    m = (bits & ((1 << 52) - 1)) | (1 << 52)
    sh = eb - 1075 + magb - e
    return m << sh if sh >= 0 else (m >> -sh if sh > -64 else 0)


def sliced_dot(a, x, W):
    f = FORMATS[W]
    S, D, HD, MAGB = f["S"], f["D"], f["HD"], f["MAGB"]
    er, fb = max(bexp(v) for v in a) - 1022, max(bexp(v) for v in x)

    def cut(v, e):
        T = mag(v, e, MAGB)
        assert T < 2 ** MAGB
        return [(-1 if v < 0 else 1) * ((T >> (W * (S - 1 - s))) & ((1 << W) - 1)) for s in range(S)]

    A, X = [cut(v, er) for v in a], [cut(v, fb - 1022) for v in x]
    Q = [0] * (D + 1)
    for s in range(S):
        for t in range(S):
            if s + t <= D:
                Q[s + t] += sum(A[k][s] * X[k][t] for k in range(len(a)))
    H = L = 0
    for d in range(HD + 1):
        H = H * (1 << W) + Q[d]
    for d in range(HD + 1, D + 1):
        L = L * (1 << W) + Q[d]
    kL = er + (fb - 1022) - 2 * MAGB + W * (2 * S - 2 - D)
    kH = kL + W * (D - HD)
    assert abs(H) < 2 ** 53 and abs(L) < 2 ** 53
    return math.ldexp(H, kH) + math.ldexp(L, kL), max(abs(q) for q in Q)


@pytest.mark.parametrize("W,K", [(6, 257), (6, 65), (7, 112), (7, 65), (9, 8)])
def test_sliced_dot_is_exact_to_one_rounding(W, K):
    rng = random.Random(W * 1000 + K)
    for _ in range(12):
        a = [rng.gauss(0, 1) * 10 ** rng.uniform(-4, 4) for _ in range(K)]
        x = [rng.gauss(0, 1) * 10 ** rng.uniform(-12, 3) for _ in range(K)]
        if rng.random() < 0.3:
            x[rng.randrange(K)] = 0.0
        y, qmax = sliced_dot(a, x, W)
        assert qmax < 2 ** 24  # every FP32 partial sum exact
        exact = sum(Fraction(p) * Fraction(q) for p, q in zip(a, x))
        scale = Fraction(max(map(abs, a))) * Fraction(max(map(abs, x)))
        # truncation and dropped pairs below 2^-56 of max|a| max|x| per product,
        # plus the final FP64 rounding of the sum
        bound = K * Fraction(1, 2 ** 56) * scale + abs(exact) * Fraction(1, 2 ** 52)
        assert abs(Fraction(y) - exact) <= bound


@pytest.mark.parametrize("p", [11, 13, 17, 19, 31])
def test_dft_butterfly_sums(p):
    # A_j = sum_q a_q cos(2 pi jq/p) and B_j = sum_q b_q sin(2 pi jq/p) of the
    # symmetric odd-prime butterfly through the 9-bit format
    h = (p - 1) // 2
    rng = random.Random(p)
    for _ in range(20):
        v = [complex(rng.gauss(0, 1), rng.gauss(0, 1)) * 10 ** rng.uniform(-9, 4) for _ in range(p)]
        for comp in (0, 1):
            part = (lambda z: z.real) if comp == 0 else (lambda z: z.imag)
            a = [part(v[q]) + part(v[p - q]) for q in range(1, h + 1)]
            b = [part(v[q]) - part(v[p - q]) for q in range(1, h + 1)]
            for j in range(1, h + 1):
                c = [math.cos(2 * math.pi * ((j * q) % p) / p) for q in range(1, h + 1)]
                s = [math.sin(2 * math.pi * ((j * q) % p) / p) for q in range(1, h + 1)]
                # the GPU scales a and b of a column by their joint maximum:
                # append it with a zero coefficient
                col = max(map(abs, a + b))
                for vals, coef in ((a, c), (b, s)):
                    y, qmax = sliced_dot(coef + [0.0], vals + [col], 9 if h <= 8 else 8)
                    assert qmax < 2 ** 24
                    exact = sum(Fraction(u) * Fraction(w) for u, w in zip(coef, vals))
                    assert abs(Fraction(y) - exact) <= abs(exact) * Fraction(1, 2 ** 52) + Fraction(col) * Fraction(1, 2 ** 57)


def test_bf16_bias_trick_of_the_packed_slices():
    # oz_slice_pair (falcon_slices.cuh): bf16(128 + q) has the bits 0x4300 + q
    # for 0 <= q < 128 (exactly representable), so subtracting 128 in bf16
    # gives q exactly (Sterbenz: 128 <= 128 + q < 256)
    import numpy as np
    for q in range(128):
        b = int(np.float32(128 + q).view(np.uint32))
        assert b & 0xFFFF == 0 and b >> 16 == 0x4300 + q
        assert float(np.float32(128 + q) - np.float32(128)) == q
