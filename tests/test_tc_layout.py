"""CPU checks of the tcgen05 contraction's encodings and shared-memory layout
(falcon-dns_gb300/csrc/falcon_tc.h, falcon_tc.cu), before any GPU run.

- The shared-memory matrix descriptor and the instruction descriptor are
  rebuilt bit by bit from their documented fields and compared with the
  library's encoders (a small C++ program compiled against falcon_tc.h).
- Under the documented no-swizzle K-major canonical layout (element (row i,
  k j) of an operand at start + (i/8) SBO + (j/8) LBO + (i%8) 16 + (j%8) 2),
  every element the MMAs read is exactly where the TMA box order (operator)
  and the producer warps (X) put it, and no descriptor reaches past its
  stage (tc_stage_layout_check, which the library also runs before it
  enables the kernel for an operator).
"""
import os
import subprocess

import pytest

from conftest import PKG

CSRC = os.path.join(PKG, "csrc")


def smem_desc(start, lbo, sbo):
    return ((start >> 4) & 0x3FFF) | (((lbo >> 4) & 0x3FFF) << 16) | (((sbo >> 4) & 0x3FFF) << 32) | (1 << 46)


def idesc(M, N):
    # D f32 (bits 4-5 = 1), A bf16 (7-9 = 1), B bf16 (10-12 = 1), K-major,
    # N >> 3 at bits 17-22, M >> 4 at bits 24-28
    return (1 << 4) | (1 << 7) | (1 << 10) | ((N >> 3) << 17) | ((M >> 4) << 24)


@pytest.fixture(scope="module")
def encoder(tmp_path_factory, fg):
    d = tmp_path_factory.mktemp("tc")
    src = d / "enc.cpp"
    src.write_text(r'''
#include <cstdio>
#include "falcon_tc.h"
int main() {
  using namespace falcon;
  std::printf("%d %d %u %u %u %u\n", kTcBM, kTcBN, kTcSbo, kTcALbo, tc_x_lbo(9), tc_x_lbo(10));
  const unsigned starts[] = {0u, 4096u, 36864u, 184320u, 227136u};
  for (unsigned s : starts)
    std::printf("%llu %llu\n", (unsigned long long)tc_smem_desc(s, kTcALbo, kTcSbo),
                (unsigned long long)tc_smem_desc(s, tc_x_lbo(9), kTcSbo));
  std::printf("%u %u\n", tc_idesc_bf16(128, 48), tc_idesc_bf16(128, 16));
  const int cases[][2] = {{7, 16}, {7, 48}, {7, 80}, {7, 112}, {6, 128}, {6, 144}, {6, 272}, {7, 20}};
  for (auto& c : cases) std::printf("%d\n", tc_stage_layout_check(c[0], c[1]));
  return 0;
}
''')
    exe = d / "enc"
    libdir = os.path.join(PKG, "_build")
    cuda = "/usr/local/cuda"
    subprocess.run(["g++", "-std=c++17", "-I" + CSRC, "-I" + os.path.join(cuda, "include"), str(src), "-o", str(exe),
                    "-L" + libdir, "-lfalcon_gpu", "-Wl,-rpath," + libdir, "-L" + os.path.join(cuda, "lib64"),
                    "-lcudart"], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    return out


def test_descriptor_encodings(encoder):
    bm, bn, sbo, alob, xlbo, xlbo10 = (int(x) for x in encoder[0].split())
    # X stages: 9 x 24 = 216 columns rounded up to 224, 10 x 24 = 240
    assert (bm, bn, sbo, alob, xlbo, xlbo10) == (128, 24, 128, 128 * 16, 224 * 16, 240 * 16)
    for line, s in zip(encoder[1:6], (0, 4096, 36864, 184320, 227136)):
        a, x = (int(v) for v in line.split())
        assert a == smem_desc(s, alob, sbo)
        assert x == smem_desc(s, xlbo, sbo)
    i48, i16 = (int(v) for v in encoder[6].split())
    assert i48 == idesc(128, 48) and i16 == idesc(128, 16)


def test_stage_layout_check(encoder):
    got = [int(x) for x in encoder[7:15]]
    assert got[:7] == [0] * 7          # every supported format and K padding
    assert got[7] != 0                 # K padding not a multiple of 16 is refused


def canonical(start, lbo, sbo, i, j):
    return start + (i // 8) * sbo + (j // 8) * lbo + (i % 8) * 16 + (j % 8) * 2


@pytest.mark.parametrize("S", [9, 10])
def test_operator_stage_matches_tma_box_order(S):
    # box {8 k, 128 rows, 2 k groups, S slices, 1 entry} lands innermost
    # first: element (k%8, row, k group, slice) at (((s 2 + kg) 128 + row) 8 + k%8) 2
    for s in range(S):
        start = s * 128 * 16 * 2
        for i in range(128):
            for j in range(16):
                tma = (((s * 2 + j // 8) * 128 + i) * 8 + j % 8) * 2
                assert canonical(start, 128 * 16, 128, i, j) == tma


def x_cols(S):
    return (S * 24 + 15) // 16 * 16


def mma_n(S, s):
    return ((S - s) * 24 + 15) // 16 * 16


@pytest.mark.parametrize("S", [9, 10])
def test_x_stage_matches_producer_stores(S):
    # producer: thread (column n, k group kg, half h) stores the 4 k values
    # 8 kg + 4 h + i of slice t as 8 bytes at (kg XG + 3 t + n/8) 128 +
    # (n%8) 16 + 8 h, XG = x_cols(S) / 8: slice t's column n is stage column
    # 24 t + n, the k groups x_cols(S) x 16 bytes apart
    lbo = x_cols(S) * 16
    xg = x_cols(S) // 8
    for t in range(S):
        for n in range(24):
            for j in range(16):
                kg, h, i = j // 8, (j % 8) // 4, j % 4
                prod = (kg * xg + 3 * t + n // 8) * 128 + (n % 8) * 16 + 8 * h + 2 * i
                assert canonical(0, lbo, 128, 24 * t + n, j) == prod
    # the padding columns (zeroed once) lie after every slice and inside the stage
    assert x_cols(S) >= S * 24 and 2 * x_cols(S) * 16 == 2 * xg * 128


@pytest.mark.parametrize("S", [9, 10])
def test_concatenated_products_land_on_their_diagonals(S):
    # the MMA of operator slice s multiplies stage columns 0 .. N-1 (the X
    # slices 0 .. S-1-s, N rounded up to a multiple of 16) into
    # accumulator columns 24 s .. 24 s + N - 1: column 24 t + n of the
    # product lands in diagonal s + t, column n; the rounding columns land
    # in the spill strip [24 S, 24 S + 8), which the epilogue never reads;
    # everything stays inside the 256-column buffer and N <= 256
    for s in range(S):
        n_mma = mma_n(S, s)
        assert n_mma % 16 == 0 and n_mma <= 256 and n_mma <= x_cols(S)
        assert 24 * s + n_mma <= 24 * S + 8 <= 256
        for i in range(n_mma):
            col = 24 * s + i
            if i < 24 * (S - s):
                t, n = divmod(i, 24)
                assert divmod(col, 24) == (s + t, n)
            else:
                assert 24 * S <= col < 24 * S + 8
