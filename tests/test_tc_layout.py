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
    assert (bm, bn, sbo, alob, xlbo, xlbo10) == (128, 48, 128, 128 * 16, 9 * 48 * 16, 10 * 48 * 16)
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


@pytest.mark.parametrize("S", [9, 10])
def test_x_stage_matches_producer_stores(S):
    # producer: unit (column n, k group kg) stores 8 k values of slice t as
    # 16 bytes at (kg S 6 + t 6 + n/8) 128 + (n%8) 16: slice t's column n is
    # stage column 48 t + n, k groups S x 768 bytes apart
    lbo = S * 48 * 16
    for t in range(S):
        for n in range(48):
            for j in range(16):
                prod = ((j // 8) * S * 6 + t * 6 + n // 8) * 128 + (n % 8) * 16 + (j % 8) * 2
                assert canonical(0, lbo, 128, 48 * t + n, j) == prod


@pytest.mark.parametrize("S", [9, 10])
def test_concatenated_products_land_on_their_diagonals(S):
    # the MMA of operator slice s multiplies the stage columns 0 .. 48 (S - s)
    # (slices t = 0 .. S-1-s) into tensor-memory columns 48 s + c: column
    # 48 t + n of the product must land in diagonal s + t, column n, in parts
    # of at most 256 columns whose widths are multiples of 16
    D = S - 1
    for s in range(S):
        ntot = (D + 1 - s) * 48
        covered = []
        for c in range(0, ntot, 256):
            n = min(256, ntot - c)
            assert n % 16 == 0 and 48 * s + c + n <= 512
            covered.extend(range(c, c + n))
        assert covered == list(range(ntot))
        for i in range(ntot):
            t, n = divmod(i, 48)
            assert divmod(48 * s + i, 48) == (s + t, n)
