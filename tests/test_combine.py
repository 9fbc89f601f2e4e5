"""The exact recombination helpers of falcon-dns_gb300/csrc/falcon_combine.h:
diag_sum (the diagonal sums of a slice product, two per 32-bit
multiply-add) against Horner's sum at the largest diagonal magnitudes of
both slice formats, and the integer-only combine_rn of the tensor-core DFT
stages against the two-term form (two exact power-of-two scalings and one FP64
add): the same bits on random sums of every sign, on exact ties of the
rounding (to nearest even), on cancellations to zero, at the edges of its
exponent range and beyond them (where it takes the two-term form itself);
and the fixed-point conversions of the DFT stages (fix_of, dbl_of_fix).
Compiled on the host with g++: no GPU."""
import os
import subprocess

import pytest

from conftest import PKG

HARNESS = r'''
#include <cstdio>
#include <cmath>
#include <cstring>
#include <random>
#include "falcon_combine.h"
using namespace falcon;
static bool same(double a, double b) { return std::memcmp(&a, &b, sizeof a) == 0; }
int main() {
  std::mt19937_64 rng(12345);
  long long checked = 0, bad = 0, fast = 0;
  const int shifts[] = {30, 32, 35, 36};
  auto check = [&](long long H, long long L, int k, int sh) {
    const double ref = i64_scaled(H, k + sh) + i64_scaled(L, k);
    const double got = combine_rn(H, L, k, sh);
    ++checked;
    if (!(k < -1022 || k + sh + 55 > 1024)) ++fast;
    if (!same(ref, got)) {
      if (bad < 5) std::printf("MISMATCH H=%lld L=%lld k=%d sh=%d ref=%a got=%a\n", H, L, k, sh, ref, got);
      ++bad;
    }
  };
  for (int it = 0; it < 2000000; ++it) {
    const int sh = shifts[rng() % 4];
    const int hb = (int)(rng() % 50), lb = (int)(rng() % 54);   // bit lengths up to 2^49, 2^53
    long long H = hb ? (long long)(rng() >> (64 - hb)) : 0, L = lb ? (long long)(rng() >> (64 - lb)) : 0;
    if (rng() & 1) H = -H;
    if (rng() & 1) L = -L;
    int k;
    switch (rng() % 4) {
      case 0: k = (int)(rng() % 200) - 150; break;            // the usual range
      case 1: k = -1022 + (int)(rng() % 8) - 4; break;        // lower edge
      case 2: k = 1024 - 55 - sh + (int)(rng() % 8) - 4; break;  // upper edge
      default: k = (int)(rng() % 2100) - 1100; break;         // anywhere, fallbacks included
    }
    check(H, L, k, sh);
  }
  // exact ties: S = m 2^s + 2^(s-1) with 53-bit m, even and odd
  for (int it = 0; it < 200000; ++it) {
    const int sh = shifts[rng() % 4];
    const int s = 1 + (int)(rng() % (sh - 1));
    const long long m = (long long)((rng() >> 11) | (1ull << 52));
    // split S = H 2^sh + L with |L| < 2^53: H = S >> sh, L = S - H 2^sh
    const unsigned __int128 S = ((unsigned __int128)m << s) + ((unsigned __int128)1 << (s - 1));
    const long long H = (long long)(S >> sh), L = (long long)(S - ((unsigned __int128)H << sh));
    const int sg = (rng() & 1) ? -1 : 1;
    check(sg * H, sg * L, (int)(rng() % 100) - 80, sh);
  }
  // cancellations and one-sided terms
  for (int it = 0; it < 100000; ++it) {
    const int sh = shifts[rng() % 4];
    const long long H = (long long)(rng() >> 20) - (1ll << 43);
    check(H, -(H * (1ll << 9)), 0, 9 + 0 * sh);  // H 2^9 - H 2^9 = 0 (sh = 9 here)
    check(H, 0, -50, sh);
    check(0, H, -50, sh);
  }
  // diag_sum against Horner's sum for both slice formats and their splits,
  // diagonals at their largest magnitudes included
  long long dbad = 0, dchecked = 0;
  auto horner = [](const int* q, int a, int b, int w) {
    long long s = 0;
    for (int d = a; d <= b; ++d) s = s * (1LL << w) + q[d];
    return s;
  };
  const int m7 = 9 * 112 * 127 * 127, m6 = 10 * 272 * 63 * 63;
  for (int it = 0; it < 400000; ++it) {
    int q[10];
    const int w = (it & 1) ? 7 : 6, m = w == 7 ? m7 : m6;
    for (int d = 0; d < 10; ++d) {
      const unsigned long long r = rng();
      q[d] = (r % 8 == 0) ? ((r & 8) ? m : -m) : (int)(r % (2ull * m + 1)) - m;
    }
    auto Q = [&](int d) { return q[d]; };
    long long h, l, hh, ll;
    if (w == 7) { h = diag_sum<7, 0, 3>(Q); l = diag_sum<7, 4, 8>(Q); hh = horner(q, 0, 3, 7); ll = horner(q, 4, 8, 7); }
    else { h = diag_sum<6, 0, 4>(Q); l = diag_sum<6, 5, 9>(Q); hh = horner(q, 0, 4, 6); ll = horner(q, 5, 9, 6); }
    dchecked += 2;
    if (h != hh || l != ll) {
      if (dbad < 5) std::printf("DIAG MISMATCH w=%d\n", w);
      ++dbad;
    }
  }
  // fix_of (a 2^(FB - e) truncated, |a| < 2^e) against the exact scaling
  // and cast; dbl_of_fix (RN(v 2^k) of any 64-bit v) against ldexp of the
  // correctly rounded conversion
  long long fbad = 0, fchecked = 0;
  for (int it = 0; it < 1000000; ++it) {
    const int e = (int)(rng() % 200) - 100;
    double a = std::ldexp((double)(rng() >> 11) / 9007199254740992.0, e - (int)(rng() % 70));
    if (rng() & 1) a = -a;
    const int fb = (it & 1) ? 58 : 57;
    const long long got = fb == 58 ? fix_of<58>(a, e) : fix_of<57>(a, e);
    const long long ref = (long long)std::ldexp(a, fb - e);
    ++fchecked;
    if (got != ref) {
      if (fbad < 5) std::printf("FIX MISMATCH a=%a e=%d\n", a, e);
      ++fbad;
    }
    long long v = (long long)rng();
    v >>= (int)(rng() % 63);
    if (rng() & 1) v = -v;
    const int k = (int)(rng() % 400) - 200;
    ++fchecked;
    if (!same(dbl_of_fix(v, k), std::ldexp((double)v, k))) {
      if (fbad < 5) std::printf("DBL MISMATCH v=%lld k=%d\n", v, k);
      ++fbad;
    }
  }
  std::printf("%lld %lld\n", fchecked, fbad);
  std::printf("%lld %lld\n", dchecked, dbad);
  std::printf("%lld %lld %lld\n", checked, fast, bad);
  return 0;
}
'''


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    d = tmp_path_factory.mktemp("combine")
    (d / "h.cpp").write_text(HARNESS)
    exe = d / "h"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I" + os.path.join(PKG, "csrc"), str(d / "h.cpp"), "-o", str(exe)],
                   check=True)
    return subprocess.run([str(exe)], check=True, capture_output=True, text=True, timeout=300).stdout


def test_pairwise_diagonal_sums_equal_horner(harness):
    dchecked, dbad = (int(x) for x in harness.strip().splitlines()[-2].split())
    assert dbad == 0 and dchecked == 800_000, harness


def test_fixed_point_conversions_are_exact(harness):
    fchecked, fbad = (int(x) for x in harness.strip().splitlines()[-3].split())
    assert fbad == 0 and fchecked == 2_000_000, harness


def test_combine_rn_is_bit_identical_to_the_two_term_form(harness):
    last = harness.strip().splitlines()[-1]
    checked, fast, bad = (int(x) for x in last.split())
    assert bad == 0, harness
    assert checked > 2_000_000 and fast > checked // 2   # most cases take the integer path
