"""The host radix sort of the AMR table builders (csrc/host_sort.h) against
std::sort, compiled for the host with g++: empty, single, sorted, reversed,
duplicate and full-width keys, and keys shaped as the reflux grouping's
(element index << 22 | discovery index)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "opencfd-amr_gb300", "csrc")

DRIVER = r"""
#include "host_sort.h"
#include <cstdio>
#include <random>
static int check(std::vector<uint64_t> k, const char* what) {
    std::vector<uint64_t> r = k;
    std::sort(r.begin(), r.end());
    ocfd::radix_sort_u64(k);
    if (k != r) { std::printf("mismatch: %s (n = %zu)\n", what, k.size()); return 1; }
    return 0;
}
int main() {
    std::mt19937_64 g(20261204);
    int bad = 0;
    bad += check({}, "empty");
    bad += check({42}, "single");
    for (size_t n : {2u, 3u, 17u, 1000u, 65537u, 200000u}) {
        std::vector<uint64_t> a(n), b(n), c(n), d(n), e(n);
        for (size_t q = 0; q < n; ++q) {
            a[q] = g();                                        // full 64-bit width
            b[q] = ((g() % (1u << 27)) << 22) | q;             // reflux keys
            c[q] = q * 3;                                      // sorted
            d[q] = (uint64_t)(n - q) << 40;                    // reversed, high digits only
            e[q] = g() % 7;                                    // many duplicates
        }
        bad += check(a, "random 64-bit") + check(b, "reflux keys") + check(c, "sorted") +
               check(d, "reversed") + check(e, "duplicates");
    }
    if (!bad) std::printf("ok\n");
    return bad ? 1 : 0;
}
"""


def test_radix_sort_matches_std_sort(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not present")
    src = tmp_path / "sort_driver.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "sort_driver"
    r = subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
