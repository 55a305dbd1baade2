"""The integer-pipe float -> double conversion (csrc/el_f2d.cuh, used by the matrix build and the
FP64 residual) against the compiler's conversion: the header compiled for the host, every one of
the 2^32 float bit patterns (NaN payloads, which both leave to the conversion, aside)."""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER_DIR = os.path.join(HERE, "..", "eulerian-liquid_gb300", "csrc")

DRIVER = r"""
#include <cstdio>
#include <cstring>
#include "el_f2d.cuh"
int main() {
    unsigned long long bad = 0;
    for (unsigned long long x = 0; x <= 0xffffffffull; ++x) {
        const unsigned u = (unsigned)x;
        if (((u >> 23) & 0xffu) == 0xffu && (u & 0x7fffffu)) continue;
        float f;
        std::memcpy(&f, &u, 4);
        const double a = el::f2d(f), b = (double)f;
        unsigned long long ba, bb;
        std::memcpy(&ba, &a, 8);
        std::memcpy(&bb, &b, 8);
        if (ba != bb && bad++ < 4) std::printf("mismatch %08x\n", u);
    }
    std::printf("%llu\n", bad);
    return bad ? 1 : 0;
}
"""


def test_f2d_matches_the_conversion_for_every_float(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no host compiler")
    src = tmp_path / "f2d.cpp"
    src.write_text(DRIVER)
    exe = tmp_path / "f2d"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", HEADER_DIR, str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().splitlines()[-1] == "0"
