"""The integer-pipe conversions of csrc/el_f2d.cuh against the compiler's: the header compiled for
the host.  float -> double (the matrix build, the FP64 residual): every one of the 2^32 float bit
patterns (NaN payloads, which both leave to the conversion, aside).  double -> float (the matrix
build's FP32 records): every exponent at the rounding boundaries, and 2 x 10^8 random patterns."""

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


D2F_DRIVER = r"""
#include <cstdio>
#include <cstring>
#include <cstdint>
#include "el_f2d.cuh"
static uint64_t state = 88172645463325252ull;
static uint64_t next() { state ^= state << 13; state ^= state >> 7; state ^= state << 17; return state; }
static unsigned long long bad = 0;
static void check(uint64_t b) {
    double d;
    std::memcpy(&d, &b, 8);
    if (d != d) return;
    const float a = el::d2f(d), c = (float)d;
    uint32_t ba, bc;
    std::memcpy(&ba, &a, 4);
    std::memcpy(&bc, &c, 4);
    if (ba != bc && bad++ < 4) std::printf("mismatch %016llx\n", (unsigned long long)b);
}
int main() {
    // every exponent, both signs, with the 29 rounding bits at and around the halfway point and
    // the kept mantissa's last bit even and odd; then random patterns
    const uint32_t rems[] = {0u, 1u, 0x0fffffffu, 0x10000000u, 0x10000001u, 0x1fffffffu};
    const uint64_t mants[] = {0ull, 1ull, 2ull, 0x7ffffeull, 0x7fffffull, 0x2aaaaaull};
    for (uint64_t s = 0; s < 2; ++s)
        for (uint64_t e = 0; e < 2048; ++e)
            for (uint64_t m : mants)
                for (uint32_t r : rems) check((s << 63) | (e << 52) | (m << 29) | r);
    for (long i = 0; i < 200000000l; ++i) check(next());
    std::printf("%llu\n", bad);
    return bad ? 1 : 0;
}
"""


def test_d2f_matches_the_conversion(tmp_path):
    cxx = shutil.which("g++")
    if not cxx:
        pytest.skip("no host compiler")
    src = tmp_path / "d2f.cpp"
    src.write_text(D2F_DRIVER)
    exe = tmp_path / "d2f"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", HEADER_DIR, str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().splitlines()[-1] == "0"


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
