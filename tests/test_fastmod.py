"""The batch sampler's row index r % count goes through the Barrett remainder of csrc/fastmod.h
(the same header the device code includes). A host program built from that header checks it
against the `%` operator on edge-case and random 64-bit operands. No GPU is used."""
import pathlib
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
CSRC = ROOT / "practical-stylized_gb300" / "csrc"

PROG = r"""
#include <cstdio>
#include <cstdint>
#include "fastmod.h"

static uint64_t s = 0x9E3779B97F4A7C15ull;
static uint64_t next() {  // splitmix64
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int main() {
    const uint64_t ds[] = {1, 2, 3, 7, 29000, 241872, 65536, 2073600, 4294967295ull, 4294967296ull,
                           4294967297ull, 9223372036854775807ull, 9223372036854775808ull,
                           9223372036854775809ull, 18446744073709551615ull, 18446744073709551614ull};
    long bad = 0, n = 0;
    for (uint64_t d : ds) {
        const uint64_t m = sty::fastmod_magic(d);
        const uint64_t rs[] = {0, 1, d - 1, d, d + 1, 2 * d - 1, 2 * d, UINT64_MAX, UINT64_MAX - 1,
                               UINT64_MAX / d * d, UINT64_MAX / d * d - 1};
        for (uint64_t r : rs) { n++; if (sty::fastmod(r, d, m) != r % d) bad++; }
        for (int i = 0; i < 200000; i++) { const uint64_t r = next(); n++; if (sty::fastmod(r, d, m) != r % d) bad++; }
    }
    for (int i = 0; i < 2000000; i++) {  // random divisors of every size
        uint64_t d = next() >> (next() % 64);
        if (d == 0) d = 1;
        const uint64_t r = next();
        n++;
        if (sty::fastmod(r, d, sty::fastmod_magic(d)) != r % d) bad++;
    }
    std::printf("%ld %ld\n", n, bad);
    return 0;
}
"""


def test_barrett_remainder_matches_modulo(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    src = tmp_path / "fastmod_check.cpp"
    src.write_text(PROG)
    exe = tmp_path / "fastmod_check"
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", str(CSRC), str(src), "-o", str(exe)], check=True,
                   capture_output=True)
    n, bad = map(int, subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split())
    assert n > 5_000_000
    assert bad == 0
