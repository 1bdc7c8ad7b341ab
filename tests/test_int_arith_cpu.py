"""Integer arithmetic of the device code, checked on the CPU.

The integer-arithmetic FP64 -> (FP32 hi, FP32 lo) split of stokes_to_gb300/csrc/fp64bits.cuh
(`split_bits`), restated step by step on Python integers and checked against the FP64
pipe's conversions (hi = fl32(d), lo = fl32(d - hi), round to nearest even) on random
doubles over the exponent range the fast path takes, on exact ties of the 29 dropped
significand bits and on significands that carry into the exponent. The GPU solves
(tests marked gpu) run the CUDA code itself: every 3D solve splits b with it. And the
multiply-high division of the box indices (internal.cuh Geom), compiled for the host."""
import struct

import numpy as np


def split_bits(d):
    b = struct.unpack("<Q", struct.pack("<d", d))[0]
    if (b << 1) & ((1 << 64) - 1) == 0:
        return float(np.float32(d)), 0.0
    e = ((b >> 52) & 0x7FF) - 1023
    if e < -74 or e > 126:
        return None  # the FP64 pipe's path
    m53 = (b & ((1 << 52) - 1)) | (1 << 52)
    top = m53 >> 29
    rem = m53 & ((1 << 29) - 1)
    r = rem
    if rem > (1 << 28) or (rem == (1 << 28) and (top & 1)):
        top += 1
        r = rem - (1 << 29)
    eh = e
    if top == (1 << 24):
        top = 1 << 23
        eh = e + 1
    sign = (b >> 32) & 0x80000000
    hi = struct.unpack("<f", struct.pack("<I", sign | ((eh + 127) << 23) | (top & 0x7FFFFF)))[0]
    if r == 0:
        return hi, 0.0
    scale = struct.unpack("<f", struct.pack("<I", (e - 52 + 127) << 23))[0]
    lo = float(np.float32(np.float32(r) * np.float32(scale)))
    return hi, (-lo if sign else lo)


def fp64_pipe(d):
    hi = np.float32(d)
    return float(hi), float(np.float32(d - np.float64(hi)))


def test_split_bits_matches_fp64_rounding():
    rng = np.random.default_rng(1)
    cases = list(rng.standard_normal(20000) * 10.0 ** rng.integers(-20, 20, 20000))
    for _ in range(4000):  # ties and near-ties of the dropped bits
        e = int(rng.integers(-70, 120))
        top = int(rng.integers(1 << 23, 1 << 24))
        low = (1 << 28) if rng.random() < 0.5 else int(rng.integers(0, 1 << 29))
        d = ((top << 29) | low) * 2.0 ** (e - 52)
        cases.append(-d if rng.random() < 0.5 else d)
    for e in range(-70, 126, 7):  # all-ones significands: the rounding carries into the exponent
        d = ((1 << 53) - 1) * 2.0 ** (e - 52)
        cases += [d, -d]
    cases += [0.0, -0.0, 1.0, -1.0, 2.0 ** -74, 2.0 ** 126]
    checked = 0
    for d in cases:
        got = split_bits(float(d))
        if got is None:
            continue
        checked += 1
        assert got == fp64_pipe(float(d)), d
    assert checked > 20000


def test_box_index_division_matches_integer_division(tmp_path):
    """Geom::box_ijk (stokes_to_gb300/csrc/internal.cuh) splits a box index with a
    multiply-high and shift instead of 64-bit division; its host form (the device form
    differs only in __umulhi) must give the quotient and remainder of the division for every
    box size the library accepts, checked here at the box's ends, around every multiple of
    n + 1 near them and at a spread of indices in between."""
    import os
    import shutil
    import subprocess

    import pytest

    nvcc = shutil.which("nvcc")
    if nvcc is None:
        pytest.skip("nvcc not available")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    src = tmp_path / "boxdiv.cu"
    src.write_text(r'''
#include <cstdio>
#include "internal.cuh"
int main() {
    long long bad = 0, checked = 0;
    for (int n = 1; n <= 1024; n++) {
        const stg::Geom g = stg::Geom::make(n);
        if (!g.dmul) { std::printf("no multiplier for n = %d\n", n); return 1; }
        const long long m = n + 1, box = g.box();
        auto check = [&](long long t) {
            if (t < 0 || t >= box) return;
            int i, j, k;
            g.box_ijk(t, i, j, k);
            checked++;
            if (k != t % m || j != (t / m) % m || i != t / (m * m)) bad++;
        };
        for (long long t = 0; t < 4 * m; t++) check(t);
        for (long long t = box - 4 * m; t < box; t++) check(t);
        for (long long q = 0; q < 4096; q++) check(q * (box / 4096) + (q * 7919) % m);
        for (long long r = 1; r < 64; r++) { check(r * m * m - 1); check(r * m * m); check(r * m - 1); }
    }
    std::printf("%lld %lld\n", checked, bad);
    return bad ? 1 : 0;
}
''')
    exe = tmp_path / "boxdiv"
    subprocess.run([nvcc, "-std=c++17", "-I", os.path.join(root, "stokes_to_gb300", "csrc"), str(src), "-o", str(exe)],
                   check=True)
    out = subprocess.run([str(exe)], stdout=subprocess.PIPE, text=True)
    assert out.returncode == 0, out.stdout
    checked, bad = map(int, out.stdout.split())
    assert checked > 1_000_000 and bad == 0
