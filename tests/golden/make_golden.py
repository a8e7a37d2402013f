"""Generate tests/golden/*.npz from the reference's own fieldize.cpp and
powerspectrum.c, compiled in this repository's oracle/_ref (see oracle/Makefile).

Run where the reference sources exist:  python tests/golden/make_golden.py
The FFT between deposit and binning is numpy's FP64 pocketfft (FFTW's r2c
convention); FFTW itself is not installed.

Fixtures:
  fieldize.npz   CIC grids of small particle sets (fieldize.cpp:46)
  power.npz      P(k), counts, keffs of those sets (powerspectrum.c:35)
  counts.npz     weighted mode counts / keffs for many (dims, nrbins)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle import oracle as O  # noqa: E402

FIELDIZE_CASES = [
    # name, dims, box, n, seed, variable masses, uniform mass, extra
    ("n5_testcpp", 5, 10.0, 10, None, True, 10.0, 1),
    ("n8_var", 8, 100.0, 600, 11, True, 0.0, 1),
    ("n16_uni", 16, 25000.0, 5000, 12, False, 0.5, 1),
    ("n16_extra0", 16, 1.0, 700, 13, False, 2.0, 0),
    ("n33_uni", 33, 3000.0, 9000, 14, False, 1.0e-2, 1),
    ("n32_var", 32, 50000.0, 8000, 15, True, 0.0, 1),
]

POWER_CASES = [
    # name, dims, box, n, seed, variable masses, mass, nrbins
    ("p4_b10", 4, 10.0, 64, 21, False, 1.0, 10),
    ("p5_b7", 5, 10.0, 200, 22, True, 0.0, 7),
    ("p8_b10", 8, 100.0, 512, 23, False, 1.0, 10),
    ("p16_b16", 16, 1000.0, 4096, 24, True, 0.0, 16),
    ("p32_b64", 32, 25000.0, 20000, 25, False, 1.0e-2, 64),
    ("p64_b64", 64, 100000.0, 60000, 26, False, 1.0, 64),
]

COUNT_DIMS = [2, 3, 4, 5, 6, 7, 8, 9, 10, 12, 15, 16, 17, 24, 31, 32, 48, 64, 100, 128, 200, 256]


def particles(n, box, seed, var):
    rng = np.random.default_rng(seed)
    pos = (rng.random((n, 3)) * box).astype(np.float32)
    masses = (rng.random(n) * 2.0 + 0.1).astype(np.float32) if var else None
    return pos, masses


def main():
    ref = O.ref()
    if ref is None:
        raise SystemExit("reference sources not found; cannot regenerate golden fixtures")
    fz = {}
    for name, dims, box, n, seed, var, mass, extra in FIELDIZE_CASES:
        if seed is None:  # test.cpp:31-50 inputs
            pos = (np.arange(3 * n) / 3.0).astype(np.float32).reshape(n, 3)
            masses = np.full(n, 10.0, dtype=np.float32)
        else:
            pos, masses = particles(n, box, seed, var)
        fdims = 2 * (dims // 2 + extra)
        grid = np.zeros(dims * dims * fdims)
        ref.fieldize(box, dims, grid, pos, masses, mass, extra)
        fz[f"{name}/meta"] = np.array([dims, box, n, extra, mass], dtype=np.float64)
        fz[f"{name}/pos"] = pos
        if masses is not None:
            fz[f"{name}/masses"] = masses
        fz[f"{name}/grid"] = grid
    np.savez_compressed(os.path.join(HERE, "fieldize.npz"), **fz)

    pw = {}
    for name, dims, box, n, seed, var, mass, nrbins in POWER_CASES:
        pos, masses = particles(n, box, seed, var)
        grid = O.zeros_grid(dims)
        ref.fieldize(box, dims, grid, pos, masses, mass, 1)
        f = O.rfft_padded(grid)
        m = O.total_mass(n, masses, mass)
        p, c, k = ref.powerspectrum(dims, f, f, nrbins, m, m)
        pw[f"{name}/meta"] = np.array([dims, box, n, mass, nrbins, m], dtype=np.float64)
        pw[f"{name}/pos"] = pos
        if masses is not None:
            pw[f"{name}/masses"] = masses
        pw[f"{name}/power"] = p
        pw[f"{name}/count"] = c
        pw[f"{name}/keffs"] = k
    np.savez_compressed(os.path.join(HERE, "power.npz"), **pw)

    ct = {}
    for dims in COUNT_DIMS:
        zero = np.zeros((dims, dims, dims // 2 + 1), dtype=np.complex128)
        for nrbins in sorted({1, 2, 10, 64, dims, 2 * dims}):
            _, c, k = ref.powerspectrum(dims, zero, zero, nrbins, 1.0, 1.0)
            ct[f"{dims}_{nrbins}/count"] = c
            ct[f"{dims}_{nrbins}/keffs"] = k
    np.savez_compressed(os.path.join(HERE, "counts.npz"), **ct)
    print("wrote", len(fz), len(pw), len(ct), "arrays")


if __name__ == "__main__":
    main()
