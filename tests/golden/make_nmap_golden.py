#!/usr/bin/env python3
"""Generates tests/golden/golden_nmap.npz from the reference build of the
nmap oracle (oracle/_ref/libfpl_ref.so: the oracle's nmap loop calling the
reference's own KS2sample::test and AD2unique::test,
src/nmap/KS2sample.hpp:96-144 and src/nmap/AD2unique.hpp:270-347).

Run where the reference tree is present:
    python tests/golden/make_nmap_golden.py [REFERENCE_ROOT]
(REFERENCE_ROOT defaults to $FRINGE_REFERENCE_ROOT, else to the default of
oracle/build_ref.sh.)  Stored: seeded sample pairs with the probability of
each test for both argument orders, and the SHP maps of two small scenes
(one with quantised amplitudes, so that samples share values) for both
methods.  Inputs are stored with the outputs.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from fringe_gb300 import synth  # noqa: E402


def main():
    root = sys.argv[1] if len(sys.argv) > 1 else None
    if not oracle.build_reference(root):
        sys.exit("reference build of the oracle is unavailable")
    out = {}
    rng = np.random.default_rng(2024)
    ns = (2, 3, 5, 10, 16, 30, 45, 64)
    for n in ns:
        a = np.zeros((64, n), np.float32)
        b = np.zeros((64, n), np.float32)
        for k in range(64):
            x = rng.rayleigh(1.0, n)
            y = rng.rayleigh(1.0, n) * rng.uniform(0.5, 2.0)
            if k % 3 == 0:                               # shared values
                x, y = np.round(x * 3) / 3, np.round(y * 3) / 3
            a[k], b[k] = np.sort(x.astype(np.float32)), np.sort(y.astype(np.float32))
        out["pairs%d/a" % n], out["pairs%d/b" % n] = a, b
        for m, f in (("ks2", oracle.ks2), ("ad2", oracle.ad2)):
            out["pairs%d/%s_ab" % (n, m)] = np.array([f(a[k], b[k], "reference") for k in range(64)])
            out["pairs%d/%s_ba" % (n, m)] = np.array([f(b[k], a[k], "reference") for k in range(64)])
    for name, kind, R, C, N, ny, nx, seed, quant in (("voronoi", "voronoi", 20, 28, 12, 3, 5, 9, False),
                                                      ("ties", "voronoi", 18, 24, 10, 2, 4, 13, True)):
        stack, _ = synth.scene(kind, R, C, N, ny, nx, seed=seed)
        if quant:
            stack = (np.round(stack.real * 2) / 2 + 1j * np.round(stack.imag * 2) / 2).astype(np.complex64)
        out[name + "/stack"] = stack
        out[name + "/shape"] = np.array([R, C, N, ny, nx], np.int32)
        for m in ("KS2", "AD2"):
            mp, cnt = oracle.nmap(stack, ny, nx, 0.05, kind="reference", method=m)
            out["%s/%s_nmap" % (name, m)] = mp
            out["%s/%s_count" % (name, m)] = cnt
    np.savez_compressed(os.path.join(HERE, "golden_nmap.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
