#!/usr/bin/env python3
"""Generates tests/golden/golden_phase_link.npz from the reference build of
the oracle (oracle/_ref/libfpl_ref.so: the oracle's per-pixel loop calling
the reference's own EVWorker, include/fringe/EigenLapack.hpp, and LAPACK).

Run where the reference tree is present:
    OPENBLAS_NUM_THREADS=1 python tests/golden/make_golden.py [REFERENCE_ROOT]
(REFERENCE_ROOT defaults to $FRINGE_REFERENCE_ROOT, else to the default of
oracle/build_ref.sh.)
Inputs (seeded synthetic scenes from fringe_gb300.synth) are stored with the
outputs, so the fixtures do not depend on the generator's reproducibility.
Phases are stored as float32 angles.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from fringe_gb300 import synth  # noqa: E402

# name: (kind, rows, cols, nbands, ny, nx, seed, [(method, semantics, extra)])
CASES = {
    "uniform10": ("uniform", 20, 20, 10, 5, 5, 1001,
                  [("MLE", "evd", {}), ("EVD", "evd", {}), ("MLE", "phase_link", {})]),
    "voronoi30": ("voronoi", 16, 24, 30, 5, 10, 1002,
                  [("MLE", "evd", {}), ("EVD", "evd", {}), ("STBAS", "evd", {"band_width": 5}),
                   ("MLE", "phase_link", {"min_neighbors": 5}),
                   ("MLE", "evd", {"mini_stack_count": 3})]),
    "illcond64": ("illcond", 12, 16, 64, 5, 10, 1003, [("MLE", "evd", {}), ("EVD", "evd", {}),
                                                       ("STBAS", "evd", {"band_width": 10}),
                                                       ("MLE", "phase_link", {})]),
    # edge depths: one date (tcorr 0/0 = NaN), two, and 17 (padded date pairs; -2 and -4 codes)
    "depth1": ("voronoi", 12, 16, 1, 2, 3, 101, [("MLE", "evd", {}), ("EVD", "evd", {})]),
    "depth2": ("voronoi", 12, 16, 2, 2, 3, 102, [("MLE", "evd", {}), ("EVD", "evd", {})]),
    "depth17": ("voronoi", 12, 16, 17, 2, 3, 117, [("MLE", "evd", {}), ("EVD", "evd", {}),
                                                   ("MLE", "phase_link", {})]),
    # |C| indefinite in every pixel: code -4 (evd), the EVD fall-back (phase_link)
    "indefabs6": ("indefabs", 12, 16, 6, 5, 10, 56, [("MLE", "evd", {}), ("MLE", "phase_link", {})]),
    "indefabs24": ("indefabs", 12, 16, 24, 5, 10, 74, [("MLE", "evd", {}), ("MLE", "phase_link", {})]),
}


def variant_key(case, method, sem, extra):
    k = "%s/%s_%s" % (case, method, sem)
    for a, b in sorted(extra.items()):
        k += "_%s%d" % (a, b)
    return k


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else None     # else FRINGE_REFERENCE_ROOT
    if not oracle.build_reference(ref_root):
        sys.exit("reference build of the oracle is unavailable")
    out = {}
    for case, (kind, R, C, N, ny, nx, seed, variants) in CASES.items():
        stack, nmap = synth.scene(kind, R, C, N, ny, nx, seed=seed)
        out[case + "/stack"] = stack
        out[case + "/nmap"] = nmap
        out[case + "/shape"] = np.array([R, C, N, ny, nx], np.int32)
        for method, sem, extra in variants:
            r = oracle.run(stack, nmap, ny, nx, method=method, semantics=sem, kind="reference", **extra)
            k = variant_key(case, method, sem, extra)
            out[k + "/phase_angle"] = np.angle(r["phase"]).astype(np.float32)
            out[k + "/phase_zero"] = (r["phase"] == 0).all(axis=0)
            out[k + "/tcorr"] = r["tcorr"]
            out[k + "/comp"] = r["comp"]
    np.savez_compressed(os.path.join(HERE, "golden_phase_link.npz"), **out)
    print("wrote", len(out), "arrays")


if __name__ == "__main__":
    main()
