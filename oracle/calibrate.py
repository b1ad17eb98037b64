#!/usr/bin/env python3
"""Speed of the oracle port against the reference-linked oracle build.

Test infrastructure only.  Where the reference tree is absent (a GPU host),
the CPU baseline can only be timed with the port (oracle/libfpl_oracle.so);
this script measures how the port's speed compares with oracle/_ref (the same
loop calling the reference's own EVWorker and LAPACK) on the same rows of the
same scene, on the same host threads, so the port's figure can be read as
the reference's.  Both libraries run the same OpenMP pixel loop with LAPACK
single-threaded (src/evd/evd.py:43 sets OPENBLAS_NUM_THREADS=1).

    OPENBLAS_NUM_THREADS=1 python oracle/calibrate.py [ROWS] [--threads T]

Prints one JSON line: px/s of each build per method and their ratio.
"""
import argparse
import json
import os
import sys
import time

os.environ.setdefault("OPENBLAS_NUM_THREADS", "1")
HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

import oracle  # noqa: E402
from fringe_gb300 import synth  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("rows", type=int, nargs="?", default=120)
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--scene", type=int, default=2048, help="scene rows = cols")
    a = ap.parse_args()
    if not oracle.build_reference():
        sys.exit("the reference-linked oracle cannot be built here (no reference tree)")
    oracle.build_port()
    stack, nmap = synth.scene("voronoi", a.scene, a.scene, 30, 5, 10, seed=1002)
    out = {"scene": "voronoi %dx%d N=30 half-window 5x10 (the headline scene)" % (a.scene, a.scene),
           "sample": "rows 0..%d (%d px)" % (a.rows, a.rows * a.scene), "threads": a.threads,
           "cpu": _cpu_model()}
    for method in ("MLE", "EVD"):
        row = {}
        for kind in ("port", "reference"):
            oracle.run(stack, nmap, 5, 10, method=method, rows=(0, 2), nthreads=a.threads, kind=kind)
            t0 = time.perf_counter()
            oracle.run(stack, nmap, 5, 10, method=method, rows=(0, a.rows), nthreads=a.threads, kind=kind)
            dt = time.perf_counter() - t0
            row[kind] = {"px_s": a.rows * a.scene / dt, "s": dt}
        row["port_over_reference"] = row["port"]["px_s"] / row["reference"]["px_s"]
        out[method] = row
    print(json.dumps(out))


def _cpu_model():
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.startswith("model name"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


if __name__ == "__main__":
    main()
