#!/usr/bin/env python3
"""Generates tests/golden/golden_integrate_ps.npz by running the reference's
own PS/DS merge (python/integratePS.py: integratePS2DS and getCoherence, with
the single-master pairs of python/Network.py) on a small seeded case.

The reference module imports GDAL and ISCE at the top; neither is needed by
these two functions, which only call ReadAsArray / GetRasterBand /
WriteArray on the datasets they are given.  The script registers empty
stand-ins for those modules and passes in-memory datasets with the same
methods.  Run where the reference tree is present:
    python tests/golden/make_ps_golden.py REFERENCE_ROOT
(or with FRINGE_REFERENCE_ROOT set).
"""
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("FRINGE_REFERENCE_ROOT")
if not REF:
    sys.exit("usage: make_ps_golden.py REFERENCE_ROOT (or set FRINGE_REFERENCE_ROOT)")


class _Band:
    def __init__(self, arr):
        self.a = arr

    def ReadAsArray(self, x0, y0, xoff, yoff):
        return self.a[y0:y0 + yoff, x0:x0 + xoff].copy()

    def WriteArray(self, data, x0, y0):
        self.a[y0:y0 + data.shape[0], x0:x0 + data.shape[1]] = data


class _Dataset:
    """bands: [nbands, rows, cols] array (band b is GetRasterBand(b + 1))."""

    def __init__(self, bands):
        self.b = bands
        self.RasterCount, self.RasterYSize, self.RasterXSize = bands.shape

    def GetRasterBand(self, k):
        return _Band(self.b[k - 1])

    def ReadAsArray(self, x0, y0, xoff, yoff):
        return self.b[0, y0:y0 + yoff, x0:x0 + xoff].copy()


def load_reference():
    for name in ("osgeo", "isce", "isceobj"):
        sys.modules.setdefault(name, types.ModuleType(name))
    sys.modules["osgeo"].gdal = types.ModuleType("gdal")
    sys.path.insert(0, os.path.join(REF, "python"))
    import integratePS  # noqa: E402
    from Network import Network  # noqa: E402
    return integratePS, Network


def main():
    ips, Network = load_reference()
    rng = np.random.default_rng(2024)
    nb, rows, cols = 6, 23, 37
    slc = (rng.standard_normal((nb, rows, cols)) + 1j * rng.standard_normal((nb, rows, cols))).astype(np.complex64)
    ph = rng.uniform(-np.pi, np.pi, (nb, rows, cols))
    ds = np.exp(1j * ph).astype(np.complex64)
    # zeros and signed zeros in both stacks (angle / product edge cases)
    slc[2, 0, :5] = 0
    slc[0, 1, :3] = np.complex64(complex(-0.0, 0.0))
    slc[3, 1, 3:6] = np.complex64(complex(-0.0, -0.0))
    ds[1, 2, :4] = 0
    tcorr = rng.uniform(0, 1, (rows, cols)).astype(np.float32)
    tcorr[3, :3] = np.nan
    ps = (rng.uniform(0, 1, (rows, cols)) < 0.3).astype(np.uint8)
    ps[4, :6] = 2            # only value 1 marks a PS pixel
    ps[0:2, :8] = 1          # the zero samples above sit on PS pixels

    lines_per_block = 10     # several blocks, the last one short (main(), :195-201)
    nblocks = int(rows / lines_per_block)
    if nblocks == 0:
        nblocks = 1
    elif rows % (nblocks * lines_per_block) != 0:
        nblocks += 1

    dates = ["2020%02d%02d" % (1 + k // 28, 1 + k % 28) for k in range(nb)]
    net = Network()
    net.dateList = sorted(dates)
    net.single_master()
    ds_sets = {d: _Dataset(ds[k:k + 1]) for k, d in enumerate(dates)}
    dsSlc = _Dataset(slc)
    dsTcor = _Dataset(tcorr[None])
    psSet = _Dataset(ps[None])
    ifg = np.zeros((len(net.pairsDates), rows, cols), np.complex64)
    for q, pair in enumerate(net.pairsDates):
        di, dj = pair.split("-")
        bi, bj = net.dateList.index(di) + 1, net.dateList.index(dj) + 1
        out = _Dataset(ifg[q:q + 1])
        ips.integratePS2DS(ds_sets[di], ds_sets[dj], dsSlc, dsTcor, psSet, out,
                           nblocks, lines_per_block, bi, bj)
    tc_out = np.zeros((1, rows, cols), np.float32)
    ips.getCoherence(dsTcor, psSet, _Dataset(tc_out), cols, rows, nblocks, lines_per_block)
    np.savez_compressed(os.path.join(HERE, "golden_integrate_ps.npz"), ds=ds, slc=slc, tcorr=tcorr,
                        ps=ps, ifg=ifg, tcorr_ds_ps=tc_out[0], numpy_version=np.__version__)
    print("wrote golden_integrate_ps.npz:", ifg.shape, "pairs", net.pairsDates)


if __name__ == "__main__":
    main()
