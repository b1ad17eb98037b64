"""CPU oracle for the PS/DS merge of python/integratePS.py -- TEST
INFRASTRUCTURE ONLY (only tests/ may import it).

Restates, in NumPy, what python/integratePS.py computes per pixel once its
GDAL reads are done:

* getCoherence (python/integratePS.py:129-152): the temporal coherence with
  PS pixels (map value 1) set to 0.95;
* the single-master network (python/Network.py:95-104): pairs
  (master, j) for every other date j, in date order;
* integratePS2DS (python/integratePS.py:94-126) for each pair: the product
  ds_j * conj(ds_master) of the phase-linked stack, replaced at PS pixels by
  exp(1j * angle(slc_j * conj(slc_master))) of the original SLCs
  (get_fullres_ifgram, python/integratePS.py:66-75).

The reference works on blocks of lines; every operation is per pixel, so the
blocking does not change any value and is not restated.  Pinned against
tests/golden/golden_integrate_ps.npz, made by running the reference's own
integratePS2DS and getCoherence (tests/golden/make_ps_golden.py).
"""
import numpy as np


def pairs(nbands, master=0):
    """Second dates of the single-master pairs, in band order."""
    return [j for j in range(nbands) if j != master]


def integrate_ps(ds, slc, tcorr, ps, master=0):
    """ds, slc: complex64 [nbands, rows, cols]; tcorr: float32 [rows, cols];
    ps: [rows, cols], 1 = PS pixel.  Returns (ifg complex64
    [nbands-1, rows, cols] for pairs (master, j), tcorr_ds_ps float32)."""
    ds = np.asarray(ds, dtype=np.complex64)
    slc = np.asarray(slc, dtype=np.complex64)
    is_ps = np.asarray(ps) == 1
    tc = np.array(tcorr, dtype=np.float32, copy=True)
    tc[is_ps] = 0.95                                     # integratePS.py:150
    out = []
    for j in pairs(ds.shape[0], master):
        ifg = ds[j] * np.conjugate(ds[master])           # integratePS.py:118
        full = np.exp(1j * np.angle(slc[j] * np.conjugate(slc[master])))   # :72-73
        ifg[is_ps] = full[is_ps]                         # integratePS.py:121
        out.append(ifg.astype(np.complex64))
    return np.stack(out) if out else np.zeros((0,) + tc.shape, np.complex64), tc
