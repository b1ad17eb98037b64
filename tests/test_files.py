"""File-level module call (fpl_process) through the reference's Python
interface (Evd / Phaselink): error codes of evd_process (CPU, they are
decided before any GPU work) and a full run against the oracle (GPU)."""
import os

import numpy as np
import pytest

import oracle
from fringe_gb300 import stackio, synth
from fringe_gb300.evdlib import Evd, Phaselink
from tests.parity import assert_parity, compare


@pytest.fixture
def scene_files(tmp_path):
    stack, nmap = synth.scene("voronoi", 40, 56, 12, 3, 5, seed=21)
    vrt = stackio.write_stack(str(tmp_path / "stack"), stack)
    wts = stackio.write_nmap(str(tmp_path / "nmap"), nmap, 3, 5)
    return stack, nmap, vrt, wts, tmp_path


def _module(cls, vrt, wts, out, **kw):
    m = cls()
    m.inputDS, m.weightsDS, m.outputFolder = vrt, wts, out
    m.halfWindowX, m.halfWindowY = 5, 3
    m.verbose = 0
    for k, v in kw.items():
        setattr(m, k, v)
    return m


def test_error_codes(scene_files):
    stack, nmap, vrt, wts, tmp = scene_files
    out = str(tmp / "out")
    assert _module(Evd, str(tmp / "missing.vrt"), wts, out).run() == 102
    assert _module(Evd, vrt, str(tmp / "missing"), out).run() == 105
    assert _module(Evd, vrt, wts, out, method="STBAS", bandWidth=0).run() == 101     # evd.cpp:78-84
    assert _module(Evd, vrt, wts, out, method="STBAS", bandWidth=11).run() == 101    # >= nbands-1
    assert _module(Evd, vrt, wts, out, halfWindowX=4).run() == 109                   # HALFWINDOWX
    # later checks overwrite earlier codes, as in evd.cpp:100-160
    assert _module(Evd, vrt, wts, out, halfWindowY=2).run() == 110
    w1 = stackio.write_nmap(str(tmp / "nmap_short"), nmap[..., :2].copy(), 3, 5)
    assert _module(Evd, vrt, w1, out).run() == 108                                   # nulong differs
    # width mismatch
    w2 = stackio.write_nmap(str(tmp / "nmap_narrow"), nmap[:, :50], 3, 5)
    assert _module(Evd, vrt, w2, out).run() == 106
    # a band without a Date in the slc domain
    txt = open(vrt).read().replace('<MDI key="Date">', '<MDI key="Dates">', 1)
    bad = str(tmp / "nodate.vrt")
    open(bad, "w").write(txt)
    assert _module(Evd, bad, wts, out).run() == 112
    # existing output folder / file
    os.makedirs(str(tmp / "exists"))
    assert _module(Evd, vrt, wts, str(tmp / "exists")).run() == 113
    open(str(tmp / "afile"), "w").write("x")
    assert _module(Evd, vrt, wts, str(tmp / "afile")).run() == 114


@pytest.mark.gpu
@pytest.mark.parametrize("cls,semantics,method", [(Evd, "evd", "MLE"), (Evd, "evd", "EVD"),
                                                  (Phaselink, "phase_link", "MLE")])
def test_module_run_matches_oracle(gpu_lib, scene_files, cls, semantics, method):
    stack, nmap, vrt, wts, tmp = scene_files
    out = str(tmp / ("out_" + semantics + method))
    # a small memsize forces several row blocks with halos (evd.cpp:169-187)
    m = _module(cls, vrt, wts, out, method=method, memsize=1, blocksize=8, minimumNeighbors=3)
    assert m.run() == 0
    dates = stackio.dates_for(stack.shape[0])
    phase = np.stack([stackio.read_envi(os.path.join(out, d + ".slc")) for d in dates])
    res = {"phase": phase, "tcorr": stackio.read_envi(os.path.join(out, "tcorr.bin")),
           "comp": stackio.read_envi(os.path.join(out, "compslc.bin"))}
    o = oracle.run(stack, nmap, 3, 5, method=method, semantics=semantics, min_neighbors=3)
    mt = compare(res, o)
    assert mt["valid_both"] > 1000, mt
    assert_parity(mt)
