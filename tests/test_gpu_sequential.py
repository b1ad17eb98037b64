"""Sequential estimator on the GPU against the oracle run through the same
ministack loop (src/sequential/sequential.py:193-254) and the wrapped datum
adjustment (python/adjustMiniStacks.py:203-223)."""
import os

import numpy as np
import pytest

import oracle
from fringe_gb300 import synth
from tests.parity import assert_parity, compare

pytestmark = pytest.mark.gpu


def _oracle_sequential(stack, nmap, ny, nx, size, method="MLE"):
    nd = stack.shape[0]
    comps, minis, count, i0 = [], [], 0, 0
    while i0 < nd:
        count += 1
        i1 = min(i0 + size, nd)
        ms = np.concatenate([np.stack(comps), stack[i0:i1]]) if comps else stack[i0:i1]
        o = oracle.run(ms, nmap, ny, nx, method=method, mini_stack_count=count)
        minis.append(o)
        comps.append(o["comp"])
        i0 += size
    cs = np.stack(comps)
    datum = oracle.run(cs, nmap, ny, nx, method=method, mini_stack_count=1)
    adj = np.empty_like(stack)
    i0 = 0
    for k, o in enumerate(minis):
        i1 = min(i0 + size, nd)
        own = o["phase"][-(i1 - i0):].astype(np.complex128)
        adj[i0:i1] = (own * datum["phase"][k].astype(np.complex128)).astype(np.complex64)
        i0 += size
    return minis, cs, datum, adj


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_sequential_matches_oracle(gpu_lib, precision):
    from fringe_gb300.sequential import sequential
    stack, nmap = synth.scene("voronoi", 24, 40, 23, 3, 5, seed=2023)
    g = sequential(stack, nmap, (3, 5), mini_stack_size=8, precision=precision)
    minis, cs, datum, adj = _oracle_sequential(stack, nmap, 3, 5, 8)
    assert [(m["count"], m["start"], m["end"]) for m in g["ministacks"]] == [(1, 0, 8), (2, 8, 16), (3, 16, 23)]
    for gm, om in zip(g["ministacks"], minis):
        assert gm["phase"].shape == om["phase"].shape
        assert_parity(compare(gm, om), phase_tol=1e-3, tcorr_tol=2e-4)
    assert_parity(compare(g["datum"], datum), phase_tol=1e-3, tcorr_tol=2e-4)
    valid = np.abs(adj).sum(axis=0) > 0
    d = np.angle(g["adjusted"][:, valid] * np.conj(adj[:, valid]))
    assert np.sqrt(np.mean(d ** 2)) < 1e-3


def test_adjust_kernel_exact(gpu_lib):
    """fpl_adjust_wrapped: complex product in double, rounded once."""
    import ctypes
    import torch
    from fringe_gb300 import _lib
    rng = np.random.default_rng(4)
    ph = (rng.standard_normal((3, 17, 9)) + 1j * rng.standard_normal((3, 17, 9))).astype(np.complex64)
    dt = (rng.standard_normal((17, 9)) + 1j * rng.standard_normal((17, 9))).astype(np.complex64)
    tp, td = torch.from_numpy(ph).cuda(), torch.from_numpy(dt).cuda()
    out = torch.empty_like(tp)
    ctx = _lib.context(0)
    _lib.check(_lib.load().fpl_adjust_wrapped(ctx.handle, ctypes.c_void_p(tp.data_ptr()),
                                              ctypes.c_void_p(td.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                              3, 17 * 9, None), ctx.handle)
    torch.cuda.synchronize()
    want = (ph.astype(np.complex128) * dt.astype(np.complex128)).astype(np.complex64)
    assert np.array_equal(out.cpu().numpy(), want)


def test_sequential_file_level_matches_in_memory(gpu_lib, tmp_path):
    from fringe_gb300 import stackio
    from fringe_gb300.sequential import main, sequential
    stack, nmap = synth.scene("voronoi", 20, 28, 12, 2, 3, seed=7)
    dates = stackio.dates_for(12)
    root = tmp_path / "in"
    for b, d in enumerate(dates):
        os.makedirs(root / d)
        slc = str(root / d / (d + ".slc"))
        np.ascontiguousarray(stack[b], dtype="<c8").tofile(slc)
        with open(slc + ".vrt", "w") as f:
            f.write('<VRTDataset rasterXSize="28" rasterYSize="20">\n  <VRTRasterBand dataType="CFloat32" '
                    'band="1" subClass="VRTRawRasterBand">\n    <sourceFilename>%s</sourceFilename>\n'
                    '    <ImageOffset>0</ImageOffset>\n    <PixelOffset>8</PixelOffset>\n'
                    '    <LineOffset>224</LineOffset>\n    <ByteOrder>LSB</ByteOrder>\n'
                    '  </VRTRasterBand>\n</VRTDataset>\n' % slc)
    wts = stackio.write_nmap(str(tmp_path / "nmap.bin"), nmap, 2, 3)
    out = tmp_path / "out"
    assert main(["-i", str(root), "-w", wts, "-o", str(out), "-x", "3", "-y", "2", "-s", "5"]) == 0
    g = sequential(stack, nmap, (2, 3), mini_stack_size=5)
    spans = [(0, 5), (5, 10), (10, 12)]
    for k, (i0, i1) in enumerate(spans):
        ev = out / "miniStacks" / (dates[i0] + "_" + dates[i1 - 1]) / "EVD"
        m = g["ministacks"][k]
        names = [os.path.basename(p)[:-4] for p in sorted(map(str, ev.glob("*.slc")))]
        assert len(names) == m["phase"].shape[0]
        for d in range(i0, i1):
            ph = stackio.read_envi(str(ev / (dates[d] + ".slc")))
            assert np.array_equal(ph, m["phase"][k + d - i0])
        assert np.array_equal(stackio.read_envi(str(ev / "tcorr.bin")), m["tcorr"])
        comp = stackio.read_envi(str(out / "compressedSlc" / dates[i1 - 1] / (dates[i1 - 1] + ".slc")))
        assert np.array_equal(comp, m["comp"])
    dev = out / "Datum_connection" / "EVD"
    for k, (i0, i1) in enumerate(spans):
        assert np.array_equal(stackio.read_envi(str(dev / (dates[i1 - 1] + ".slc"))), g["datum"]["phase"][k])
