"""PS/DS merge of the integratePS workflow step (python/integratePS.py).

The oracle (oracle/integrate_ps.py) is pinned to golden vectors made by
running the reference's own integratePS2DS and getCoherence
(tests/golden/make_ps_golden.py); the GPU kernel (fpl_integrate_ps) is
checked against both.  The interferogram products are float work: NumPy's
complex64 multiply fuses multiply-adds in its vectorised loop and not in its
scalar tail, so its bits depend on the platform and array length; products
agree to 2 ulp, the PS phasors (atan2 + sincos) to 1e-6, tcorr exactly.
"""
import os

import numpy as np
import pytest

from oracle.integrate_ps import integrate_ps as oracle_merge, pairs

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden", "golden_integrate_ps.npz")


def assert_merge_close(ifg, tc, want_ifg, want_tc, ps):
    assert ifg.shape == want_ifg.shape and ifg.dtype == np.complex64
    assert np.array_equal(tc, want_tc, equal_nan=True)
    is_ps = (np.asarray(ps) == 1)[None].repeat(ifg.shape[0], 0)
    d = np.abs(ifg - want_ifg)
    scale = np.maximum(np.abs(want_ifg), np.float32(1e-30))
    ds_err = d[~is_ps] / scale[~is_ps]
    assert ds_err.size == 0 or ds_err.max() <= 2.0 ** -22, ds_err.max()
    ps_err = d[is_ps]
    assert ps_err.size == 0 or ps_err.max() <= 1e-6, ps_err.max()


def random_case(rng, nb, rows, cols, ps_frac=0.3):
    slc = (rng.standard_normal((nb, rows, cols)) + 1j * rng.standard_normal((nb, rows, cols))).astype(np.complex64)
    ds = np.exp(1j * rng.uniform(-np.pi, np.pi, (nb, rows, cols))).astype(np.complex64)
    tcorr = rng.uniform(0, 1, (rows, cols)).astype(np.float32)
    ps = (rng.uniform(0, 1, (rows, cols)) < ps_frac).astype(np.uint8)
    return ds, slc, tcorr, ps


def test_oracle_matches_reference_golden():
    g = np.load(GOLDEN)
    ifg, tc = oracle_merge(g["ds"], g["slc"], g["tcorr"], g["ps"])
    assert_merge_close(ifg, tc, g["ifg"], g["tcorr_ds_ps"], g["ps"])
    # PS pixels carry unit phasors, with angle(0) = 0 giving 1 + 0j
    assert g["ifg"][1, 0, 0] == np.complex64(1)


def test_oracle_pairs_and_edges():
    assert pairs(5, 0) == [1, 2, 3, 4] and pairs(5, 2) == [0, 1, 3, 4] and pairs(1) == []
    rng = np.random.default_rng(7)
    ds, slc, tc, ps = random_case(rng, 3, 4, 5)
    ps[0, 0] = 2                          # only 1 marks a PS pixel
    ifg, tco = oracle_merge(ds, slc, tc, ps, master=1)
    assert ifg.shape == (2, 4, 5)
    assert tco[0, 0] == tc[0, 0]
    np.testing.assert_allclose(ifg[0][ps == 0], (ds[0] * np.conj(ds[1]))[ps == 0], rtol=1e-6)


@pytest.mark.gpu
def test_gpu_matches_reference_golden():
    from fringe_gb300 import integrate_ps
    g = np.load(GOLDEN)
    out = integrate_ps(g["ds"], g["slc"], g["tcorr"], g["ps"])
    assert_merge_close(out["ifg"], out["tcorr"], g["ifg"], g["tcorr_ds_ps"], g["ps"])


@pytest.mark.gpu
@pytest.mark.parametrize("nb,rows,cols,master", [(20, 257, 311, 0), (7, 64, 96, 3), (1, 8, 8, 0), (2, 0, 16, 0)])
def test_gpu_matches_oracle(nb, rows, cols, master):
    from fringe_gb300 import integrate_ps
    rng = np.random.default_rng(100 + nb)
    ds, slc, tc, ps = random_case(rng, nb, rows, cols)
    if rows:
        slc[:, 0, :3] = 0                 # zero products on PS and DS pixels
        ds[master, 1, :3] = 0
        tc[2, :2] = np.nan
    out = integrate_ps(ds, slc, tc, ps, master=master)
    want_ifg, want_tc = oracle_merge(ds, slc, tc, ps, master=master)
    assert_merge_close(out["ifg"], out["tcorr"], want_ifg, want_tc, ps)


@pytest.mark.gpu
def test_gpu_device_tensors_and_ps_values():
    import torch
    from fringe_gb300 import integrate_ps
    rng = np.random.default_rng(11)
    ds, slc, tc, ps = random_case(rng, 5, 33, 47)
    ps16 = ps.astype(np.int16)
    ps16[0, :4] = 257                     # not 1: a DS pixel (no wrap to uint8)
    out = integrate_ps(torch.from_numpy(ds).cuda(), torch.from_numpy(slc).cuda(),
                       torch.from_numpy(tc).cuda(), torch.from_numpy(ps16).cuda())
    assert out["ifg"].is_cuda
    want_ifg, want_tc = oracle_merge(ds, slc, tc, ps16)
    assert_merge_close(out["ifg"].cpu().numpy(), out["tcorr"].cpu().numpy(), want_ifg, want_tc, ps16)
