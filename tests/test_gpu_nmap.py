"""SHP map on the GPU (fpl_nmap) against the oracle's restatement of the
nmap module: bit-exact maps and counts."""
import numpy as np
import pytest

import oracle
from fringe_gb300 import synth

pytestmark = pytest.mark.gpu


def _check(stack, ny, nx, prob=0.05, mask=None, amp_const=None, method="KS2"):
    from fringe_gb300 import nmap
    g = nmap(stack, (ny, nx), prob=prob, mask=mask, amp_const=amp_const, method=method)
    o_map, o_cnt = oracle.nmap(stack, ny, nx, prob, mask=mask, amp_const=amp_const, method=method)
    assert np.array_equal(g["count"], o_cnt), int((g["count"] != o_cnt).sum())
    assert np.array_equal(g["nmap"], o_map)
    return g


@pytest.mark.parametrize("R,C,N,ny,nx,seed", [
    (40, 72, 30, 5, 10, 1002),
    (33, 45, 10, 5, 5, 1001),
    (20, 40, 45, 3, 5, 45),
    (17, 35, 16, 2, 3, 16),
    (17, 35, 17, 2, 3, 17),
    (12, 20, 64, 1, 2, 64),
    (10, 12, 1, 1, 1, 1),
])
@pytest.mark.parametrize("method", ["KS2", "AD2"])
def test_nmap_matches_oracle(gpu_lib, R, C, N, ny, nx, seed, method):
    stack, _ = synth.scene("voronoi", R, C, N, ny, nx, seed=seed)
    g = _check(stack, ny, nx, method=method)
    assert (g["count"] > 0).all()                     # every pixel valid: centre bit set


@pytest.mark.parametrize("method", ["KS2", "AD2"])
def test_nmap_mask_constants_invalid_pixels_and_ties(gpu_lib, method):
    rng = np.random.default_rng(5)
    stack, _ = synth.scene("voronoi", 30, 40, 20, 3, 4, seed=8)
    stack[:, 5, 6] = 0                                # zero amplitude in every date
    stack[3, 9, 9] = np.nan                           # NaN in one date
    stack[:, 20:24, 30:36] = np.round(stack[:, 20:24, 30:36].real * 2) / 2   # ties
    mask = (rng.random((30, 40)) > 0.05).astype(np.uint8)
    const = rng.uniform(0.5, 2.0, 20)
    g = _check(stack, 3, 4, prob=0.1, mask=mask, amp_const=const, method=method)
    assert g["count"][5, 6] == 0 and g["count"][9, 9] == 0


@pytest.mark.parametrize("method", ["KS2", "AD2"])
def test_nmap_thresholds(gpu_lib, method):
    stack, _ = synth.scene("voronoi", 24, 30, 30, 2, 4, seed=11)
    for prob in (0.0, 0.01, 0.5, 0.9, 1.0):
        _check(stack, 2, 4, prob=prob, method=method)


def test_ad2_ties_use_the_reference_argument_order(gpu_lib):
    """Quantised amplitudes make neighbours share values, where the AD test
    depends on which pixel is the first sample: the map still equals the
    reference's (the golden maps its own tests wrote) bit for bit."""
    import os
    g = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_nmap.npz"))
    from fringe_gb300 import nmap
    for name in ("voronoi", "ties"):
        R, C, N, ny, nx = [int(x) for x in g[name + "/shape"]]
        for m in ("KS2", "AD2"):
            d = nmap(g[name + "/stack"], (ny, nx), method=m)
            assert np.array_equal(d["nmap"], g["%s/%s_nmap" % (name, m)]), (name, m)
            assert np.array_equal(d["count"], g["%s/%s_count" % (name, m)]), (name, m)
    # a scene where every neighbour pair shares values
    stack, _ = synth.scene("voronoi", 26, 34, 20, 3, 5, seed=31)
    q = (np.round(np.abs(stack) * 2) / 2).astype(np.complex64)
    _check(q, 3, 5, method="AD2")


def test_nmap_device_path_feeds_phase_linking(gpu_lib):
    torch = pytest.importorskip("torch")
    from fringe_gb300 import nmap, phase_link
    stack, _ = synth.scene("voronoi", 40, 48, 30, 5, 10, seed=21)
    d = nmap(torch.from_numpy(stack).cuda(), (5, 10))
    o_map, o_cnt = oracle.nmap(stack, 5, 10, 0.05)
    assert np.array_equal(d["nmap"].cpu().numpy().view(np.uint32), o_map)
    assert np.array_equal(d["count"].cpu().numpy(), o_cnt)
    g = phase_link(torch.from_numpy(stack).cuda(), d["nmap"], (5, 10), method="MLE")
    h = phase_link(stack, o_map, (5, 10), method="MLE")
    assert np.array_equal(g["tcorr"].cpu().numpy(), h["tcorr"], equal_nan=True)
