"""Row bands on the GPU: each band computed from only its own rows (plus the
apron) gives the whole scene's results bit for bit, in both forms."""
import numpy as np
import pytest

from fringe_gb300 import synth
from fringe_gb300.shard import phase_link_band, row_bands

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_bands_equal_whole_scene(gpu_lib, precision):
    from fringe_gb300 import phase_link
    stack, nmap = synth.scene("voronoi", 61, 40, 30, 5, 10, seed=61)
    whole = phase_link(stack, nmap, (5, 10), method="MLE", precision=precision)
    for b in row_bands(61, 3, 5):
        out = phase_link_band(np.ascontiguousarray(stack[:, b.s0:b.s1]), np.ascontiguousarray(nmap[b.s0:b.s1]),
                              (5, 10), b, method="MLE", precision=precision)
        lr0, lr1 = b.local_rows
        for key in ("phase", "tcorr", "comp"):
            got = out[key][..., lr0:lr1, :]
            want = whole[key][..., b.r0:b.r1, :]
            assert np.array_equal(got, want, equal_nan=True), (key, b)
