"""Host logic of the sequential estimator (no GPU): the ministack loop, the
reference's command line, and the VRTs written for each ministack."""
import os
import re

import numpy as np
import pytest

from fringe_gb300 import sequential as seq


def _reference_loop(ndates, size):
    # the while loop of src/sequential/sequential.py:193-254, restated
    out, count, ind = [], 0, 0
    while ind < ndates:
        count += 1
        end = min(ind + size, ndates)
        out.append((count, ind, end))
        ind += size
    return out


@pytest.mark.parametrize("ndates,size", [(25, 10), (20, 10), (7, 10), (5, 1), (1, 3), (31, 7)])
def test_ministack_plan(ndates, size):
    assert seq.ministack_plan(ndates, size) == _reference_loop(ndates, size)


def test_ministack_plan_rejects_empty_ministacks():
    with pytest.raises(ValueError):
        seq.ministack_plan(10, 0)


def test_command_line_defaults_match_the_reference():
    a = seq.cmd_line_parser(["-i", "in", "-w", "w.bin", "-o", "out"])
    assert (a.linesPerBlock, a.memorySize, a.halfWindowX, a.halfWindowY, a.minNeighbors,
            a.miniStackSize, a.forceprocessing, a.bbox) == (64, 2048, 29, 9, 5, 10, False, None)


def _slc_tree(root, dates, rows, cols, seed=0):
    rng = np.random.default_rng(seed)
    for d in dates:
        os.makedirs(os.path.join(root, d))
        slc = os.path.join(root, d, d + ".slc")
        (rng.standard_normal((rows, cols)) + 1j * rng.standard_normal((rows, cols))).astype("<c8").tofile(slc)
        with open(slc + ".vrt", "w") as f:
            f.write('<VRTDataset rasterXSize="%d" rasterYSize="%d">\n  <VRTRasterBand dataType="CFloat32" '
                    'band="1" subClass="VRTRawRasterBand">\n    <sourceFilename>%s</sourceFilename>\n'
                    '  </VRTRasterBand>\n</VRTDataset>\n' % (cols, rows, slc))


def test_stack_vrts(tmp_path):
    dates = ["20220113", "20220101", "20220125"]
    _slc_tree(str(tmp_path / "in"), dates, 6, 9)
    st = seq.SlcStack.gather(str(tmp_path / "in"), bbox=(1, 5, 2, 8))
    assert st.dates == sorted(dates)
    st.apply_bbox = [False, True, True]
    vrt = st.write_vrts(str(tmp_path / "out"))
    text = open(vrt).read()
    assert re.search(r'<VRTDataset rasterXSize="6" rasterYSize="4">', text)
    assert re.findall(r'<MDI key="Date">(\d+)</MDI>', text) == sorted(dates)
    rects = re.findall(r'<SrcRect xOff="(\d+)" yOff="(\d+)" xSize="(\d+)" ySize="(\d+)"/>', text)
    assert rects == [("0", "0", "9", "6"), ("2", "1", "6", "4"), ("2", "1", "6", "4")]
    for d in dates:
        per = open(str(tmp_path / "out" / "slcs" / (d + ".vrt"))).read()
        assert "VRTRawRasterBand" in per and "<LineOffset>72</LineOffset>" in per


def test_bbox_from_vrt(tmp_path):
    p = tmp_path / "b.vrt"
    p.write_text('<VRTDataset><VRTRasterBand><SimpleSource><SrcRect xOff="3" yOff="4" xSize="10" '
                 'ySize="20"/></SimpleSource></VRTRasterBand></VRTDataset>')
    assert seq._bbox_from_vrt(str(p)) == (4, 24, 3, 13)
