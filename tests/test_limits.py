"""Limits of the in-memory job, checked through the C ABI.

The CPU tests call fpl_run_noalloc with jobs that its validation rejects
before any CUDA call (so they need no GPU): the reference's option checks
(STBAS bandwidth, src/evd/evd.cpp:74-91; reference date within the stack)
and this library's own limits (64 dates, 1024 window taps = 32 mask words,
rows and row ranges, missing buffers).  The GPU tests run the largest
window the limits allow, in both forms and for both SHP tests, against the
oracle, and an empty row range."""
import ctypes

import numpy as np
import pytest

from fringe_gb300 import _lib, synth

CODES = _lib.header_defines()


def _job(**kw):
    from fringe_gb300 import linker
    a = dict(nb=10, R=8, C=8, ny=2, nx=2, method="MLE", semantics="evd", mini=1, bw=-1, minn=2,
             precision="fp32", rows=None, memory=_lib.FPL_MEM_DEVICE)
    a.update(kw)
    p = ctypes.c_void_p(16) if kw.get("ptr", True) else None
    return linker._make_job(a["nb"], a["R"], a["C"], a["ny"], a["nx"], a["method"], a["semantics"], a["mini"],
                            a["bw"], a["minn"], a["precision"], a["rows"], a["memory"], p, p, p, p, p, None)


@pytest.mark.parametrize("kw,code", [
    (dict(nb=65), "FPL_ERR_UNSUPPORTED"),                    # more than 64 dates
    (dict(ny=16, nx=16), "FPL_ERR_UNSUPPORTED"),             # 33 x 33 taps > 32 mask words
    (dict(ny=-1), "FPL_ERR_OPTIONS"),
    (dict(R=0), "FPL_ERR_OPTIONS"),
    (dict(nb=0), "FPL_ERR_OPTIONS"),
    (dict(method="STBAS", bw=0), "FPL_ERR_OPTIONS"),         # evd.cpp:74-91
    (dict(method="STBAS", bw=9), "FPL_ERR_OPTIONS"),         # bw >= nbands - 1
    (dict(mini=11), "FPL_ERR_OPTIONS"),                      # reference date past the stack
    (dict(mini=0), "FPL_ERR_OPTIONS"),
    (dict(rows=(5, 3)), "FPL_ERR_OPTIONS"),                  # reversed row range
    (dict(rows=(0, 9)), "FPL_ERR_OPTIONS"),                  # past the last row
    (dict(ptr=False), "FPL_ERR_NULL"),
])
def test_validation_rejects_before_any_device_work(kw, code):
    lib = _lib.load()
    job = _job(**kw)
    assert lib.fpl_run_noalloc(ctypes.byref(job), None) == CODES[code]


def test_largest_window_is_accepted_by_validation():
    """31 x 33 = 1023 taps (32 mask words) passes validation; with no GPU the
    call then fails at its first CUDA call, not at validation.  The job's
    buffers are placeholders, so the test runs only where no GPU is visible
    (with one the call would launch kernels on them); the GPU tests below
    run that window size on real buffers."""
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("placeholder buffers: runs only where no GPU is visible")
    lib = _lib.load()
    rc = lib.fpl_run_noalloc(ctypes.byref(_job(ny=15, nx=16)), None)
    assert rc not in (CODES["FPL_ERR_UNSUPPORTED"], CODES["FPL_ERR_OPTIONS"])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_largest_window_matches_oracle(gpu_lib, precision):
    import oracle
    from fringe_gb300 import phase_link
    from tests.parity import assert_parity, compare
    stack, nmap = synth.scene("voronoi", 40, 56, 12, 15, 16, seed=1023)
    assert nmap.shape[2] == 32
    for method in ("MLE", "EVD"):
        g = phase_link(stack, nmap, (15, 16), method=method, precision=precision)
        o = oracle.run(stack, nmap, 15, 16, method=method)
        m = compare(g, o)
        assert m["valid_both"] > 1000, m
        tol = dict(phase_tol=1e-3, tcorr_tol=2e-4) if precision == "mixed" else {}
        assert_parity(m, **tol)


@pytest.mark.gpu
@pytest.mark.parametrize("method", ["KS2", "AD2"])
def test_largest_window_shp_map(gpu_lib, method):
    import oracle
    from fringe_gb300 import nmap
    stack, _ = synth.scene("voronoi", 30, 40, 12, 15, 16, seed=1024)
    g = nmap(stack, (15, 16), method=method)
    om, oc = oracle.nmap(stack, 15, 16, 0.05, method=method)
    assert np.array_equal(g["nmap"], om) and np.array_equal(g["count"], oc)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp32", "mixed"])
def test_empty_row_range_writes_nothing(gpu_lib, precision):
    from fringe_gb300 import phase_link
    stack, nmap = synth.scene("voronoi", 24, 32, 10, 3, 5, seed=3)
    out = {"phase": np.full((10, 24, 32), 7 + 7j, np.complex64), "tcorr": np.full((24, 32), 7, np.float32),
           "comp": np.full((24, 32), 7 + 7j, np.complex64)}
    phase_link(stack, nmap, (3, 5), method="MLE", precision=precision, rows=(8, 8), out=out)
    assert np.all(out["tcorr"] == 7) and np.all(out["phase"] == 7 + 7j) and np.all(out["comp"] == 7 + 7j)
