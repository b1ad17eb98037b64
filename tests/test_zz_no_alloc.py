"""The allocation-free entry point, fpl_run_noalloc, against fpl_run_async.

fpl_run_noalloc exists for callers that cannot call cudaMalloc (their device
memory belongs to another allocator, or they must not allocate once
running); its scratch is a fixed array inside the library.  These tests call
it through the C ABI on caller-owned CUDA buffers, twice in a row on the same
array, and compare each result with the context-based fpl_run_async under
the parity tolerances used elsewhere.  This file is named so that pytest
collects it last.
"""
import ctypes

import numpy as np
import pytest

from fringe_gb300 import synth
from tests.parity import assert_parity, compare

pytestmark = pytest.mark.gpu


def _outputs(torch, nb, R, C):
    return {"phase": torch.zeros((nb, R, C), dtype=torch.complex64, device="cuda"),
            "tcorr": torch.zeros((R, C), dtype=torch.float32, device="cuda"),
            "comp": torch.zeros((R, C), dtype=torch.complex64, device="cuda")}


def _noalloc(lib, linker, torch, ts, tn, ny, nx, method, semantics, rows=None, out=None):
    from fringe_gb300 import _lib
    nb, R, C = ts.shape
    out = out if out is not None else _outputs(torch, nb, R, C)
    job = linker._make_job(nb, R, C, ny, nx, method, semantics, 1, -1, 2, "fp32", rows,
                           _lib.FPL_MEM_DEVICE, ts.data_ptr(), tn.data_ptr(),
                           out["phase"].data_ptr(), out["tcorr"].data_ptr(),
                           out["comp"].data_ptr(), None)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.fpl_run_noalloc(ctypes.byref(job), ctypes.c_void_p(stream))
    assert rc == 0, lib.fpl_error_string(rc)
    torch.cuda.synchronize()
    return out


def _host(out):
    return {k: v.cpu().numpy() for k, v in out.items()}


@pytest.mark.parametrize("method,semantics", [("MLE", "evd"), ("EVD", "evd"), ("MLE", "phase_link")])
def test_noalloc_matches_context_run_twice(gpu_lib, method, semantics):
    torch = pytest.importorskip("torch")
    from fringe_gb300 import linker
    stack, nmap = synth.scene("voronoi", 48, 80, 30, 5, 10, seed=77)
    ts = torch.from_numpy(stack).cuda()
    tn = torch.from_numpy(nmap.view(np.int32)).cuda()
    ref = linker.phase_link(ts, tn, (5, 10), method=method, semantics=semantics)
    torch.cuda.synchronize()
    ref = _host(ref)
    for _ in range(2):
        got = _host(_noalloc(gpu_lib, linker, torch, ts, tn, 5, 10, method, semantics))
        m = compare(got, ref)
        assert m["valid_both"] > 1000, m
        assert_parity(m)


def test_noalloc_row_ranges_equal_whole_scene(gpu_lib):
    """A job split into row ranges (the way to run a scene larger than the
    array) gives the whole-scene call's results bit for bit."""
    torch = pytest.importorskip("torch")
    from fringe_gb300 import linker
    stack, nmap = synth.scene("voronoi", 48, 80, 30, 5, 10, seed=78)
    ts = torch.from_numpy(stack).cuda()
    tn = torch.from_numpy(nmap.view(np.int32)).cuda()
    whole = _host(_noalloc(gpu_lib, linker, torch, ts, tn, 5, 10, "MLE", "evd"))
    out = _outputs(torch, *ts.shape)
    _noalloc(gpu_lib, linker, torch, ts, tn, 5, 10, "MLE", "evd", rows=(0, 24), out=out)
    _noalloc(gpu_lib, linker, torch, ts, tn, 5, 10, "MLE", "evd", rows=(24, 48), out=out)
    split = _host(out)
    assert (whole["tcorr"] > 0).sum() > 1000
    for k in whole:
        assert np.array_equal(whole[k].view(np.uint8), split[k].view(np.uint8)), k


def test_noalloc_limit_is_the_header_constant(gpu_lib):
    """A job of exactly FPL_NOALLOC_MAX_PIXELS pixels runs; one row more is
    rejected with FPL_ERR_NOALLOC_LIMIT before anything is launched."""
    torch = pytest.importorskip("torch")
    from fringe_gb300 import _lib, linker
    limit = _lib.FPL_NOALLOC_MAX_PIXELS
    cols = 1024
    assert limit % cols == 0
    rows = limit // cols + 1
    nb = 2
    # an empty SHP map: every pixel is skipped (centre bit clear), so the
    # accepted call is cheap and its outputs stay zero
    ts = torch.zeros((nb, rows, cols), dtype=torch.complex64, device="cuda")
    tn = torch.zeros((rows, cols, 8), dtype=torch.int32, device="cuda")
    out = _noalloc(gpu_lib, linker, torch, ts, tn, 5, 10, "MLE", "evd", rows=(0, rows - 1))
    assert int(torch.count_nonzero(out["tcorr"]).item()) == 0
    job = linker._make_job(nb, rows, cols, 5, 10, "MLE", "evd", 1, -1, 2, "fp32", (0, rows),
                           _lib.FPL_MEM_DEVICE, ts.data_ptr(), tn.data_ptr(), out["phase"].data_ptr(),
                           out["tcorr"].data_ptr(), out["comp"].data_ptr(), None)
    rc = gpu_lib.fpl_run_noalloc(ctypes.byref(job), None)
    assert rc == _lib.header_defines()["FPL_ERR_NOALLOC_LIMIT"]
    assert b"FPL_NOALLOC_MAX_PIXELS" in gpu_lib.fpl_error_string(rc)
