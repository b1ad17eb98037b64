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


def _noalloc(lib, linker, torch, ts, tn, ny, nx, method, semantics):
    nb, R, C = ts.shape
    out = {"phase": torch.zeros((nb, R, C), dtype=torch.complex64, device="cuda"),
           "tcorr": torch.zeros((R, C), dtype=torch.float32, device="cuda"),
           "comp": torch.zeros((R, C), dtype=torch.complex64, device="cuda")}
    from fringe_gb300 import _lib
    job = linker._make_job(nb, R, C, ny, nx, method, semantics, 1, -1, 2, "fp32", None,
                           _lib.FPL_MEM_DEVICE, ts.data_ptr(), tn.data_ptr(),
                           out["phase"].data_ptr(), out["tcorr"].data_ptr(),
                           out["comp"].data_ptr(), None)
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.fpl_run_noalloc(ctypes.byref(job), ctypes.c_void_p(stream))
    assert rc == 0, lib.fpl_error_string(rc)
    torch.cuda.synchronize()
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
    ref = {k: v.cpu().numpy() for k, v in ref.items()}
    for _ in range(2):
        got = _noalloc(gpu_lib, linker, torch, ts, tn, 5, 10, method, semantics)
        m = compare(got, ref)
        assert m["valid_both"] > 1000, m
        assert_parity(m)


def test_noalloc_rejects_jobs_beyond_its_scratch(gpu_lib):
    torch = pytest.importorskip("torch")
    from fringe_gb300 import _lib, linker
    buf = torch.zeros(16, dtype=torch.complex64, device="cuda")
    limit = 524288
    rows, cols = 1024, limit // 1024 + 1          # one row of pixels too many
    p = buf.data_ptr()
    job = linker._make_job(30, rows, cols, 5, 10, "MLE", "evd", 1, -1, 2, "fp32", None,
                           _lib.FPL_MEM_DEVICE, p, p, p, p, p, None)
    rc = gpu_lib.fpl_run_noalloc(ctypes.byref(job), None)
    assert rc == 206
    assert b"FPL_NOALLOC_MAX_PIXELS" in gpu_lib.fpl_error_string(rc)
