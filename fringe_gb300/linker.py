"""In-memory phase linking through the C ABI (fpl_run).

``phase_link`` is the array-level entry point: one call runs the reference's
per-pixel evd / phase_link loop (src/evd/evd.cpp:512-788,
src/phase_link/phase_link.cpp:479-666) over a whole scene on the GPU.

Inputs may be NumPy arrays (host memory: the call copies them to the device
and the results back) or CUDA torch tensors (device memory: no copies).
"""
import ctypes

import numpy as np

from . import _lib


def _is_torch(x):
    return type(x).__module__.startswith("torch")


def phase_link(stack, nmap, half_window, method="MLE", semantics="evd",
               mini_stack_count=1, band_width=-1, min_neighbors=2,
               precision="fp32", rows=None, want_status=False, device=0,
               out=None, ctx=None):
    """Phase-link a scene.

    stack : complex64 [nbands, rows, cols] (band-planar, as the reference's
            ``cpxdata``), NumPy or CUDA torch tensor.
    nmap  : uint32 [rows, cols, nulong] SHP bitmask (Ulongmask layout), or
            int32 of the same shape for torch.
    half_window : (Ny, Nx).
    Returns dict(phase [nbands,rows,cols] complex64, tcorr [rows,cols] float32,
    comp [rows,cols] complex64, status [rows,cols] int32 when want_status).
    """
    ny, nx = half_window
    ctx = ctx or _lib.context(device)
    lib = _lib.load()
    if _is_torch(stack):
        return _run_torch(lib, ctx, stack, nmap, ny, nx, method, semantics,
                          mini_stack_count, band_width, min_neighbors, precision,
                          rows, want_status, out)
    stack = np.ascontiguousarray(stack, dtype=np.complex64)
    nmap = np.ascontiguousarray(nmap).view(np.uint32)
    nb, R, C = stack.shape
    if out is None:
        out = {"phase": np.zeros((nb, R, C), np.complex64),
               "tcorr": np.zeros((R, C), np.float32),
               "comp": np.zeros((R, C), np.complex64)}
        if want_status:
            out["status"] = np.zeros((R, C), np.int32)
    job = _make_job(nb, R, C, ny, nx, method, semantics, mini_stack_count, band_width,
                    min_neighbors, precision, rows, _lib.FPL_MEM_HOST,
                    stack.ctypes.data, nmap.ctypes.data, out["phase"].ctypes.data,
                    out["tcorr"].ctypes.data, out["comp"].ctypes.data,
                    out["status"].ctypes.data if "status" in out else None)
    _lib.check(lib.fpl_run(ctx.handle, ctypes.byref(job)), ctx.handle)
    return out


def _make_job(nb, R, C, ny, nx, method, semantics, mini, bw, minn, precision, rows,
              memory, p_stack, p_nmap, p_phase, p_tcorr, p_comp, p_status):
    r0, r1 = (0, R) if rows is None else rows
    return _lib.FplJob(R, C, nb, ny, nx, _lib.FPL_METHOD[method],
                       _lib.FPL_SEMANTICS[semantics], mini, bw, minn,
                       _lib.FPL_PRECISION[precision], memory, r0, r1,
                       p_stack, p_nmap, p_phase, p_tcorr, p_comp, p_status)


def _run_torch(lib, ctx, stack, nmap, ny, nx, method, semantics, mini, bw, minn,
               precision, rows, want_status, out):
    import torch
    if not stack.is_cuda:
        raise ValueError("torch inputs must be CUDA tensors (use NumPy for host memory)")
    stack = stack.contiguous()
    nmap = nmap.contiguous()
    nb, R, C = stack.shape
    dev = stack.device
    if out is None:
        out = {"phase": torch.zeros((nb, R, C), dtype=torch.complex64, device=dev),
               "tcorr": torch.zeros((R, C), dtype=torch.float32, device=dev),
               "comp": torch.zeros((R, C), dtype=torch.complex64, device=dev)}
        if want_status:
            out["status"] = torch.zeros((R, C), dtype=torch.int32, device=dev)
    job = _make_job(nb, R, C, ny, nx, method, semantics, mini, bw, minn, precision, rows,
                    _lib.FPL_MEM_DEVICE, stack.data_ptr(), nmap.data_ptr(),
                    out["phase"].data_ptr(), out["tcorr"].data_ptr(), out["comp"].data_ptr(),
                    out["status"].data_ptr() if "status" in out else None)
    stream = torch.cuda.current_stream(dev).cuda_stream
    _lib.check(lib.fpl_run_async(ctx.handle, ctypes.byref(job), ctypes.c_void_p(stream)),
               ctx.handle)
    return out
