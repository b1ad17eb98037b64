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


class PhaseLinkBatch:
    """Many CUDA-tensor jobs in one persistent launch (fpl_batch_*).

    ``jobs`` is a list of dicts with keys stack, nmap (CUDA tensors),
    half_window, and optionally method, semantics, mini_stack_count,
    band_width, min_neighbors, precision ("fp32" or "mixed"; default the
    batch's ``precision``).  Outputs are allocated once; ``run()`` fills
    them (replaying a captured CUDA graph when ``graph=True``).
    """

    def __init__(self, jobs, graph=True, autotune=False, device=0, ctx=None, precision="fp32"):
        import torch
        self.ctx = ctx or _lib.context(device)
        self.lib = _lib.load()
        self.outputs = []
        self._keep = []
        arr = (_lib.FplJob * len(jobs))()
        for k, j in enumerate(jobs):
            stack = j["stack"].contiguous()
            nmap = j["nmap"].contiguous()
            nb, R, C = stack.shape
            ny, nx = j["half_window"]
            out = {"phase": torch.zeros((nb, R, C), dtype=torch.complex64, device=stack.device),
                   "tcorr": torch.zeros((R, C), dtype=torch.float32, device=stack.device),
                   "comp": torch.zeros((R, C), dtype=torch.complex64, device=stack.device)}
            self.outputs.append(out)
            self._keep += [stack, nmap]
            arr[k] = _make_job(nb, R, C, ny, nx, j.get("method", "MLE"), j.get("semantics", "evd"),
                               j.get("mini_stack_count", 1), j.get("band_width", -1),
                               j.get("min_neighbors", 2), j.get("precision", precision), j.get("rows"),
                               _lib.FPL_MEM_DEVICE,
                               stack.data_ptr(), nmap.data_ptr(), out["phase"].data_ptr(),
                               out["tcorr"].data_ptr(), out["comp"].data_ptr(), None)
        flags = (_lib.FPL_BATCH_GRAPH if graph else 0) | (_lib.FPL_BATCH_AUTOTUNE if autotune else 0)
        h = ctypes.c_void_p()
        _lib.check(self.lib.fpl_batch_create(self.ctx.handle, arr, len(jobs), flags, ctypes.byref(h)),
                   self.ctx.handle)
        self.handle = h

    def run(self, stream=None):
        import torch
        s = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        _lib.check(self.lib.fpl_batch_run(self.handle, ctypes.c_void_p(s)), self.ctx.handle)
        return self.outputs

    def stats(self):
        st = _lib.FplStats()
        _lib.check(self.lib.fpl_batch_stats(self.handle, ctypes.byref(st)), self.ctx.handle)
        return {k: getattr(st, k) for k, _ in _lib.FplStats._fields_}

    def close(self):
        if getattr(self, "handle", None):
            self.lib.fpl_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def nmap(stack, half_window, prob=0.05, mask=None, amp_const=None, device=0, out=None, ctx=None,
         method="KS2"):
    """SHP neighbourhood map of a stack (the nmap module, KS2 or AD2 method).

    stack : complex64 [nbands, rows, cols], NumPy (host) or CUDA torch tensor.
    half_window : (Ny, Nx).  prob: similarity threshold (nmapOptions::prob).
    method : "KS2" (two-sample Kolmogorov-Smirnov) or "AD2" (two-sample
    Anderson-Darling), nmapOptions::method.
    mask : optional uint8 [rows, cols] (0 = excluded); amp_const: optional
    per-band amplitude calibration constants.  Returns dict(nmap uint32
    [rows, cols, nulong] (int32 for torch), count int32 [rows, cols]).
    """
    ny, nx = half_window
    ctx = ctx or _lib.context(device)
    lib = _lib.load()
    nul = ((2 * ny + 1) * (2 * nx + 1) + 31) // 32
    a = None if amp_const is None else np.ascontiguousarray(amp_const, dtype=np.float64)
    if _is_torch(stack):
        import torch
        if not stack.is_cuda:
            raise ValueError("torch inputs must be CUDA tensors (use NumPy for host memory)")
        stack = stack.contiguous()
        nb, R, C = stack.shape
        if out is None:
            out = {"nmap": torch.zeros((R, C, nul), dtype=torch.int32, device=stack.device),
                   "count": torch.zeros((R, C), dtype=torch.int32, device=stack.device)}
        m = None if mask is None else mask.contiguous()
        job = _lib.FplNmapJob(R, C, nb, ny, nx, float(prob), _lib.FPL_MEM_DEVICE, stack.data_ptr(),
                              m.data_ptr() if m is not None else None,
                              a.ctypes.data if a is not None else None,
                              out["nmap"].data_ptr(), out["count"].data_ptr(), _lib.FPL_NMAP_METHOD[method])
        _lib.check(lib.fpl_nmap(ctx.handle, ctypes.byref(job)), ctx.handle)
        return out
    stack = np.ascontiguousarray(stack, dtype=np.complex64)
    nb, R, C = stack.shape
    if out is None:
        out = {"nmap": np.zeros((R, C, nul), np.uint32), "count": np.zeros((R, C), np.int32)}
    m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
    job = _lib.FplNmapJob(R, C, nb, ny, nx, float(prob), _lib.FPL_MEM_HOST, stack.ctypes.data,
                          m.ctypes.data if m is not None else None,
                          a.ctypes.data if a is not None else None,
                          out["nmap"].ctypes.data, out["count"].ctypes.data, _lib.FPL_NMAP_METHOD[method])
    _lib.check(lib.fpl_nmap(ctx.handle, ctypes.byref(job)), ctx.handle)
    return out


def integrate_ps(ds, slc, tcorr, ps, master=0, device=0, ctx=None):
    """PS/DS merge of python/integratePS.py over the single-master network
    (python/Network.py:95-104): for every band j != master, in band order,
    ds_j * conj(ds_master), replaced at PS pixels (ps == 1) by
    exp(1j * angle(slc_j * conj(slc_master))); and tcorr with PS pixels set
    to 0.95.

    ds, slc : complex64 [nbands, rows, cols] (phase-linked and original
    stacks); tcorr : float32 [rows, cols]; ps : [rows, cols] PS map.  NumPy
    arrays (copied through the device) or CUDA torch tensors.  Returns
    dict(ifg complex64 [nbands-1, rows, cols], tcorr float32 [rows, cols]),
    of the inputs' kind.
    """
    import torch
    ctx = ctx or _lib.context(device)
    lib = _lib.load()
    host = not _is_torch(ds)
    dev = torch.device("cuda", ctx.device) if host else ds.device

    def on_dev(a, dt):
        if _is_torch(a):
            if not a.is_cuda:
                raise ValueError("torch inputs must be CUDA tensors (use NumPy for host memory)")
            return a.to(dt).contiguous()
        return torch.from_numpy(np.ascontiguousarray(a)).to(device=dev, dtype=dt)

    d_ds = on_dev(ds, torch.complex64)
    d_slc = on_dev(slc, torch.complex64)
    d_tc = on_dev(tcorr, torch.float32)
    # the reference tests psPixels == 1 in the map's own type
    if _is_torch(ps):
        d_ps = ps.contiguous() if ps.dtype == torch.uint8 else (ps == 1).to(torch.uint8)
        d_ps = on_dev(d_ps, torch.uint8)
    else:
        p_np = np.asarray(ps)
        d_ps = on_dev(p_np if p_np.dtype == np.uint8 else (p_np == 1).astype(np.uint8), torch.uint8)
    nb, R, C = d_ds.shape
    if tuple(d_slc.shape) != (nb, R, C) or tuple(d_tc.shape) != (R, C) or tuple(d_ps.shape) != (R, C):
        raise ValueError("ds, slc must be [nbands, rows, cols] and tcorr, ps [rows, cols]")
    ifg = torch.empty((max(nb - 1, 0), R, C), dtype=torch.complex64, device=dev)
    tc_out = torch.empty((R, C), dtype=torch.float32, device=dev)
    job = _lib.FplPsJob(R, C, nb, int(master), d_ds.data_ptr(), d_slc.data_ptr(), d_tc.data_ptr(),
                        d_ps.data_ptr(), ifg.data_ptr() if ifg.numel() else None, tc_out.data_ptr())
    stream = torch.cuda.current_stream(dev).cuda_stream
    _lib.check(lib.fpl_integrate_ps(ctx.handle, ctypes.byref(job), ctypes.c_void_p(stream)), ctx.handle)
    if host:
        torch.cuda.synchronize(dev)
        return {"ifg": ifg.cpu().numpy(), "tcorr": tc_out.cpu().numpy()}
    return {"ifg": ifg, "tcorr": tc_out}
