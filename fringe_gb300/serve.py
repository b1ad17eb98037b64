"""Continuous-batching phase-linking service (fpl_server_* in the C ABI).

    srv = Server(memory_budget=80 << 30)
    t = srv.submit(stack, nmap, (5, 10), method="MLE")   # host arrays
    info = srv.wait(t)              # outputs filled; info has queue/run/total ms
    out = srv.result(t)

Jobs are admitted by a device-memory budget and share the GPU in waves; a
job's result is the same alone and in any mix.
"""
import ctypes

import numpy as np

from . import _lib
from .linker import _make_job


class Server:
    def __init__(self, memory_budget=80 << 30, wave_pixels=1 << 20, device=0):
        self.lib = _lib.load()
        cfg = _lib.FplServerConfig()
        self.lib.fpl_server_config_default(ctypes.byref(cfg))
        cfg.memory_budget = int(memory_budget)
        cfg.wave_pixels = int(wave_pixels)
        cfg.device = int(device)
        h = ctypes.c_void_p()
        _lib.check(self.lib.fpl_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self.handle = h
        self._jobs = {}

    def submit(self, stack, nmap, half_window, method="MLE", semantics="evd", mini_stack_count=1,
               band_width=-1, min_neighbors=2, out=None, precision="fp32"):
        """Queue a job on host arrays; returns its ticket.  The arrays must stay
        alive until wait() returns (the server keeps references).  precision
        "mixed" runs the job in the mixed-precision form."""
        stack = np.ascontiguousarray(stack, dtype=np.complex64)
        nmap = np.ascontiguousarray(nmap).view(np.uint32)
        nb, R, C = stack.shape
        if out is None:
            out = {"phase": np.zeros((nb, R, C), np.complex64), "tcorr": np.zeros((R, C), np.float32),
                   "comp": np.zeros((R, C), np.complex64)}
        ny, nx = half_window
        job = _make_job(nb, R, C, ny, nx, method, semantics, mini_stack_count, band_width,
                        min_neighbors, precision, None, _lib.FPL_MEM_HOST, stack.ctypes.data,
                        nmap.ctypes.data, out["phase"].ctypes.data, out["tcorr"].ctypes.data,
                        out["comp"].ctypes.data, None)
        t = ctypes.c_ulonglong()
        _lib.check(self.lib.fpl_server_submit(self.handle, ctypes.byref(job), ctypes.byref(t)))
        self._jobs[t.value] = (stack, nmap, out)
        return t.value

    def wait(self, ticket, timeout=600.0):
        info = _lib.FplTicketInfo()
        rc = self.lib.fpl_server_wait(self.handle, ctypes.c_ulonglong(ticket), float(timeout),
                                      ctypes.byref(info))
        _lib.check(rc)
        return {"queue_ms": info.queue_ms, "run_ms": info.run_ms, "total_ms": info.total_ms}

    def result(self, ticket):
        return self._jobs.pop(ticket)[2]

    def close(self):
        if getattr(self, "handle", None):
            self.lib.fpl_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
