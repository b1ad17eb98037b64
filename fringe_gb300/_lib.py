"""ctypes binding of libfringe_gb300.so (the C ABI in include/fringe_gb300.h).

The library is built in-tree (``fringe_gb300/build.py``).  Loading fails
loudly when it is missing: there is no CPU fallback behind this module.
"""
import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libfringe_gb300.so")

FPL_METHOD = {"MLE": 0, "EVD": 1, "STBAS": 2}
FPL_SEMANTICS = {"evd": 0, "phase_link": 1}
FPL_PRECISION = {"fp32": 0, "mixed": 1}
FPL_MEM_HOST, FPL_MEM_DEVICE = 0, 1
FPL_BATCH_GRAPH, FPL_BATCH_AUTOTUNE = 1, 2
HEADER = os.path.join(os.path.dirname(HERE), "include", "fringe_gb300.h")


def header_defines(path=HEADER):
    """Integer #define constants of the C header, read from the header itself
    so that Python callers and tests cannot drift from it."""
    out = {}
    with open(path) as f:
        for line in f:
            parts = line.split()
            if len(parts) >= 3 and parts[0] == "#define":
                try:
                    out[parts[1]] = int(parts[2], 0)
                except ValueError:
                    pass
    return out


FPL_NOALLOC_MAX_PIXELS = header_defines()["FPL_NOALLOC_MAX_PIXELS"]


class FplJob(ctypes.Structure):
    _fields_ = [
        ("rows", ctypes.c_int), ("cols", ctypes.c_int), ("nbands", ctypes.c_int),
        ("half_window_y", ctypes.c_int), ("half_window_x", ctypes.c_int),
        ("method", ctypes.c_int), ("semantics", ctypes.c_int),
        ("mini_stack_count", ctypes.c_int), ("band_width", ctypes.c_int),
        ("min_neighbors", ctypes.c_int), ("precision", ctypes.c_int),
        ("memory", ctypes.c_int), ("row_begin", ctypes.c_int), ("row_end", ctypes.c_int),
        ("stack", ctypes.c_void_p), ("nmap", ctypes.c_void_p), ("phase", ctypes.c_void_p),
        ("tcorr", ctypes.c_void_p), ("comp", ctypes.c_void_p), ("status", ctypes.c_void_p),
    ]


class FplStats(ctypes.Structure):
    _fields_ = [("pixels", ctypes.c_longlong), ("fp64_pixels", ctypes.c_longlong),
                ("mixed_fp64_inverse", ctypes.c_longlong), ("slow_path_pixels", ctypes.c_longlong),
                ("kernel_ms", ctypes.c_float), ("total_ms", ctypes.c_float)]


class FplNmapJob(ctypes.Structure):
    _fields_ = [("rows", ctypes.c_int), ("cols", ctypes.c_int), ("nbands", ctypes.c_int),
                ("half_window_y", ctypes.c_int), ("half_window_x", ctypes.c_int),
                ("prob", ctypes.c_double), ("memory", ctypes.c_int),
                ("stack", ctypes.c_void_p), ("mask", ctypes.c_void_p), ("amp_const", ctypes.c_void_p),
                ("nmap", ctypes.c_void_p), ("count", ctypes.c_void_p), ("method", ctypes.c_int)]


FPL_NMAP_METHOD = {"KS2": 0, "AD2": 1}


class FplPsJob(ctypes.Structure):
    _fields_ = [("rows", ctypes.c_int), ("cols", ctypes.c_int), ("nbands", ctypes.c_int),
                ("master", ctypes.c_int), ("ds", ctypes.c_void_p), ("slc", ctypes.c_void_p),
                ("tcorr", ctypes.c_void_p), ("ps", ctypes.c_void_p), ("ifg", ctypes.c_void_p),
                ("tcorr_out", ctypes.c_void_p)]


class FplServerConfig(ctypes.Structure):
    _fields_ = [("memory_budget", ctypes.c_size_t), ("wave_pixels", ctypes.c_longlong),
                ("device", ctypes.c_int)]


class FplTicketInfo(ctypes.Structure):
    _fields_ = [("queue_ms", ctypes.c_double), ("run_ms", ctypes.c_double),
                ("total_ms", ctypes.c_double), ("rc", ctypes.c_int)]


class FplOptions(ctypes.Structure):
    _fields_ = [
        ("inputDS", ctypes.c_char_p), ("wtsDS", ctypes.c_char_p),
        ("outputFolder", ctypes.c_char_p), ("outputCompressedSlcFolder", ctypes.c_char_p),
        ("compSlc", ctypes.c_char_p), ("blocksize", ctypes.c_int), ("memsize", ctypes.c_int),
        ("Nx", ctypes.c_int), ("Ny", ctypes.c_int), ("minNeighbors", ctypes.c_int),
        ("miniStackCount", ctypes.c_int), ("method", ctypes.c_char_p),
        ("bandWidth", ctypes.c_int), ("semantics", ctypes.c_int), ("precision", ctypes.c_int),
        ("device", ctypes.c_int), ("verbose", ctypes.c_int),
    ]


# every function declared in include/fringe_gb300.h, with its ctypes signature
_P = ctypes.c_void_p
_SIGS = {
    "fpl_ctx_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]),
    "fpl_ctx_destroy": (ctypes.c_int, [_P]),
    "fpl_run": (ctypes.c_int, [_P, ctypes.POINTER(FplJob)]),
    "fpl_run_async": (ctypes.c_int, [_P, ctypes.POINTER(FplJob), _P]),
    "fpl_last_stats": (ctypes.c_int, [_P, ctypes.POINTER(FplStats)]),
    "fpl_options_default": (None, [ctypes.POINTER(FplOptions)]),
    "fpl_process": (ctypes.c_int, [ctypes.POINTER(FplOptions)]),
    "fpl_error_string": (ctypes.c_char_p, [ctypes.c_int]),
    "fpl_version": (ctypes.c_char_p, []),
    "fpl_run_noalloc": (ctypes.c_int, [ctypes.POINTER(FplJob), _P]),
    "fpl_batch_create": (ctypes.c_int, [_P, ctypes.POINTER(FplJob), ctypes.c_int, ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_void_p)]),
    "fpl_batch_run": (ctypes.c_int, [_P, _P]),
    "fpl_batch_stats": (ctypes.c_int, [_P, ctypes.POINTER(FplStats)]),
    "fpl_batch_destroy": (ctypes.c_int, [_P]),
    "fpl_server_config_default": (None, [ctypes.POINTER(FplServerConfig)]),
    "fpl_server_create": (ctypes.c_int, [ctypes.POINTER(FplServerConfig), ctypes.POINTER(ctypes.c_void_p)]),
    "fpl_server_submit": (ctypes.c_int, [_P, ctypes.POINTER(FplJob), ctypes.POINTER(ctypes.c_ulonglong)]),
    "fpl_server_wait": (ctypes.c_int, [_P, ctypes.c_ulonglong, ctypes.c_double,
                                       ctypes.POINTER(FplTicketInfo)]),
    "fpl_server_destroy": (ctypes.c_int, [_P]),
    "fpl_ctx_set_tuning": (ctypes.c_int, [_P, ctypes.c_float, ctypes.c_int]),
    "fpl_ctx_set_shift": (ctypes.c_int, [_P, ctypes.c_float, ctypes.c_float]),
    "fpl_adjust_wrapped": (ctypes.c_int, [_P, _P, _P, _P, ctypes.c_int, ctypes.c_longlong, _P]),
    "fpl_ctx_last_error": (ctypes.c_char_p, [_P]),
    "fpl_ctx_set_profiling": (ctypes.c_int, [_P, ctypes.c_int]),
    "fpl_ctx_profile": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double),
                                       ctypes.POINTER(ctypes.c_double),
                                       ctypes.POINTER(ctypes.c_int)]),
    "fpl_ctx_profile_kernels": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_double), ctypes.c_int]),
    "fpl_nmap": (ctypes.c_int, [_P, ctypes.POINTER(FplNmapJob)]),
    "fpl_integrate_ps": (ctypes.c_int, [_P, ctypes.POINTER(FplPsJob), _P]),
}
_EXTRA = {}

_lib = None
_lock = threading.Lock()


class FplError(RuntimeError):
    def __init__(self, code, where=""):
        self.code = code
        msg = "fringe_gb300 error %d (%s)" % (code, error_string(code))
        if where:
            msg += ": " + where
        super().__init__(msg)


def load():
    """Load libfringe_gb300.so; raises if it has not been built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                "libfringe_gb300.so is not built (run fringe_gb300/build.py or "
                "__graft_entry__.build()); there is no CPU fallback")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in list(_SIGS.items()) + list(_EXTRA.items()):
            f = getattr(lib, name)
            f.restype = res
            f.argtypes = args
        _lib = lib
        return lib


def error_string(code):
    try:
        return load().fpl_error_string(code).decode()
    except Exception:  # pragma: no cover - only when the library is missing
        return "?"


def check(code, ctx=None):
    if code != 0:
        where = ""
        if ctx:
            where = load().fpl_ctx_last_error(ctx).decode()
        raise FplError(code, where)


class Context:
    """Owns one fpl_ctx (a CUDA stream and scratch buffers on one device)."""

    def __init__(self, device=0):
        lib = load()
        h = ctypes.c_void_p()
        check(lib.fpl_ctx_create(device, ctypes.byref(h)))
        self.handle = h
        self.device = device

    def close(self):
        if self.handle:
            load().fpl_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def stats(self):
        s = FplStats()
        check(load().fpl_last_stats(self.handle, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in FplStats._fields_}

    def set_profiling(self, on=True):
        check(load().fpl_ctx_set_profiling(self.handle, int(on)), self.handle)

    def profile(self):
        """(fp32_ms, fp64_ms, runs) summed over runs since the last call."""
        a, b, n = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
        check(load().fpl_ctx_profile(self.handle, ctypes.byref(a), ctypes.byref(b),
                                     ctypes.byref(n)), self.handle)
        return a.value, b.value, n.value

    def profile_kernels(self):
        """Per-kernel milliseconds of the runs read by the last profile():
        {"fp32": plain pixel kernel, "gram": tensor-core Gamma, "solve":
        eigen-solves of the mixed form, "fp64": FP64 settle pass}."""
        ms = (ctypes.c_double * 4)()
        check(load().fpl_ctx_profile_kernels(self.handle, ms, 4), self.handle)
        return dict(zip(("fp32", "gram", "solve", "fp64"), list(ms)))

    def set_tuning(self, amb_scale=-1.0, force_fp64=False):
        check(load().fpl_ctx_set_tuning(self.handle, float(amb_scale), int(force_fp64)), self.handle)

    def set_shift(self, shift=0.999, backoff=0.97):
        """Shifts of the FP32 MLE inverse iteration (fpl_ctx_set_shift)."""
        check(load().fpl_ctx_set_shift(self.handle, float(shift), float(backoff)), self.handle)


_contexts = {}


def context(device=0):
    with _lock:
        c = _contexts.get(device)
    if c is None:
        c = Context(device)
        with _lock:
            _contexts[device] = c
    return c
