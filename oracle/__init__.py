"""CPU oracle for the phase-linking hot path -- TEST INFRASTRUCTURE ONLY.

Python access to the oracle libraries built from ``fpl_oracle.c``:

* ``port``      -- ``oracle/libfpl_oracle.so``: this project's FP64 restatement
  of FRInGE's per-pixel loop (src/evd/evd.cpp:512-788,
  src/phase_link/phase_link.cpp:479-666) with its own restatement of the LAPACK
  algorithms the reference calls;
* ``reference`` -- ``oracle/_ref/libfpl_ref.so``: the same loop calling the
  reference's own EVWorker (include/fringe/EigenLapack.hpp) and a real LAPACK.
  Only buildable where the reference tree is present.

Only the test-suite, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU
baseline may import this package.  The product library never does.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "libfpl_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libfpl_ref.so")

METHODS = {"MLE": 0, "EVD": 1, "STBAS": 2}
SEMANTICS = {"evd": 0, "phase_link": 1}


class _Params(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in (
        "rows", "cols", "nbands", "ny", "nx", "method", "semantics",
        "mini_stack_count", "band_width", "min_neighbors", "row_begin",
        "row_end", "nthreads")]


class _NmapParams(ctypes.Structure):
    _fields_ = [("rows", ctypes.c_int), ("cols", ctypes.c_int), ("nbands", ctypes.c_int),
                ("ny", ctypes.c_int), ("nx", ctypes.c_int), ("prob", ctypes.c_double),
                ("nthreads", ctypes.c_int), ("method", ctypes.c_int)]


NMAP_METHODS = {"KS2": 0, "AD2": 1}


def build_port(force=False):
    """Compile the port library with the committed Makefile."""
    if force or not os.path.exists(PORT_SO):
        subprocess.check_call(["make", "-s", "-C", HERE, "libfpl_oracle.so"])
    return PORT_SO


def build_reference(reference_root=None):
    """Compile oracle/_ref/libfpl_ref.so; returns its path or None.

    reference_root: the reference source tree; default the environment
    variable FRINGE_REFERENCE_ROOT, else build_ref.sh's own default.  Where
    the tree is absent the recipe exits without building (None here)."""
    root = reference_root or os.environ.get("FRINGE_REFERENCE_ROOT")
    cmd = [os.path.join(HERE, "build_ref.sh")] + ([root] if root else [])
    r = subprocess.run(cmd, capture_output=True, text=True)
    return REF_SO if r.returncode == 0 and os.path.exists(REF_SO) else None


def reference_root():
    """The reference source tree the recipes use (FRINGE_REFERENCE_ROOT, else
    build_ref.sh's default), or None where it is absent (a GPU host)."""
    r = subprocess.run([os.path.join(HERE, "build_ref.sh"), "--root"], capture_output=True, text=True)
    root = r.stdout.strip()
    return root if root and os.path.isfile(os.path.join(root, "include", "fringe", "EigenLapack.hpp")) else None


_LIBS = {}


def load(kind="port"):
    """Load the ``port`` or ``reference`` oracle library (ctypes CDLL)."""
    if kind in _LIBS:
        return _LIBS[kind]
    if kind == "port":
        path = build_port()
    elif kind == "reference":
        path = REF_SO
        if not os.path.exists(path):
            raise FileNotFoundError("oracle/_ref/libfpl_ref.so not built")
    else:
        raise ValueError(kind)
    lib = ctypes.CDLL(path)
    P = ctypes.c_void_p
    lib.fpl_oracle_run.argtypes = [ctypes.POINTER(_Params), P, P, P, P, P, P]
    lib.fpl_oracle_run.restype = ctypes.c_int
    lib.fpl_oracle_eig_index.argtypes = [ctypes.c_int, P, ctypes.c_int, ctypes.c_int, P, P]
    lib.fpl_oracle_eig_index.restype = ctypes.c_int
    lib.fpl_oracle_pd_inverse.argtypes = [ctypes.c_int, P]
    lib.fpl_oracle_pd_inverse.restype = ctypes.c_int
    lib.fpl_oracle_kind.restype = ctypes.c_char_p
    lib.fpl_oracle_nmap.argtypes = [ctypes.POINTER(_NmapParams), P, P, P, P, P]
    lib.fpl_oracle_nmap.restype = ctypes.c_int
    lib.fpl_oracle_ks2.argtypes = [ctypes.c_int, P, P]
    lib.fpl_oracle_ks2.restype = ctypes.c_double
    lib.fpl_oracle_ad2.argtypes = [ctypes.c_int, P, P]
    lib.fpl_oracle_ad2.restype = ctypes.c_double
    _LIBS[kind] = lib
    return lib


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def run(stack, nmap, ny, nx, method="MLE", semantics="evd", mini_stack_count=1,
        band_width=-1, min_neighbors=2, rows=None, nthreads=0, kind="port"):
    """Run the oracle over a whole scene (or the row range ``rows``).

    stack: complex64 [nbands, rows, cols]; nmap: uint32 [rows, cols, nulong].
    Returns dict(phase complex64 [nbands,rows,cols], tcorr float32 [rows,cols],
    comp complex64 [rows,cols], npix int32 [rows,cols]).
    """
    lib = load(kind)
    stack = np.ascontiguousarray(stack, dtype=np.complex64)
    nmap = np.ascontiguousarray(nmap, dtype=np.uint32)
    nb, R, C = stack.shape
    r0, r1 = (0, R) if rows is None else rows
    phase = np.zeros((nb, R, C), np.complex64)
    tcorr = np.zeros((R, C), np.float32)
    comp = np.zeros((R, C), np.complex64)
    npix = np.zeros((R, C), np.int32)
    p = _Params(R, C, nb, ny, nx, METHODS[method], SEMANTICS[semantics],
                mini_stack_count, band_width, min_neighbors, r0, r1, nthreads)
    rc = lib.fpl_oracle_run(ctypes.byref(p), _ptr(stack), _ptr(nmap), _ptr(phase),
                            _ptr(tcorr), _ptr(comp), _ptr(npix))
    if rc != 0:
        raise ValueError("oracle rejected the parameters (%d)" % rc)
    return {"phase": phase, "tcorr": tcorr, "comp": comp, "npix": npix}


def eig_index(A, index, want_vec=True, kind="port"):
    """One eigenpair by 1-based ascending index (zheevr RANGE='I' semantics).

    A: complex128 [n,n] Hermitian (upper triangle used).  Returns (info, w, z).
    """
    lib = load(kind)
    n = A.shape[0]
    a = np.asfortranarray(A, dtype=np.complex128).copy(order="F")
    w = np.zeros(1, np.float64)
    z = np.zeros(n, np.complex128)
    info = lib.fpl_oracle_eig_index(n, _ptr(a), index, int(want_vec), _ptr(w), _ptr(z))
    return info, float(w[0]), z


def pd_inverse(A, kind="port"):
    """Hermitian PD inverse (zpotrf+zpotri+fill).  Returns (info, Ainv)."""
    lib = load(kind)
    n = A.shape[0]
    a = np.asfortranarray(A, dtype=np.complex128).copy(order="F")
    info = lib.fpl_oracle_pd_inverse(n, _ptr(a))
    return info, a


def nmap(stack, ny, nx, prob=0.05, mask=None, amp_const=None, nthreads=0, kind="port", method="KS2"):
    """SHP map of the nmap module (method "KS2" or "AD2") over a whole scene.

    stack: complex64 [nbands, rows, cols]; mask: optional uint8 [rows, cols];
    amp_const: optional per-band calibration constants.  Returns
    (nmap uint32 [rows, cols, nulong], count int32 [rows, cols]).
    """
    lib = load(kind)
    stack = np.ascontiguousarray(stack, dtype=np.complex64)
    nb, R, C = stack.shape
    nul = ((2 * ny + 1) * (2 * nx + 1) + 31) // 32
    out = np.zeros((R, C, nul), np.uint32)
    count = np.zeros((R, C), np.int32)
    m = None if mask is None else np.ascontiguousarray(mask, dtype=np.uint8)
    a = None if amp_const is None else np.ascontiguousarray(amp_const, dtype=np.float64)
    p = _NmapParams(R, C, nb, ny, nx, float(prob), nthreads, NMAP_METHODS[method])
    rc = lib.fpl_oracle_nmap(ctypes.byref(p), _ptr(stack), _ptr(m), _ptr(a), _ptr(out), _ptr(count))
    if rc != 0:
        raise ValueError("oracle rejected the parameters (%d)" % rc)
    return out, count


def ad2(a, b, kind="port"):
    """p-value of the two-sample Anderson-Darling test of two equal-length
    samples (sorted ascending here, as the nmap module sorts them); a is the
    reference's first argument."""
    lib = load(kind)
    a = np.ascontiguousarray(np.sort(np.asarray(a, np.float32)))
    b = np.ascontiguousarray(np.sort(np.asarray(b, np.float32)))
    assert a.shape == b.shape
    return lib.fpl_oracle_ad2(len(a), _ptr(a), _ptr(b))


def ks2(a, b, kind="port"):
    """Probability of the two-sample KS test of two equal-length samples
    (sorted ascending here, as the nmap module sorts them)."""
    lib = load(kind)
    a = np.ascontiguousarray(np.sort(np.asarray(a, np.float32)))
    b = np.ascontiguousarray(np.sort(np.asarray(b, np.float32)))
    assert a.shape == b.shape
    pad_a = np.concatenate([a, a[-1:]])     # the reference may read one past the end
    pad_b = np.concatenate([b, b[-1:]])
    return lib.fpl_oracle_ks2(len(a), _ptr(pad_a), _ptr(pad_b))
