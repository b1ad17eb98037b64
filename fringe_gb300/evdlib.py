"""Module wrappers with the reference's Python interface.

``Evd`` mirrors ``evdlib.Evd`` (pybind11, src/evd/evdlib.cpp:14-40) and
``Phaselink`` mirrors ``phase_linklib.Phaselink`` (Cython,
src/phase_link/phase_linklib.pyx:33-157): the same property names and
defaults (src/evd/evd.hpp:58-68), ``print()`` and ``run()``.  ``run()`` calls
``fpl_process`` in libfringe_gb300.so and returns its code (0, or the
reference's module codes 101-121; the reference's wrappers discard it).
The top-level modules ``evdlib`` and ``phase_linklib`` at the repository root
re-export these classes under the reference's module names.
"""
import ctypes
import os

from . import _lib

_PROPS = {
    # python name: (fpl_options field, kind)
    "inputDS": ("inputDS", "s"),
    "weightsDS": ("wtsDS", "s"),
    "outputFolder": ("outputFolder", "s"),
    "outputCompressedSlcFolder": ("outputCompressedSlcFolder", "s"),
    "compSlc": ("compSlc", "s"),
    "blocksize": ("blocksize", "i"),
    "memsize": ("memsize", "i"),
    "halfWindowX": ("Nx", "i"),
    "halfWindowY": ("Ny", "i"),
    "minimumNeighbors": ("minNeighbors", "i"),
    "miniStackCount": ("miniStackCount", "i"),
    "method": ("method", "s"),
    "bandWidth": ("bandWidth", "i"),
}


class _Module:
    _semantics = _lib.FPL_SEMANTICS["evd"]

    def __init__(self):
        o = _lib.FplOptions()
        _lib.load().fpl_options_default(ctypes.byref(o))
        self._v = {}
        for py, (field, kind) in _PROPS.items():
            val = getattr(o, field)
            self._v[py] = (val.decode() if isinstance(val, bytes) else (val or "")) if kind == "s" else val
        # evdOptions leaves the compressed-SLC names empty; the scripts set them
        self._v["outputCompressedSlcFolder"] = ""
        self._v["compSlc"] = ""
        self.precision = os.environ.get("FRINGE_GB300_PRECISION", "fp32")
        if self.precision not in _lib.FPL_PRECISION:
            raise ValueError("FRINGE_GB300_PRECISION must be one of %s" % sorted(_lib.FPL_PRECISION))
        self.device = 0
        self.verbose = 1

    def __getattr__(self, name):
        if name != "_v" and name in _PROPS:
            return self._v[name]
        raise AttributeError(name)

    def __setattr__(self, name, value):
        if name in _PROPS:
            kind = _PROPS[name][1]
            self._v[name] = str(value) if kind == "s" else int(value)
        else:
            object.__setattr__(self, name, value)

    def print(self):
        """evdOptions::print (src/evd/evd.hpp:165-185)."""
        v = self._v
        print("Input Dataset: %s" % v["inputDS"])
        print("Weights Dataset: %s" % v["weightsDS"])
        print("Output Folder %s" % v["outputFolder"])
        print("Output compressed SLC folder %s" % v["outputCompressedSlcFolder"])
        print("Output compressed SLC %s" % v["compSlc"])
        print("Window size: %d %d" % (v["halfWindowX"], v["halfWindowY"]))
        print("Memsize: %d Mb " % v["memsize"])
        print("Blocksize: %d lines " % v["blocksize"])
        print("Minimum neighbors: %d" % v["minimumNeighbors"])
        print("Mini-stack counter: %d" % v["miniStackCount"])
        print("Decomposition method: %s" % v["method"])
        if v["method"] == "STBAS":
            print("STBAS Bandwidth: %d" % v["bandWidth"])

    def run(self):
        o = _lib.FplOptions()
        lib = _lib.load()
        lib.fpl_options_default(ctypes.byref(o))
        keep = []
        for py, (field, kind) in _PROPS.items():
            val = self._v[py]
            if kind == "s":
                b = val.encode() if val else None
                keep.append(b)
                setattr(o, field, b)
            else:
                setattr(o, field, val)
        o.semantics = self._semantics
        o.precision = _lib.FPL_PRECISION[self.precision]
        o.device = int(self.device)
        o.verbose = int(self.verbose)
        return lib.fpl_process(ctypes.byref(o))


class Evd(_Module):
    """Drop-in for evdlib.Evd: the evd module (src/evd/evd.cpp)."""
    _semantics = _lib.FPL_SEMANTICS["evd"]


class Phaselink(_Module):
    """Drop-in for phase_linklib.Phaselink: the phase_link module
    (src/phase_link/phase_link.cpp): MLE with the EVD fallback."""
    _semantics = _lib.FPL_SEMANTICS["phase_link"]
