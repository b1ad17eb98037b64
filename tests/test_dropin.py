"""The reference's module scripts run unchanged against the top-level drop-in
modules ``evdlib`` and ``phase_linklib``.

src/evd/evd.py:37-66 and src/phase_link/phase_link.py:37-66 import
``evdlib`` / ``phase_linklib``, set the module properties one by one and call
``run()``.  These tests load those scripts from the reference tree where it
is present (skipped elsewhere), call their ``runEvd`` with the command line
parsed by their own ``cmdLineParser``, and check that every property reaches
``fpl_process`` as the matching ``fpl_options`` field.  ``fpl_process`` is
replaced by a recorder, so no GPU is needed; the file-level run itself is
checked against the oracle on the GPU by tests/test_files.py.
"""
import ctypes
import os
import runpy
import sys

import pytest

import oracle
from fringe_gb300 import _lib


def test_top_level_modules_have_the_reference_classes_and_defaults():
    import evdlib
    import phase_linklib
    for cls in (evdlib.Evd, phase_linklib.Phaselink):
        m = cls()
        # evdOptions::evdOptions, src/evd/evd.hpp:58-68
        assert (m.blocksize, m.memsize, m.halfWindowX, m.halfWindowY) == (64, 2048, 5, 5)
        assert (m.minimumNeighbors, m.miniStackCount, m.method, m.bandWidth) == (2, 1, "MLE", -1)
        assert m.precision == "fp32"
        with pytest.raises(AttributeError):
            m.noSuchProperty  # noqa: B018
    assert evdlib.Evd._semantics == _lib.FPL_SEMANTICS["evd"]
    assert phase_linklib.Phaselink._semantics == _lib.FPL_SEMANTICS["phase_link"]


class _Recorder:
    """Stands in for libfringe_gb300.so: the options of every fpl_process call."""

    def __init__(self, lib):
        self.lib = lib
        self.calls = []

    def __getattr__(self, name):
        return getattr(self.lib, name)

    def fpl_process(self, p_opts):
        o = ctypes.cast(p_opts, ctypes.POINTER(_lib.FplOptions)).contents
        rec = {}
        for field, _ in _lib.FplOptions._fields_:
            v = getattr(o, field)
            rec[field] = v.decode() if isinstance(v, bytes) else v
        self.calls.append(rec)
        return 0


ARGV = ["-i", "stack/slcs.vrt", "-w", "nmap/nmap", "-o", "out", "-l", "32", "-r", "1024",
        "-x", "10", "-y", "5", "-n", "7", "-m", "STBAS", "-b", "4"]


@pytest.mark.parametrize("script,semantics", [("src/evd/evd.py", "evd"),
                                              ("src/phase_link/phase_link.py", "phase_link")])
def test_reference_script_drives_the_drop_in(monkeypatch, script, semantics):
    root = oracle.reference_root()
    if root is None:
        pytest.skip("reference tree absent")
    path = os.path.join(root, script)
    rec = _Recorder(_lib.load())
    monkeypatch.setattr(_lib, "load", lambda: rec)
    monkeypatch.setattr(sys, "argv", [path] + ARGV)
    # load the script's functions without running its __main__ block (evd.py's
    # also writes output VRTs with GDAL, which is not part of this path)
    mod = runpy.run_path(path, run_name="reference_script")
    mod["runEvd"](mod["cmdLineParser"]())
    assert len(rec.calls) == 1
    o = rec.calls[0]
    assert (o["inputDS"], o["wtsDS"], o["outputFolder"]) == ("stack/slcs.vrt", "nmap/nmap", "out")
    assert (o["outputCompressedSlcFolder"], o["compSlc"]) == ("out", "compslc.bin")
    assert (o["blocksize"], o["memsize"], o["Nx"], o["Ny"]) == (32, 1024, 10, 5)
    assert (o["minNeighbors"], o["method"], o["bandWidth"], o["miniStackCount"]) == (7, "STBAS", 4, 1)
    assert o["semantics"] == _lib.FPL_SEMANTICS[semantics]
    assert o["precision"] == _lib.FPL_PRECISION["fp32"]
    assert os.environ.get("OPENBLAS_NUM_THREADS") == "1"     # set by the script itself


def test_precision_from_the_environment(monkeypatch):
    import evdlib
    monkeypatch.setenv("FRINGE_GB300_PRECISION", "mixed")
    assert evdlib.Evd().precision == "mixed"
    monkeypatch.setenv("FRINGE_GB300_PRECISION", "fp16")
    with pytest.raises(ValueError):
        evdlib.Evd()
