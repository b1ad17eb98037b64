"""Drop-in for the reference's ``phase_linklib`` extension module.

The reference's phase_link script does ``import phase_linklib`` and drives
``phase_linklib.Phaselink`` (Cython, src/phase_link/phase_linklib.pyx:33-157;
caller src/phase_link/phase_link.py:45).  With this repository's root on
``PYTHONPATH`` the same script gets this module instead: ``Phaselink`` has
the same properties and defaults, ``print()`` and ``run()``, and ``run()``
phase-links on the GPU through ``fpl_process`` with the phase_link module's
semantics (MLE with the EVD fallback).  The computation form is the plain
FP32 drop-in unless the environment variable FRINGE_GB300_PRECISION is
"mixed".
"""
from fringe_gb300.evdlib import Phaselink  # noqa: F401

__all__ = ["Phaselink"]
