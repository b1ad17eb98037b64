"""Drop-in for the reference's ``evdlib`` extension module.

The reference's evd scripts do ``import evdlib`` and drive ``evdlib.Evd``
(pybind11, src/evd/evdlib.cpp:14-40; callers src/evd/evd.py:45,
src/sequential/sequential.py:73).  With this repository's root on
``PYTHONPATH`` the same scripts get this module instead: ``Evd`` has the same
properties and defaults (evdOptions, src/evd/evd.hpp:58-68), ``print()`` and
``run()``, and ``run()`` phase-links on the GPU through ``fpl_process`` in
libfringe_gb300.so.  The computation form is the plain FP32 drop-in unless
the environment variable FRINGE_GB300_PRECISION is "mixed".
"""
from fringe_gb300.evdlib import Evd  # noqa: F401

__all__ = ["Evd"]
