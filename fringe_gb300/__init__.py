"""fringe_gb300 -- GB300-native (sm_103a) phase linking for FRInGE stacks.

The hot path of FRInGE's evd / phase_link modules (SHP gather, coherence
matrix, EVD / MLE / STBAS eigen-solve, phase referencing, compressed SLC and
temporal coherence) runs as CUDA kernels behind the C ABI declared in
``include/fringe_gb300.h``.  Python entry points:

* ``phase_link(stack, nmap, half_window, ...)`` -- in-memory run;
* ``nmap(stack, half_window, prob=0.05, ...)`` -- the SHP bitmask (nmap
  module, two-sample KS test) that phase linking consumes;
* ``integrate_ps(ds, slc, tcorr, ps)`` -- the PS/DS merge of the
  integratePS workflow step (single-master interferograms, PS coherence);
* ``fringe_gb300.evdlib.Evd`` / ``fringe_gb300.evdlib.Phaselink`` -- drop-in
  replacements of the reference's module wrappers (file level), re-exported
  under the reference's module names by the top-level modules ``evdlib`` and
  ``phase_linklib`` at the repository root;
* ``synth`` -- seeded synthetic stacks and SHP bitmasks.
"""
from .linker import integrate_ps, nmap, phase_link  # noqa: F401

__all__ = ["phase_link", "nmap", "integrate_ps"]
