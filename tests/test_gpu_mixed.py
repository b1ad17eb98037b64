"""Mixed-precision form: coherence matrices on the tensor cores (bf16 hi/lo
split, FP32 accumulate) against the FP64 oracle.  Target: phase within
1e-3 rad RMS of the oracle, identical validity codes."""
import numpy as np
import pytest

import oracle
from fringe_gb300 import synth
from tests.parity import assert_parity, compare

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,R,C,N,ny,nx,seed", [
    ("voronoi", 8, 12, 30, 5, 10, 5),          # tiny first case
    ("voronoi", 40, 72, 30, 5, 10, 1002),
    ("uniform", 32, 32, 10, 5, 5, 1001),
    ("voronoi", 24, 40, 17, 3, 5, 17),
])
@pytest.mark.parametrize("method,semantics", [("MLE", "evd"), ("EVD", "evd"), ("MLE", "phase_link")])
def test_mixed_matches_oracle(gpu_lib, kind, R, C, N, ny, nx, seed, method, semantics):
    from fringe_gb300 import phase_link
    stack, nmap = synth.scene(kind, R, C, N, ny, nx, seed=seed)
    g = phase_link(stack, nmap, (ny, nx), method=method, semantics=semantics, precision="mixed")
    o = oracle.run(stack, nmap, ny, nx, method=method, semantics=semantics)
    m = compare(g, o)
    assert m["valid_both"] > 0, m
    assert_parity(m, phase_tol=1e-3, tcorr_tol=2e-4)


def test_mixed_large_window_chunks(gpu_lib):
    """More than 256 SHPs per pixel: the operand is staged in several chunks
    accumulated in tensor memory."""
    from fringe_gb300 import phase_link
    stack, nmap = synth.scene("uniform", 20, 40, 12, 8, 10, seed=3)     # 17 x 21 = 357 taps
    g = phase_link(stack, nmap, (8, 10), method="MLE", precision="mixed")
    o = oracle.run(stack, nmap, 8, 10, method="MLE")
    assert_parity(compare(g, o), phase_tol=1e-3, tcorr_tol=2e-4)
