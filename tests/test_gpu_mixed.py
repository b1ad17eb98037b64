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


@pytest.mark.parametrize("ny,nx", [(3, 0), (0, 3), (1, 1), (7, 0)])
def test_mixed_thin_windows(gpu_lib, ny, nx):
    """Windows one column or one row wide.  With Nx = 0 a union row of a
    tile holds 16 samples, so each 32-sample chunk of the Gamma kernel spans
    two whole union rows."""
    from fringe_gb300 import phase_link
    stack, nmap = synth.scene("voronoi", 24, 40, 6, ny, nx, seed=31 + ny + nx)
    for method in ("MLE", "EVD"):
        g = phase_link(stack, nmap, (ny, nx), method=method, precision="mixed")
        o = oracle.run(stack, nmap, ny, nx, method=method)
        m = compare(g, o)
        assert m["valid_both"] > 0, m
        assert_parity(m, phase_tol=1e-3, tcorr_tol=2e-4)


def _mixed_and_oracle(stack, nmap, ny, nx, **kw):
    from fringe_gb300 import phase_link
    g = phase_link(stack, nmap, (ny, nx), precision="mixed", want_status=True, **kw)
    okw = {k: v for k, v in kw.items() if k in ("method", "semantics", "min_neighbors", "rows")}
    o = oracle.run(stack, nmap, ny, nx, **okw)
    return g, o


@pytest.mark.parametrize("nb", [1, 2, 5, 16, 17, 33, 64])
def test_mixed_depths(gpu_lib, nb):
    """Every stack depth: odd counts pad the date pairs; from 21 dates on a
    tile's Gamma takes more than one pass (512 columns per pass) over its
    samples."""
    stack, nmap = synth.scene("voronoi", 20, 24, nb, 2, 3, seed=100 + nb)
    for method, sem in (("MLE", "evd"), ("EVD", "evd"), ("MLE", "phase_link")):
        g, o = _mixed_and_oracle(stack, nmap, 2, 3, method=method, semantics=sem)
        assert_parity(compare(g, o), phase_tol=1e-3, tcorr_tol=2e-4)
        if nb == 1:
            assert np.array_equal(np.isnan(g["tcorr"]), np.isnan(o["tcorr"]))


def test_mixed_illconditioned_n64(gpu_lib):
    stack, nmap = synth.scene("illcond", 24, 40, 64, 5, 10, seed=1003)
    for method, sem in (("MLE", "evd"), ("MLE", "phase_link"), ("EVD", "evd")):
        g, o = _mixed_and_oracle(stack, nmap, 5, 10, method=method, semantics=sem)
        assert_parity(compare(g, o), phase_tol=1e-3, tcorr_tol=2e-4)


def test_mixed_edge_masks_and_shapes(gpu_lib):
    stack, nmap = synth.scene("uniform", 12, 15, 8, 2, 2, seed=5)
    g, o = _mixed_and_oracle(stack, np.zeros_like(nmap), 2, 2, method="MLE")
    assert not np.any(g["phase"]) and not np.any(g["tcorr"]) and np.all(g["status"] == 1)
    c = np.zeros_like(nmap)
    flat = 2 * 5 + 2
    c[..., flat // 32] = np.uint32(1 << (flat % 32))
    g, o = _mixed_and_oracle(stack, c, 2, 2, method="EVD")
    assert not np.any(g["phase"]) and np.all(g["status"] == 2)
    # scenes smaller than one 8 x 16 tile, single rows / columns, partial tiles
    for shape in ((3, 4), (1, 17), (19, 1), (1, 1), (9, 17), (17, 33)):
        st, nm = synth.scene("uniform", shape[0], shape[1], 6, 5, 10, seed=9)
        for method in ("MLE", "EVD"):
            g, o = _mixed_and_oracle(st, nm, 5, 10, method=method)
            assert_parity(compare(g, o), phase_tol=1e-3, tcorr_tol=2e-4)
    g, o = _mixed_and_oracle(stack, nmap, 2, 2, method="MLE", semantics="phase_link", min_neighbors=26)
    assert not np.any(g["tcorr"]) and not np.any(o["tcorr"])


def test_mixed_row_range(gpu_lib):
    from fringe_gb300 import phase_link
    stack, nmap = synth.scene("voronoi", 40, 36, 12, 3, 5, seed=21)
    full = phase_link(stack, nmap, (3, 5), method="MLE", precision="mixed")
    part = phase_link(stack, nmap, (3, 5), method="MLE", precision="mixed", rows=(5, 30))
    # tiles start at the first row of the range: same sums, other grouping
    m = compare({k: v[..., 5:30, :] for k, v in part.items()},
                {k: v[..., 5:30, :] for k, v in full.items()})
    assert_parity(m, phase_tol=1e-4, tcorr_tol=1e-5)
    assert not np.any(part["tcorr"][:5]) and not np.any(part["tcorr"][30:])


@pytest.mark.parametrize("nb", [10, 40])
def test_mixed_out_of_range_samples(gpu_lib, nb):
    """NaN samples, and magnitudes outside the bf16 split's range, send the
    pixels whose SHPs include them to the FP64 path; other pixels of the same
    tile are unaffected.  At 40 dates a tile takes four passes over its
    samples, and the hand-off found in the first pass holds for all four."""
    stack, nmap = synth.scene("uniform", 24, 40, nb, 2, 3, seed=77)
    stack[2, 5, 7] = np.nan
    stack[:, 15, 30] = 3e17
    stack[4, 20, 3] = 1e-17 + 1e-17j
    for method, sem in (("MLE", "evd"), ("EVD", "evd"), ("MLE", "phase_link")):
        g, o = _mixed_and_oracle(stack, nmap, 2, 3, method=method, semantics=sem)
        m = compare(g, o)
        assert_parity(m, phase_tol=1e-3, tcorr_tol=2e-4)
        # the NaN neighbourhood reports the oracle's codes
        assert np.array_equal(g["tcorr"][3:8, 4:11] < 0, o["tcorr"][3:8, 4:11] < 0)


@pytest.mark.parametrize("precision", ["mixed", "fp32"])
@pytest.mark.parametrize("nb", [6, 24, 64])
def test_indefinite_abs_coherence_resolved_in_fp32(gpu_lib, precision, nb):
    """Every pixel of the scene has an indefinite |C| (its C drawn from a
    positive definite coherence whose magnitude matrix is indefinite).  A
    failed FP32 sweep of |C| whose failing row, after at most a few power
    steps, gives a quadratic form below minus the error bands proves |C| not
    positive definite, so these pixels get their code (or the EVD fall-back)
    without the FP64 path.  Six dates run the two-pixels-per-warp solve of
    the mixed form; at 64 dates about half the pixels need a power step."""
    from fringe_gb300 import _lib, phase_link
    from tests.parity import codes
    stack, nmap = synth.scene("indefabs", 24, 40, nb, 5, 10, seed=50 + nb)
    ctx = _lib.Context(0)
    for sem in ("evd", "phase_link"):
        g = phase_link(stack, nmap, (5, 10), method="MLE", semantics=sem, precision=precision, ctx=ctx)
        settled = ctx.stats()["fp64_pixels"]
        o = oracle.run(stack, nmap, 5, 10, method="MLE", semantics=sem)
        assert_parity(compare(g, o), phase_tol=1e-3, tcorr_tol=2e-4)
        if sem == "evd":
            n_indef = int(np.sum(codes(o) == -4))
            assert n_indef > 0.8 * stack.shape[1] * stack.shape[2], n_indef
        assert settled <= 0.05 * stack.shape[1] * stack.shape[2], settled


def test_mixed_results_do_not_depend_on_row_ranges(gpu_lib):
    """Tiles sit on the absolute 8-row grid, so a pixel's coherence matrix is
    accumulated in the same order whatever row range a run covers: the scene
    run in pieces that do not start on the grid equals the whole run."""
    from fringe_gb300 import phase_link
    stack, nmap = synth.scene("voronoi", 45, 52, 20, 5, 10, seed=44)
    whole = phase_link(stack, nmap, (5, 10), precision="mixed")
    parts = None
    for r0, r1 in ((0, 13), (13, 30), (30, 45)):
        parts = phase_link(stack, nmap, (5, 10), precision="mixed", rows=(r0, r1), out=parts)
    for key in ("phase", "tcorr", "comp"):
        assert np.array_equal(whole[key], parts[key], equal_nan=True), key
