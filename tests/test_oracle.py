"""CPU tests of the oracle (no GPU): the port against the reference's own
known answers and against golden vectors produced by the reference's EVWorker
and LAPACK, plus the SHP bitmask layout fixtures of the reference's tests."""
import re

import numpy as np
import pytest

import oracle
from fringe_gb300 import synth
from tests.parity import assert_parity, codes, compare, load_golden

# the known 3x3 matrix of tests/eigen/test_eig.cpp:55-64
A3 = np.array([[3, -2, 4], [-2, 8, 2], [4, 2, 3]], dtype=np.complex128)


def test_known_3x3_eigenpairs():
    w_ref, v_ref = np.linalg.eigh(A3)
    for index, k in ((3, -1), (1, 0)):            # largestEigen / smallestEigen
        info, w, z = oracle.eig_index(A3, index)
        assert info == 0
        assert abs(w - w_ref[k]) < 1e-12
        # eigenvector up to a unit phase
        ph = np.vdot(v_ref[:, k], z)
        assert abs(abs(ph) - 1) < 1e-12
        assert np.allclose(z, v_ref[:, k] * ph, atol=1e-12)
    assert abs(oracle.eig_index(A3, 3)[1] - 8.81507) < 1e-5   # value printed by the reference's test


def test_known_3x3_positive_definite_inverse():
    # tests/eigen/test_eig.cpp:92-117: (A + 2I) inverted through zpotrf/zpotri
    Apos = A3 + 2 * np.eye(3)
    info, inv = oracle.pd_inverse(Apos)
    assert info == 0
    assert np.allclose(Apos @ inv, np.eye(3), atol=1e-12)
    assert np.allclose(inv, inv.conj().T)
    # A itself is indefinite: zpotrf reports the first non-positive pivot
    info, _ = oracle.pd_inverse(A3)
    assert info > 0


def _reference_bitmask_bytes(wy, wx):
    """tests/evd/test_evd.py:114-148, restated: all window bits set except the
    first (top-left), LSB first within each byte, padded to 32-bit words."""
    nwords = int(np.ceil(wy * wx / 32))
    bits = ("0" + "1" * (wx * wy - 1)).ljust(nwords * 32, "0")
    return bytes(int(octet[::-1], 2) for octet in re.findall(r"\d{8}", bits))


def test_bitmask_layout_matches_reference_fixture():
    ny, nx = 5, 5
    words = synth.nmap_all_ones(1, 1, ny, nx)[0, 0].copy()
    words[0] &= ~np.uint32(1)                     # clear (ii,jj) = (-ny,-nx)
    assert words.astype("<u4").tobytes() == _reference_bitmask_bytes(2 * ny + 1, 2 * nx + 1)
    # 120 neighbours, and the unpacked little-endian bits give the window
    nb = np.unpackbits(words.view(np.uint8), bitorder="little")
    assert nb.sum() == 120
    win = nb[:121].reshape(11, 11)
    expected = np.ones((11, 11), np.uint8)
    expected[0, 0] = 0
    assert np.array_equal(win, expected)


@pytest.mark.parametrize("ny,nx,nwords", [(2, 2, 1), (7, 7, 8)])
def test_bitmask_single_bits(ny, nx, nwords):
    """tests/bitmask/test_bits.cpp:6-57: bit (ii,jj) is bit flat%32 of word
    flat/32 with flat = (ii+Ny)(2Nx+1) + jj+Nx."""
    assert synth.nulong_for(ny, nx) == nwords
    for ii in range(-ny, ny + 1):
        for jj in range(-nx, nx + 1):
            flat = (ii + ny) * (2 * nx + 1) + jj + nx
            # only the centre and (ii, jj) share the centre's class
            cls = np.ones((2 * ny + 1, 2 * nx + 1), np.int32)
            cls[ny, nx] = 7
            cls[ny + ii, nx + jj] = 7
            words = synth.nmap_from_classes(cls, ny, nx)[ny, nx]
            expect = np.zeros(nwords, np.uint32)
            expect[flat // 32] |= np.uint32(1 << (flat % 32))
            centre = ny * (2 * nx + 1) + nx
            expect[centre // 32] |= np.uint32(1 << (centre % 32))
            assert np.array_equal(words, expect), (ii, jj)


@pytest.fixture(scope="module")
def golden():
    return load_golden()


def test_port_matches_reference_golden_vectors(golden):
    for case, g in golden.items():
        for var, (method, sem, extra, ref) in g["variants"].items():
            got = oracle.run(g["stack"], g["nmap"], g["ny"], g["nx"], method=method,
                             semantics=sem, **extra)
            m = compare(got, ref)
            # a variant may code every pixel (-4 everywhere on the indefinite-|C| scenes)
            assert m["valid_both"] > 0 or np.all(codes(ref) < 0), (case, var, m)
            assert_parity(m, phase_tol=1e-6, tcorr_tol=1e-6)
            assert m["phase_max"] < 1e-5, (case, var, m)


def test_reference_build_matches_golden_when_available(golden):
    try:
        oracle.load("reference")
    except (FileNotFoundError, OSError):
        pytest.skip("oracle/_ref not built (needs the reference tree)")
    g = golden["voronoi30"]
    method, sem, extra, ref = g["variants"]["MLE_evd"]
    got = oracle.run(g["stack"], g["nmap"], g["ny"], g["nx"], method=method, semantics=sem,
                     kind="reference", **extra)
    m = compare(got, ref)
    assert m["code_mismatch"] == 0 and m["phase_max"] < 1e-6
    assert m["comp_max"] == 0.0 and m["comp_zero_mismatch"] == 0, m


def test_row_ranges_are_block_invariant():
    """The reference's block/halo logic (src/evd/evd.cpp:419-443) makes every
    line's result depend only on its full window: row ranges compose."""
    stack, nmap = synth.scene("voronoi", 30, 40, 12, 3, 5, seed=11)
    full = oracle.run(stack, nmap, 3, 5, method="MLE")
    top = oracle.run(stack, nmap, 3, 5, method="MLE", rows=(0, 13))
    bot = oracle.run(stack, nmap, 3, 5, method="MLE", rows=(13, 30))
    for k in ("phase", "tcorr", "comp"):
        joined = top[k].copy()
        joined[..., 13:, :] = bot[k][..., 13:, :]
        assert np.array_equal(joined, full[k]), k


@pytest.mark.parametrize("nb", [6, 24])
def test_indefinite_abs_scene_codes(nb):
    """The "indefabs" scene (every pixel drawn from a positive definite
    coherence whose magnitude matrix is indefinite) is what the GPU test of
    the FP32 not-positive-definite proof relies on: the evd module reports
    -4 for every pixel (the Cholesky of |C| fails, src/evd/evd.cpp:626-641),
    and phase_link falls back to the EVD estimator for every pixel
    (src/phase_link/phase_link.cpp:540-618), so its MLE output equals its
    EVD output."""
    stack, nmap = synth.scene("indefabs", 16, 24, nb, 5, 10, seed=50 + nb)
    evd = oracle.run(stack, nmap, 5, 10, method="MLE", semantics="evd")
    assert np.all(evd["tcorr"] == -4)
    mle = oracle.run(stack, nmap, 5, 10, method="MLE", semantics="phase_link")
    ref = oracle.run(stack, nmap, 5, 10, method="EVD", semantics="phase_link")
    assert np.all(mle["tcorr"] > 0)
    for k in ("phase", "tcorr", "comp"):
        assert np.array_equal(mle[k], ref[k]), k


def test_oracle_rejects_invalid_options():
    stack, nmap = synth.scene("uniform", 8, 8, 6, 1, 1, seed=1)
    with pytest.raises(ValueError):
        oracle.run(stack, nmap, 1, 1, method="STBAS", band_width=0)     # evd.cpp:78-84
    with pytest.raises(ValueError):
        oracle.run(stack, nmap, 1, 1, method="STBAS", band_width=5)     # >= nbands-1
    with pytest.raises(ValueError):
        oracle.run(stack, nmap, 1, 1, mini_stack_count=7)
