"""Synthetic inputs: the indefinite-|C| coherence used by the scenes that
exercise the reference's code -4 and phase_link's EVD fall-back."""
import numpy as np
import pytest

from fringe_gb300 import synth


@pytest.mark.parametrize("nb", [6, 24, 64])
def test_indefinite_abs_coherence(nb):
    rng = np.random.default_rng(nb)
    C0 = synth.indefinite_abs_coherence(nb, rng)
    assert C0.shape == (nb, nb)
    assert np.allclose(C0, C0.conj().T)
    assert np.allclose(np.diag(C0), 1.0)
    assert np.linalg.eigvalsh(C0)[0] > 0                  # positive definite
    assert np.linalg.eigvalsh(np.abs(C0))[0] < -0.3       # its magnitude is not


def test_indefinite_abs_coherence_is_bounded():
    # a 2 x 2 magnitude matrix [[1, a], [a, 1]], |a| <= 1, is never indefinite
    with pytest.raises(ValueError):
        synth.indefinite_abs_coherence(2, np.random.default_rng(0), tries=200)


def test_indefabs_scene_shapes():
    stack, nmap = synth.scene("indefabs", 5, 7, 6, 2, 3, seed=1)
    assert stack.shape == (6, 5, 7) and stack.dtype == np.complex64
    assert np.array_equal(nmap, synth.nmap_all_ones(5, 7, 2, 3))
