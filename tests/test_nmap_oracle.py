"""CPU checks of the nmap oracle (test infrastructure): the port's two-sample
KS and Anderson-Darling tests against the reference's own KS2sample and
AD2unique (the reference-linked oracle where it is built; everywhere, the
golden vectors it wrote, tests/golden/golden_nmap.npz), known answers, and
the structure of the map it builds."""
import os

import numpy as np
import pytest

import oracle
from fringe_gb300 import synth


def test_ks2_known_answers():
    a = np.arange(1, 31, dtype=np.float32)
    assert oracle.ks2(a, a) == 1.0                       # D = 0
    p = oracle.ks2(a, a + 100.0)                         # disjoint samples: D = 1
    z = np.sqrt(30 * 30 / 60.0)
    assert abs(p - 2 * (np.exp(-2 * z * z) - np.exp(-8 * z * z))) < 1e-15
    assert p < 0.05


@pytest.mark.skipif(not os.path.exists(oracle.REF_SO), reason="reference-linked oracle not built")
def test_ks2_port_matches_reference_header():
    """The port restates KS2sample::test (src/nmap/KS2sample.hpp:96-144); the
    reference build runs the header itself."""
    rng = np.random.default_rng(3)
    for n in (1, 2, 5, 10, 30, 45, 64):
        for _ in range(200):
            a = rng.rayleigh(1.0, n).astype(np.float32)
            b = (rng.rayleigh(1.0, n) * rng.uniform(0.5, 2.0)).astype(np.float32)
            if rng.random() < 0.3:                       # ties across and within samples
                a = np.round(a * 4) / 4
                b = np.round(b * 4) / 4
            assert oracle.ks2(a, b, "port") == oracle.ks2(a, b, "reference")


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden_nmap.npz")


def test_port_matches_reference_golden_tests():
    """Both tests, both argument orders, samples with and without shared
    values: the port's probabilities equal the reference's bit for bit."""
    g = np.load(GOLDEN)
    for n in (2, 3, 5, 10, 16, 30, 45, 64):
        a, b = g["pairs%d/a" % n], g["pairs%d/b" % n]
        for m, f in (("ks2", oracle.ks2), ("ad2", oracle.ad2)):
            ab = np.array([f(a[k], b[k]) for k in range(len(a))])
            ba = np.array([f(b[k], a[k]) for k in range(len(a))])
            assert np.array_equal(ab, g["pairs%d/%s_ab" % (n, m)]), (n, m)
            assert np.array_equal(ba, g["pairs%d/%s_ba" % (n, m)]), (n, m)
    # the AD test is not symmetric when the samples share values
    assert not np.array_equal(g["pairs10/ad2_ab"], g["pairs10/ad2_ba"])
    assert np.array_equal(g["pairs10/ks2_ab"], g["pairs10/ks2_ba"])


def test_port_maps_match_reference_golden_maps():
    g = np.load(GOLDEN)
    for name in ("voronoi", "ties"):
        R, C, N, ny, nx = [int(x) for x in g[name + "/shape"]]
        for m in ("KS2", "AD2"):
            mp, cnt = oracle.nmap(g[name + "/stack"], ny, nx, 0.05, method=m)
            assert np.array_equal(mp, g["%s/%s_nmap" % (name, m)]), (name, m)
            assert np.array_equal(cnt, g["%s/%s_count" % (name, m)]), (name, m)


def test_ad2_known_answers():
    """Identical samples give the smallest statistic (p near 1); disjoint
    samples the largest (p near 0)."""
    a = np.arange(1, 31, dtype=np.float32)
    assert oracle.ad2(a, a) > 0.99
    assert oracle.ad2(a, a + 100.0) < 1e-4
    assert oracle.ad2(a + 100.0, a) < 1e-4


@pytest.mark.skipif(not os.path.exists(oracle.REF_SO), reason="reference-linked oracle not built")
def test_ad2_port_matches_reference_header():
    """The port restates AD2unique::test (src/nmap/AD2unique.hpp:270-347);
    the reference build runs the header itself."""
    rng = np.random.default_rng(4)
    for n in (1, 2, 5, 10, 30, 45, 64):
        for _ in range(200):
            a = rng.rayleigh(1.0, n).astype(np.float32)
            b = (rng.rayleigh(1.0, n) * rng.uniform(0.5, 2.0)).astype(np.float32)
            if rng.random() < 0.3:
                a = np.round(a * 4) / 4
                b = np.round(b * 4) / 4
            pa, ra = oracle.ad2(a, b, "port"), oracle.ad2(a, b, "reference")
            assert pa == ra or (np.isnan(pa) and np.isnan(ra))


@pytest.mark.skipif(not os.path.exists(oracle.REF_SO), reason="reference-linked oracle not built")
def test_nmap_port_matches_reference_build():
    stack, _ = synth.scene("voronoi", 24, 30, 12, 3, 5, seed=9)
    stack[:, 3, 4] = 0                                  # an invalid pixel
    stack[:, 10:14, 6:12] = np.round(stack[:, 10:14, 6:12].real)      # shared values
    for m in ("KS2", "AD2"):
        a = oracle.nmap(stack, 3, 5, 0.05, kind="port", method=m)
        b = oracle.nmap(stack, 3, 5, 0.05, kind="reference", method=m)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]), m


def _bit(m, ny, nx, ii, jj):
    f = (ii + ny) * (2 * nx + 1) + (jj + nx)
    return (m[..., f >> 5] >> np.uint32(f & 31)) & 1


def test_nmap_oracle_structure():
    """Symmetric relation, centre bit on every valid pixel, count = set bits,
    invalid pixels (zero amplitude or masked) empty."""
    ny, nx = 2, 3
    stack, _ = synth.scene("voronoi", 20, 22, 10, ny, nx, seed=4)
    stack[4, 7, 8] = 0
    mask = np.ones((20, 22), np.uint8)
    mask[10, 11] = 0
    m, cnt = oracle.nmap(stack, ny, nx, 0.05, mask=mask)
    R, C = cnt.shape
    assert _bit(m, ny, nx, 0, 0)[7, 8] == 0 and cnt[7, 8] == 0
    assert _bit(m, ny, nx, 0, 0)[10, 11] == 0 and cnt[10, 11] == 0
    pop = np.zeros_like(cnt)
    for ii in range(-ny, ny + 1):
        for jj in range(-nx, nx + 1):
            b = _bit(m, ny, nx, ii, jj).astype(np.int32)
            pop += b
            for r in range(R):
                for c in range(C):
                    rr, cc = r + ii, c + jj
                    if b[r, c]:
                        assert 0 <= rr < R and 0 <= cc < C
                        assert _bit(m, ny, nx, -ii, -jj)[rr, cc] == 1
    assert np.array_equal(pop, cnt)
    valid = cnt > 0
    assert valid.sum() == R * C - 2


def test_float_modulus_formula_matches_libm():
    """The GPU forms |x| as sqrt(x^2 + y^2) in FP64 rounded to float; the
    reference's std::abs(complex<float>) calls libm's cabsf / hypotf.  Pin
    that they agree on this machine's libm."""
    import ctypes
    import ctypes.util
    libm = ctypes.CDLL(ctypes.util.find_library("m"))
    f = libm.hypotf
    f.restype = ctypes.c_float
    f.argtypes = [ctypes.c_float, ctypes.c_float]
    rng = np.random.default_rng(7)
    x = (rng.standard_normal(20000) * 10.0 ** rng.uniform(-15, 15, 20000)).astype(np.float32)
    y = (rng.standard_normal(20000) * 10.0 ** rng.uniform(-15, 15, 20000)).astype(np.float32)
    ref = np.array([f(float(a), float(b)) for a, b in zip(x, y)], np.float32)
    mine = np.sqrt(x.astype(np.float64) ** 2 + y.astype(np.float64) ** 2).astype(np.float32)
    assert np.array_equal(ref, mine)
