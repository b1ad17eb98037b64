"""Seeded synthetic SLC stacks and SHP bitmasks.

Scenes follow the coherence / deformation model of FRInGE's own test
simulator (tests/evd/test_evd.py:14-71): a per-pixel coherence matrix
``G_ij = gamma(|t_i - t_j|) * exp(i (phi_i - phi_j))`` with
``gamma(dt) = (gamma0 - gamma_inf) * exp(-dt / tau) + gamma_inf``, and samples
``x = sqrt(G) z`` where ``sqrt`` is the eigen square root with eigenvalues
below 1e-3 clipped to zero (test_evd.py:17-20) and ``z`` is circular Gaussian
with unit-variance real and imaginary parts (so |x| is Rayleigh, sigma = 1).

Because ``exp(i phi)`` enters as a diagonal unitary ``D``,
``sqrt(D G0 D^H) z = D sqrt(G0) (D^H z)`` and ``D^H z`` has the law of ``z``;
one square root per distinct ``G0`` therefore serves every pixel.

The neighbourhood bitmask uses the Ulongmask layout
(include/fringe/ulongmask.hpp:55-94): offset (ii, jj) in [-Ny,Ny] x [-Nx,Nx]
maps to flat index (ii+Ny)(2Nx+1)+jj+Nx, bit flat%32 of uint32 word flat/32.
"""
from __future__ import annotations

import math

import numpy as np

WAVELENGTH_M = 0.0555      # C-band, 5.55 cm
DAYS_PER_YEAR = 365.25


def nulong_for(ny: int, nx: int) -> int:
    """uint32 words per pixel for a (2ny+1) x (2nx+1) window (evd.cpp:47-48)."""
    return ((2 * ny + 1) * (2 * nx + 1) + 31) // 32


def coherence_matrix(nbands: int, gamma0: float = 0.9, gamma_inf: float = 0.2,
                     tau_days: float = 24.0, spacing_days: float = 12.0) -> np.ndarray:
    """Real temporal coherence G0 (unit diagonal) on a regular date grid."""
    t = np.arange(nbands) * spacing_days
    dt = np.abs(t[:, None] - t[None, :])
    g = (gamma0 - gamma_inf) * np.exp(-dt / tau_days) + gamma_inf
    np.fill_diagonal(g, 1.0)
    return g


def eig_sqrt(g: np.ndarray, clip: float = 1e-3) -> np.ndarray:
    """Eigen square root with small eigenvalues clipped (test_evd.py:17-20)."""
    w, v = np.linalg.eigh(g)
    w = np.where(w < clip, 0.0, w)
    return (v * np.sqrt(w)[None, :]) @ v.conj().T


def velocity_ramp(rows: int, cols: int, vmax_m_per_yr: float = 0.030) -> np.ndarray:
    """Smooth 2-D ramp of line-of-sight velocity, 0 .. vmax over the scene."""
    r = np.linspace(0.0, 1.0, rows, dtype=np.float64)[:, None]
    c = np.linspace(0.0, 1.0, cols, dtype=np.float64)[None, :]
    return vmax_m_per_yr * 0.5 * (r + c)


def voronoi_classes(rows: int, cols: int, nclasses: int, rng: np.random.Generator,
                    cell_px: float = 18.0) -> np.ndarray:
    """Piecewise-constant class map from seeded Voronoi cells."""
    nsites = max(1, int(rows * cols / (cell_px * cell_px)))
    sy = rng.uniform(0, rows, nsites)
    sx = rng.uniform(0, cols, nsites)
    cls = rng.integers(0, nclasses, nsites)
    try:
        from scipy.spatial import cKDTree
        tree = cKDTree(np.stack([sy, sx], axis=1))
        out = np.empty((rows, cols), np.int32)
        yy = np.arange(rows, dtype=np.float64)
        xx = np.arange(cols, dtype=np.float64)
        step = max(1, 1 << 20 // max(cols, 1))
        for r0 in range(0, rows, step):
            r1 = min(rows, r0 + step)
            q = np.stack(np.meshgrid(yy[r0:r1], xx, indexing="ij"), axis=-1).reshape(-1, 2)
            _, idx = tree.query(q)
            out[r0:r1] = cls[idx].reshape(r1 - r0, cols)
        return out
    except ImportError:  # brute force fallback for small scenes
        yy, xx = np.mgrid[0:rows, 0:cols]
        d = (yy[..., None] - sy) ** 2 + (xx[..., None] - sx) ** 2
        return cls[np.argmin(d, axis=-1)].astype(np.int32)


def nmap_from_classes(classes: np.ndarray, ny: int, nx: int) -> np.ndarray:
    """SHP bitmask: bit set iff the neighbour lies in the scene and has the
    centre pixel's class.  Returns uint32 [rows, cols, nulong]."""
    rows, cols = classes.shape
    nl = nulong_for(ny, nx)
    out = np.zeros((rows, cols, nl), np.uint32)
    wx = 2 * nx + 1
    for ii in range(-ny, ny + 1):
        for jj in range(-nx, nx + 1):
            flat = (ii + ny) * wx + jj + nx
            w, b = divmod(flat, 32)
            r0, r1 = max(0, -ii), min(rows, rows - ii)
            c0, c1 = max(0, -jj), min(cols, cols - jj)
            if r0 >= r1 or c0 >= c1:
                continue
            eq = classes[r0:r1, c0:c1] == classes[r0 + ii:r1 + ii, c0 + jj:c1 + jj]
            out[r0:r1, c0:c1, w] |= (eq.astype(np.uint32) << np.uint32(b))
    return out


def nmap_all_ones(rows: int, cols: int, ny: int, nx: int) -> np.ndarray:
    """Every window bit set (the reference clips the window to the scene)."""
    nl = nulong_for(ny, nx)
    k = (2 * ny + 1) * (2 * nx + 1)
    words = np.zeros(nl, np.uint32)
    for f in range(k):
        words[f // 32] |= np.uint32(1) << np.uint32(f % 32)
    return np.broadcast_to(words, (rows, cols, nl)).copy()


def simulate_stack(rows: int, cols: int, nbands: int, seed: int, *,
                   gamma0=0.9, gamma_inf=0.2, tau_days=24.0, spacing_days=12.0,
                   amp_scale: np.ndarray | None = None,
                   vmax_m_per_yr: float = 0.030) -> np.ndarray:
    """complex64 stack [nbands, rows, cols], band-planar like the reference.

    gamma0 / gamma_inf may be scalars or per-pixel arrays [rows, cols]; per
    pixel values are quantised to 1/256 so that one square root serves each
    distinct pair.
    """
    rng = np.random.Generator(np.random.PCG64(seed))
    npx = rows * cols
    z = (rng.standard_normal((nbands, npx), dtype=np.float32)
         + 1j * rng.standard_normal((nbands, npx), dtype=np.float32)).astype(np.complex64)
    g0 = np.broadcast_to(np.asarray(gamma0, np.float64), (rows, cols)).reshape(-1)
    gi = np.broadcast_to(np.asarray(gamma_inf, np.float64), (rows, cols)).reshape(-1)
    q0 = np.round(g0 * 256.0).astype(np.int64)
    qi = np.round(gi * 256.0).astype(np.int64)
    key = q0 * 1024 + qi
    x = np.empty_like(z)
    for k in np.unique(key):
        sel = np.nonzero(key == k)[0]
        a0, ai = (k // 1024) / 256.0, (k % 1024) / 256.0
        L = eig_sqrt(coherence_matrix(nbands, a0, ai, tau_days, spacing_days)).astype(np.complex64)
        x[:, sel] = L @ z[:, sel]
    t_yr = np.arange(nbands) * spacing_days / DAYS_PER_YEAR
    v = velocity_ramp(rows, cols, vmax_m_per_yr).reshape(-1)
    for k in range(nbands):
        ph = (2.0 * math.pi / WAVELENGTH_M) * v * t_yr[k]
        x[k] *= np.exp(1j * ph).astype(np.complex64)
    if amp_scale is not None:
        x *= np.asarray(amp_scale, np.float32).reshape(1, -1)
    return x.reshape(nbands, rows, cols)


def indefinite_abs_coherence(nbands: int, rng: np.random.Generator,
                              below: float = -0.3, tries: int = 20000,
                              ridge: float = 0.02) -> np.ndarray:
    """A coherence matrix C0 = V V^H + ridge I (V complex, nbands x 2) scaled
    to a unit diagonal, drawn until its magnitude |C0| has an eigenvalue
    below `below`.  C0 is positive definite; the sample coherence of a
    window of its draws keeps an indefinite magnitude (the reference's code
    -4 in the evd module, the EVD fall-back in phase_link).  From 4 dates up
    a draw is found quickly; at 2 none exists (a 2 x 2 |C0| is positive
    semi-definite) and at 3 none turned up in 20,000 draws: ValueError after
    `tries` draws."""
    for _ in range(tries):
        V = rng.standard_normal((nbands, 2)) + 1j * rng.standard_normal((nbands, 2))
        C0 = V @ V.conj().T + ridge * np.eye(nbands)
        d = np.sqrt(np.real(np.diag(C0)))
        C0 = C0 / np.outer(d, d)
        if np.linalg.eigvalsh(np.abs(C0))[0] < below:
            return C0
    raise ValueError("no %d-date coherence with lambda_min(|C|) < %g in %d draws" % (nbands, below, tries))


def scene(kind: str, rows: int, cols: int, nbands: int, ny: int, nx: int,
          seed: int):
    """Build (stack, nmap) for one of the workload families.

    kind = "uniform"  : gamma(dt)=0.7exp(-dt/24)+0.2, nmap all ones.
    kind = "voronoi"  : same coherence, 8 amplitude classes on Voronoi cells,
                        nmap = same-class neighbours.
    kind = "illcond"  : gamma0 ~ U(0.05, 0.9) per pixel, 10% of pixels with
                        gamma_inf = 0 (else 0.2), Voronoi nmap.
    kind = "indefabs" : every pixel drawn from one positive definite
                        coherence whose magnitude matrix is indefinite (see
                        indefinite_abs_coherence; ridge 0.02 up to 32 dates,
                        0.5 above, which keeps lambda_min(C) of a window's
                        sample coherence near 0.016 at 64 dates, clear of
                        the FP32 rounding band of the 1e-6 test), nmap all
                        ones.
    """
    rng = np.random.Generator(np.random.PCG64(seed + 7919))
    if kind == "uniform":
        st = simulate_stack(rows, cols, nbands, seed)
        return st, nmap_all_ones(rows, cols, ny, nx)
    if kind == "indefabs":
        ridge = 0.02 if nbands <= 32 else 0.5
        L = np.linalg.cholesky(indefinite_abs_coherence(nbands, rng, ridge=ridge))
        z = (rng.standard_normal((nbands, rows * cols))
             + 1j * rng.standard_normal((nbands, rows * cols))) / np.sqrt(2.0)
        st = (L @ z).reshape(nbands, rows, cols).astype(np.complex64)
        return st, nmap_all_ones(rows, cols, ny, nx)
    classes = voronoi_classes(rows, cols, 8, rng)
    amp = (1.0 + 0.5 * classes).astype(np.float32)
    if kind == "voronoi":
        st = simulate_stack(rows, cols, nbands, seed, amp_scale=amp)
    elif kind == "illcond":
        g0 = rng.uniform(0.05, 0.9, (rows, cols))
        gi = np.where(rng.uniform(0, 1, (rows, cols)) < 0.1, 0.0, 0.2)
        gi = np.minimum(gi, g0)
        st = simulate_stack(rows, cols, nbands, seed, gamma0=g0, gamma_inf=gi,
                            amp_scale=amp)
    else:
        raise ValueError(kind)
    return st, nmap_from_classes(classes, ny, nx)
