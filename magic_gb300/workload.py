"""Seeded synthetic inputs and the per-level field set of the radial loop.

Field set (src/rIter.f90): spectral -> grid (transform_to_grid_space,
:466-622) takes 13 spectral fields and produces 15 grids; grid -> spectral
(transform_to_lm_space, :624-712) takes 10 grids and produces 10 spectral
fields.  Spectra are Gaussian with standard deviation (l+1)^-2, the m = 0
imaginary parts are zero, levels are independent, and an optional radial
envelope sin(pi (r - r_i)/(r_o - r_i)) on Chebyshev-Gauss-Lobatto radii in
[0.538, 1.538] modulates the amplitude.
"""
from __future__ import annotations

import numpy as np

from ._lib import GRID_SPACE_IN, LM_SPACE_IN

R_ICB, R_CMB = 0.538, 1.538

# grid -> spectral inputs taken from the inverse outputs when no nonlinear
# products are formed (the standalone forward benchmark)
FORWARD_FROM_INVERSE = {
    "Advr": "vrc", "Advt": "vtc", "Advp": "vpc",
    "VSr": "cvrc", "VSt": "cvtc", "VSp": "cvpc",
    "VxBr": "brc", "VxBt": "btc", "VxBp": "bpc",
    "heatTerms": "sc",
}


def lm_arrays(l_max: int, minc: int, m_max: int = 0):
    if m_max <= 0:
        m_max = (l_max // minc) * minc
    ell = np.array([l for m in range(0, m_max + 1, minc) for l in range(m, l_max + 1)])
    em = np.array([m for m in range(0, m_max + 1, minc) for l in range(m, l_max + 1)])
    return ell, em


def radii(n_r: int) -> np.ndarray:
    """Chebyshev-Gauss-Lobatto radii mapped onto [r_icb, r_cmb] (outer first)."""
    k = np.arange(n_r)
    x = np.cos(np.pi * k / max(n_r - 1, 1))
    return 0.5 * (R_CMB + R_ICB) + 0.5 * (R_CMB - R_ICB) * x


def spectra(l_max: int, minc: int, n_levels: int, seed: int, envelope: bool = False,
            m_max: int = 0) -> np.ndarray:
    """(n_levels, lm_max) complex128 with std (l+1)^-2, Im = 0 for m = 0."""
    ell, em = lm_arrays(l_max, minc, m_max)
    rng = np.random.Generator(np.random.PCG64(seed))
    K = ell.size
    re = rng.standard_normal((n_levels, K))
    im = rng.standard_normal((n_levels, K))
    s = (re + 1j * im) * (ell + 1.0) ** -2
    s[:, em == 0] = s[:, em == 0].real
    if envelope:
        r = radii(n_levels)
        env = np.sin(np.pi * (r - R_ICB) / (R_CMB - R_ICB))
        env[np.abs(env) < 1e-3] = 1e-3  # keep the boundary levels non-trivial
        s = s * env[:, None]
    return s


def grid_space_inputs(l_max: int, minc: int, n_levels: int, seed: int = 1234,
                      envelope: bool = True, fields=GRID_SPACE_IN) -> dict:
    out = {}
    for i, k in enumerate(fields):
        out[k] = spectra(l_max, minc, n_levels, seed + 1000 * i, envelope)
    return out


def or2_levels(n_levels: int) -> np.ndarray:
    return 1.0 / radii(n_levels) ** 2
