"""The oracle (CPU restatement of the reference's native transforms) against
independent known answers: Gauss-Legendre nodes from numpy, orthonormal
Legendre functions from scipy (the reference's norm=2, no Condon-Shortley
phase, src/plms.f90:14-189), numpy FFT for the fft991 definition
(src/fft.f90:262-268), analytic spherical harmonics, round-trip identities
and the committed golden vectors."""
import os

import numpy as np
import pytest

from conftest import rel_l2, rel_max

GOLD = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def kat():
    return np.load(os.path.join(GOLD, "kat.npz"))


def test_gauleg_matches_numpy(oracle_mod, kat):
    for n in (24, 96):
        th, w = oracle_mod.gauleg(n)
        assert np.abs(th - kat["gauss_theta_%d" % n]).max() < 1e-13
        assert np.abs(w - kat["gauss_w_%d" % n]).max() < 1e-13


def test_plm_matches_scipy(oracle_mod, kat):
    L = int(kat["plm_L"])
    for i, t in enumerate(kat["plm_theta"]):
        p, dp = oracle_mod.plm_theta(t, L, L, 1)
        assert np.abs(p - kat["plm"][i]).max() < 1e-13
        assert np.abs(dp - kat["dplm_fd"][i]).max() < 1e-7


def test_fft_conventions(oracle_mod, kat):
    for P in (24, 192):
        c = oracle_mod.rfft_forward(kat["fft_x_%d" % P])
        assert np.abs(c - kat["fft_fwd_%d" % P]).max() < 1e-14
        x = oracle_mod.rfft_inverse(kat["fft_c_%d" % P], P)
        assert np.abs(x - kat["fft_inv_%d" % P]).max() < 1e-12


def _grid_angles(o):
    th, _ = oracle_mod_gauleg(o.n_theta_max)
    rows = np.empty(o.n_theta_max)
    rows[0::2] = th[: o.n_theta_max // 2]            # north, scrambled order
    rows[1::2] = th[::-1][: o.n_theta_max // 2]      # matching south points
    phi = 2 * np.pi * np.arange(o.n_phi_max) / (o.n_phi_max * o.minc)
    return rows, phi


def oracle_mod_gauleg(n):
    from oracle import oracle
    return oracle.gauleg(n)


def test_analytic_harmonics(oracle_mod):
    o = oracle_mod.OracleSHT(15, 1, 24, 48)
    th, ph = _grid_angles(o)
    TH, PH = np.meshgrid(th, ph)  # (n_phi, n_theta)
    S = np.zeros(o.lm_max, complex)
    S[0] = 1.0
    assert np.abs(o.scal_to_spat(S) - 1 / np.sqrt(4 * np.pi)).max() < 1e-14
    S[:] = 0
    S[1] = 1.0  # l=1, m=0
    assert np.abs(o.scal_to_spat(S) - np.sqrt(3 / (4 * np.pi)) * np.cos(TH)).max() < 1e-14
    S[:] = 0
    c = 0.3 - 0.7j
    S[o.l_max + 1] = c  # l=1, m=1 (first entry of the m=1 block)
    ref = 2 * np.sqrt(3 / (8 * np.pi)) * np.sin(TH) * (c.real * np.cos(PH) - c.imag * np.sin(PH))
    assert np.abs(o.scal_to_spat(S) - ref).max() < 1e-14
    # spheroidal l=1,m=0: v_theta (Robert form) = S sin(theta) dY10/dtheta
    S[:] = 0
    S[1] = 1.0
    vt, vp = o.sphtor_to_spat(S, np.zeros_like(S))
    assert np.abs(vt + np.sqrt(3 / (4 * np.pi)) * np.sin(TH) ** 2).max() < 1e-14
    assert np.abs(vp).max() < 1e-14


def test_round_trips(oracle_mod):
    from magic_gb300.workload import spectra
    for (L, minc, N, P) in ((31, 1, 48, 96), (64, 4, 96, 48)):
        o = oracle_mod.OracleSHT(L, minc, N, P)
        S = spectra(L, minc, 3, seed=3, m_max=o.m_max)
        ell = np.array([l for m in range(0, o.m_max + 1, minc) for l in range(m, L + 1)])
        assert rel_max(o.scal_to_SH(o.scal_to_spat(S[0])), S[0]) < 1e-13
        W, dW, Z = S
        W[0] = dW[0] = Z[0] = 0
        q, s, t = o.spat_to_qst(*o.torpol_to_spat(W, dW, Z))
        assert rel_max(q, ell * (ell + 1) * W) < 1e-12
        assert rel_max(s, dW) < 1e-12 and rel_max(t, Z) < 1e-12


def test_lcut_truncates(oracle_mod):
    from magic_gb300.workload import spectra
    o = oracle_mod.OracleSHT(31, 1, 48, 96)
    S = spectra(31, 1, 1, seed=9)[0]
    ell = np.array([l for m in range(0, 32) for l in range(m, 32)])
    St = S.copy()
    St[ell > 20] = 0
    assert rel_max(o.scal_to_spat(S, 20), o.scal_to_spat(St)) < 1e-15
    f = o.scal_to_spat(S)
    out = o.scal_to_SH(f, 20)
    assert np.all(out[ell > 20] == 0)
    assert rel_max(out[ell <= 20], S[ell <= 20]) < 1e-13


def test_golden_vectors(oracle_mod):
    g = np.load(os.path.join(GOLD, "oracle_small.npz"))
    o = oracle_mod.OracleSHT(15, 1, 24, 48)
    S = g["s15_in"]
    assert rel_max(o.scal_to_spat(S[0]), g["s15_scal"]) < 1e-14
    assert rel_max(o.scal_to_spat(S[0], 11), g["s15_scal_lcut11"]) < 1e-14
    assert rel_max(np.array(o.torpol_to_spat(S[0], S[1], S[2])), g["s15_qst"]) < 1e-14
    assert rel_max(np.array(o.torpol_to_curl_spat(0.7, S[0], S[3], S[1], S[2])), g["s15_curl"]) < 1e-14
    assert rel_max(np.array(o.torpol_to_dphspat(S[1], S[2])), g["s15_dph"]) < 1e-14
    q = g["s15_qst"]
    assert rel_max(np.array(o.spat_to_qst(q[0], q[1], q[2])), g["s15_fwd_qst"]) < 1e-13
    L, minc, N, P = [int(x) for x in g["cp_dims"]]
    cp = np.load(os.path.join(GOLD, "checkpoint_spectra.npz"))
    o = oracle_mod.OracleSHT(L, minc, N, P)
    assert o.lm_max == int(cp["lm_max"])
    w, z, s = cp["wpol"][2], cp["ztor"][2], cp["entropy"][2]
    assert rel_max(o.scal_to_spat(s), g["cp_scal"]) < 1e-14
    assert rel_max(np.array(o.torpol_to_spat(w, w, z)), g["cp_qst"]) < 1e-14


def test_truncation_rules(oracle_mod):
    from magic_gb300.sht import truncation
    for L in (63, 64, 127, 128, 255, 511, 85, 170):
        for minc in (1, 4):
            a = truncation(L, minc=minc)
            b = oracle_mod.truncation(L, 20, minc)
            for k in ("n_theta_max", "n_phi_tot", "n_phi_max", "m_max", "n_m_max", "lm_max"):
                assert a[k] == b[k], (L, minc, k)
    assert truncation(255)["n_theta_max"] == 384 and truncation(255)["n_phi_max"] == 768
    assert truncation(511)["n_theta_max"] == 768


def test_radial_blocks():
    from magic_gb300.radial import radial_blocks
    for n in (1, 7, 33, 129):
        for p in (1, 2, 3, 4, 8):
            if p > n:
                continue
            b = radial_blocks(n, p)
            assert b[0][0] == 0 and b[-1][1] == n
            for (s0, e0), (s1, e1) in zip(b, b[1:]):
                assert e0 == s1 and e0 > s0
            sizes = [e - s for s, e in b]
            assert max(sizes) - min(sizes) <= 1
            assert sizes == sorted(sizes)  # remainder on the last ranks
