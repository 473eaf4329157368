"""Generate the committed golden fixtures of tests/golden/.

Run in the development container (it reads the reference tree, which is not
present where the tests later run):

    python tests/golden/make_golden.py /path/to/magic-reference

Produces
  kat.npz                 analytic / independent known answers: Gauss-Legendre
                          nodes (numpy.polynomial.legendre.leggauss), orthonormal
                          P_lm without Condon-Shortley phase and sin(theta) dP/dtheta
                          (scipy.special.sph_harm_y), real-FFT conventions
                          (numpy.fft) of the reference's fft991 definition.
  checkpoint_spectra.npz  real spectra of the reference's own sample
                          samples/boussBenchSat/checkpoint_end.start (l_max=64,
                          minc=4), read with the reference's python reader
                          python/magic/checkpoint.py (MagicCheckpoint.read).
  oracle_small.npz        inputs and outputs of the oracle (oracle/sht_oracle.cpp)
                          for small seeded cases and for the checkpoint spectra.
"""
from __future__ import annotations

import importlib.util
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def load_reference_checkpoint_reader(ref: str):
    # the reference package imports matplotlib in its __init__; load only the
    # checkpoint module with the three helpers it names stubbed out
    pkg = types.ModuleType("magic")
    pkg.__path__ = []
    lib = types.ModuleType("magic.libmagic")
    # Gauss-Lobatto points (only the inner-core radii of the reader use it)
    lib.chebgrid = lambda nr, a, b: 0.5 * (a + b) + 0.5 * (a - b) * np.cos(np.pi * np.arange(nr + 1) / nr)
    lib.fd_grid = lambda *a, **k: None
    lib.scanDir = lambda *a, **k: []
    sys.modules["magic"] = pkg
    sys.modules["magic.libmagic"] = lib
    spec = importlib.util.spec_from_file_location(
        "magic.checkpoint", os.path.join(ref, "python", "magic", "checkpoint.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def make_kat(path):
    from scipy.special import sph_harm_y
    out = {}
    for n in (24, 96):
        x, w = np.polynomial.legendre.leggauss(n)
        # reference order: colatitudes north -> south, i.e. cos(theta) descending
        out["gauss_theta_%d" % n] = np.arccos(x[::-1])
        out["gauss_w_%d" % n] = w[::-1].copy()
    L = 20
    thetas = np.array([0.1, 0.55, 1.0, 1.4, 1.5707963267948966])
    P = []
    dP = []
    h = 1e-6
    for t in thetas:
        row, drow = [], []
        for m in range(0, L + 1):
            for l in range(m, L + 1):
                ph = (-1) ** m
                row.append(ph * np.real(sph_harm_y(l, m, t, 0.0)))
                fp = ph * np.real(sph_harm_y(l, m, t + h, 0.0))
                fm = ph * np.real(sph_harm_y(l, m, t - h, 0.0))
                drow.append((fp - fm) / (2 * h) * np.sin(t))
        P.append(row)
        dP.append(drow)
    out["plm_L"] = np.array(L)
    out["plm_theta"] = thetas
    out["plm"] = np.array(P)
    out["dplm_fd"] = np.array(dP)
    rng = np.random.Generator(np.random.PCG64(11))
    for P_ in (24, 192):
        x = rng.standard_normal(P_)
        out["fft_x_%d" % P_] = x
        out["fft_fwd_%d" % P_] = np.fft.rfft(x) / P_
        c = rng.standard_normal(P_ // 2 + 1) + 1j * rng.standard_normal(P_ // 2 + 1)
        out["fft_c_%d" % P_] = c
        out["fft_inv_%d" % P_] = np.fft.irfft(c, P_) * P_
    np.savez_compressed(path, **out)


def make_checkpoint(ref, path):
    mod = load_reference_checkpoint_reader(ref)
    chk = mod.MagicCheckpoint(l_read=False)
    chk.read(os.path.join(ref, "samples", "boussBenchSat", "checkpoint_end.start"))
    levels = np.array([0, 8, 16, 24, 32])
    out = dict(l_max=np.array(chk.l_max), minc=np.array(chk.minc), m_max=np.array(chk.m_max),
               n_theta_max=np.array(chk.n_theta_max), n_phi_tot=np.array(chk.n_phi_tot),
               lm_max=np.array(chk.lm_max), radius=chk.radius[levels], levels=levels,
               wpol=chk.wpol[levels], ztor=chk.ztor[levels], entropy=chk.entropy[levels])
    if getattr(chk, "bpol", None) is not None:
        out["bpol"] = chk.bpol[levels]
        out["btor"] = chk.btor[levels]
    np.savez_compressed(path, **out)


def make_oracle(cp_path, path):
    from oracle.oracle import OracleSHT
    from magic_gb300.workload import spectra
    out = {}
    # seeded case, l_max=15, minc=1, n_theta=24, n_phi=48, lcut=11
    L, minc, N, P = 15, 1, 24, 48
    o = OracleSHT(L, minc, N, P)
    S = spectra(L, minc, 4, seed=5)
    out["s15_in"] = S
    out["s15_scal"] = o.scal_to_spat(S[0])
    out["s15_scal_lcut11"] = o.scal_to_spat(S[0], 11)
    out["s15_qst"] = np.array(o.torpol_to_spat(S[0], S[1], S[2]))
    out["s15_curl"] = np.array(o.torpol_to_curl_spat(0.7, S[0], S[3], S[1], S[2]))
    out["s15_sphtor"] = np.array(o.sphtor_to_spat(S[1], S[2]))
    out["s15_grad"] = np.array(o.scal_to_grad_spat(S[0]))
    out["s15_dph"] = np.array(o.torpol_to_dphspat(S[1], S[2]))
    g = out["s15_qst"]
    out["s15_fwd_qst"] = np.array(o.spat_to_qst(g[0], g[1], g[2]))
    out["s15_fwd_sh_lcut11"] = o.scal_to_SH(g[0], 11)
    # the reference's own checkpoint spectra (l_max=64, minc=4)
    cp = np.load(cp_path)
    L, minc = int(cp["l_max"]), int(cp["minc"])
    N = int(cp["n_theta_max"])
    P = int(cp["n_phi_tot"]) // minc
    o = OracleSHT(L, minc, N, P)
    w, z, s = cp["wpol"][2], cp["ztor"][2], cp["entropy"][2]
    out["cp_dims"] = np.array([L, minc, N, P])
    out["cp_scal"] = o.scal_to_spat(s)
    out["cp_qst"] = np.array(o.torpol_to_spat(w, w, z))
    g = out["cp_qst"]
    out["cp_fwd_qst"] = np.array(o.spat_to_qst(g[0], g[1], g[2]))
    np.savez_compressed(path, **out)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MAGIC_REFERENCE", "")
    if not ref or not os.path.isdir(ref):
        sys.exit("usage: make_golden.py <reference tree>")
    make_kat(os.path.join(HERE, "kat.npz"))
    make_checkpoint(ref, os.path.join(HERE, "checkpoint_spectra.npz"))
    make_oracle(os.path.join(HERE, "checkpoint_spectra.npz"), os.path.join(HERE, "oracle_small.npz"))
    for f in ("kat.npz", "checkpoint_spectra.npz", "oracle_small.npz"):
        print(f, os.path.getsize(os.path.join(HERE, f)), "bytes")
