"""ORACLE — test infrastructure only.

ctypes wrapper around ``oracle/sht_oracle.cpp``, the CPU FP64 restatement of
MagIC's native spherical-harmonic transforms (src/sht_native.f90,
src/shtransforms.f90, src/plms.f90, src/horizontal.f90:279-340, src/fft.f90).
Only the tests, ``__graft_entry__.smoke()`` and the CPU legs of ``bench.py``
use it, as the checker / the timed CPU reference.  The GPU library never
loads it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "sht_oracle.cpp")
_LIB = os.path.join(_HERE, "liboracle_sht.so")

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)


def build_oracle(force: bool = False) -> str:
    """Compile the oracle with g++ (OpenMP over theta blocks like the reference)."""
    if (not force and os.path.exists(_LIB)
            and os.path.getmtime(_LIB) >= os.path.getmtime(_SRC)):
        return _LIB
    tmp = _LIB + ".tmp%d" % os.getpid()
    cmd = ["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-o", tmp, _SRC]
    subprocess.check_call(cmd)
    os.replace(tmp, _LIB)
    return _LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build_oracle()
        L = ctypes.CDLL(_LIB)
        vp = ctypes.c_void_p
        L.oracle_init.restype = vp
        L.oracle_init.argtypes = [ctypes.c_int] * 5
        L.oracle_free.argtypes = [vp]
        L.oracle_sizes.argtypes = [vp, _I]
        L.oracle_tables.argtypes = [vp, _D, _D, _D, _D]
        L.oracle_gauleg.argtypes = [ctypes.c_int, _D, _D]
        L.oracle_plm_theta.argtypes = [ctypes.c_double] + [ctypes.c_int] * 4 + [_D, _D]
        L.oracle_truncation.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, _I]
        L.oracle_set_threads.argtypes = [ctypes.c_int]
        L.oracle_max_threads.restype = ctypes.c_int
        L.oracle_rfft_inverse.argtypes = [ctypes.c_int, _D, _D]
        L.oracle_rfft_forward.argtypes = [ctypes.c_int, _D, _D]
        i = ctypes.c_int
        d = ctypes.c_double
        sig = {
            "scal_to_spat": [vp, _D, _D, i],
            "scal_to_grad_spat": [vp, _D, _D, _D, i],
            "pol_to_grad_spat": [vp, _D, _D, _D, i],
            "torpol_to_spat": [vp, _D, _D, _D, _D, _D, _D, i],
            "sphtor_to_spat": [vp, _D, _D, _D, _D, i],
            "torpol_to_curl_spat_IC": [vp, d, d, _D, _D, _D, _D, _D, _D, _D],
            "torpol_to_spat_IC": [vp, d, d, _D, _D, _D, _D, _D, _D],
            "torpol_to_dphspat": [vp, _D, _D, _D, _D, i],
            "pol_to_curlr_spat": [vp, _D, _D, i],
            "torpol_to_curl_spat": [vp, d, _D, _D, _D, _D, _D, _D, _D, i],
            "scal_to_SH": [vp, _D, _D, i],
            "spat_to_qst": [vp, _D, _D, _D, _D, _D, _D, i],
            "spat_to_sphertor": [vp, _D, _D, _D, _D, i],
            "axi_to_spat": [vp, _D, _D],
            "toraxi_to_spat": [vp, _D, _D, _D, i],
        }
        for name, args in sig.items():
            f = getattr(L, "oracle_" + name)
            f.argtypes = args
            f.restype = None
        _lib = L
    return _lib


def _p(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_D)


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def gauleg(n: int):
    th = np.zeros(n)
    w = np.zeros(n)
    lib().oracle_gauleg(n, _p(th), _p(w))
    return th, w


def plm_theta(theta: float, l_max: int, m_max: int, minc: int):
    K = sum(l_max - m + 1 for m in range(0, m_max + 1, minc))
    p = np.zeros(K + 1)
    dp = np.zeros(K + 1)
    lib().oracle_plm_theta(float(theta), l_max, 0, m_max, minc, _p(p), _p(dp))
    return p[:K], dp[:K]


def truncation(l_max: int, nalias: int = 20, minc: int = 1) -> dict:
    out = (ctypes.c_int * 6)()
    lib().oracle_truncation(l_max, nalias, minc, out)
    keys = ["n_theta_max", "n_phi_tot", "n_phi_max", "m_max", "n_m_max", "lm_max"]
    return dict(zip(keys, list(out)))


def rfft_inverse(c: np.ndarray, P: int) -> np.ndarray:
    c = np.ascontiguousarray(c, dtype=np.complex128)
    x = np.zeros(P)
    lib().oracle_rfft_inverse(P, c.view(np.float64).ctypes.data_as(_D), _p(x))
    return x


def rfft_forward(x: np.ndarray) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    P = x.shape[0]
    c = np.zeros(P // 2 + 1, dtype=np.complex128)
    lib().oracle_rfft_forward(P, _p(x), c.view(np.float64).ctypes.data_as(_D))
    return c


class OracleSHT:
    """The reference's `module sht` on the CPU, with its public names.

    Spectral arrays: complex128 (lm_max,) in st_map order.  Grid arrays:
    float64 (n_phi_max, n_theta_max) C-order == Fortran f(n_theta, n_phi).
    """

    def __init__(self, l_max: int, minc: int, n_theta_max: int, n_phi_max: int,
                 m_max: int = 0):
        h = lib().oracle_init(l_max, minc, n_theta_max, n_phi_max, m_max)
        if not h:
            raise ValueError("oracle_init rejected the grid")
        self._h = ctypes.c_void_p(h)
        s = (ctypes.c_int * 7)()
        lib().oracle_sizes(self._h, s)
        (self.l_max, self.m_max, self.minc, self.n_theta_max, self.n_phi_max,
         self.n_m_max, self.lm_max) = list(s)

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                lib().oracle_free(self._h)
                self._h = None
        except Exception:
            pass

    # -- helpers
    def _grid(self):
        return np.zeros((self.n_phi_max, self.n_theta_max))

    def _spec(self):
        return np.zeros(self.lm_max, dtype=np.complex128)

    @staticmethod
    def _c(a):
        a = np.ascontiguousarray(a, dtype=np.complex128)
        return a, a.view(np.float64).ctypes.data_as(_D)

    @staticmethod
    def _r(a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        return a, a.ctypes.data_as(_D)

    def tables(self):
        nh = self.n_theta_max // 2
        th = np.zeros(self.n_theta_max)
        w = np.zeros(self.n_theta_max)
        P = np.zeros((nh, self.lm_max))
        dP = np.zeros((nh, self.lm_max))
        lib().oracle_tables(self._h, _p(th), _p(w), _p(P), _p(dP))
        return th, w, P, dP

    def _lc(self, lcut):
        return self.l_max if lcut is None else int(lcut)

    # -- public names of src/sht_native.f90:16-20
    def scal_to_spat(self, Slm, lcut=None):
        S, ps = self._c(Slm)
        f = self._grid()
        lib().oracle_scal_to_spat(self._h, ps, _p(f), self._lc(lcut))
        return f

    def scal_to_grad_spat(self, Slm, lcut=None):
        S, ps = self._c(Slm)
        a, b = self._grid(), self._grid()
        lib().oracle_scal_to_grad_spat(self._h, ps, _p(a), _p(b), self._lc(lcut))
        return a, b

    def pol_to_grad_spat(self, Slm, lcut=None):
        S, ps = self._c(Slm)
        a, b = self._grid(), self._grid()
        lib().oracle_pol_to_grad_spat(self._h, ps, _p(a), _p(b), self._lc(lcut))
        return a, b

    def torpol_to_spat(self, Wlm, dWlm, Zlm, lcut=None):
        W, pw = self._c(Wlm)
        dW, pdw = self._c(dWlm)
        Z, pz = self._c(Zlm)
        a, b, c = self._grid(), self._grid(), self._grid()
        lib().oracle_torpol_to_spat(self._h, pw, pdw, pz, _p(a), _p(b), _p(c), self._lc(lcut))
        return a, b, c

    def sphtor_to_spat(self, dWlm, Zlm, lcut=None):
        dW, pdw = self._c(dWlm)
        Z, pz = self._c(Zlm)
        a, b = self._grid(), self._grid()
        lib().oracle_sphtor_to_spat(self._h, pdw, pz, _p(a), _p(b), self._lc(lcut))
        return a, b

    def torpol_to_curl_spat_IC(self, r, r_ICB, dBlm, ddBlm, Jlm, dJlm):
        arrs = [self._c(x) for x in (dBlm, ddBlm, Jlm, dJlm)]
        a, b, c = self._grid(), self._grid(), self._grid()
        lib().oracle_torpol_to_curl_spat_IC(self._h, float(r), float(r_ICB),
                                            *[p for _, p in arrs], _p(a), _p(b), _p(c))
        return a, b, c

    def torpol_to_spat_IC(self, r, r_ICB, Wlm, dWlm, Zlm):
        arrs = [self._c(x) for x in (Wlm, dWlm, Zlm)]
        a, b, c = self._grid(), self._grid(), self._grid()
        lib().oracle_torpol_to_spat_IC(self._h, float(r), float(r_ICB),
                                       *[p for _, p in arrs], _p(a), _p(b), _p(c))
        return a, b, c

    def torpol_to_dphspat(self, dWlm, Zlm, lcut=None):
        dW, pdw = self._c(dWlm)
        Z, pz = self._c(Zlm)
        a, b = self._grid(), self._grid()
        lib().oracle_torpol_to_dphspat(self._h, pdw, pz, _p(a), _p(b), self._lc(lcut))
        return a, b

    def pol_to_curlr_spat(self, Qlm, lcut=None):
        Q, pq = self._c(Qlm)
        f = self._grid()
        lib().oracle_pol_to_curlr_spat(self._h, pq, _p(f), self._lc(lcut))
        return f

    def torpol_to_curl_spat(self, or2, Blm, ddBlm, Jlm, dJlm, lcut=None):
        arrs = [self._c(x) for x in (Blm, ddBlm, Jlm, dJlm)]
        a, b, c = self._grid(), self._grid(), self._grid()
        lib().oracle_torpol_to_curl_spat(self._h, float(or2), *[p for _, p in arrs],
                                         _p(a), _p(b), _p(c), self._lc(lcut))
        return a, b, c

    def scal_to_SH(self, f, lcut=None):
        F, pf = self._r(f)
        out = self._spec()
        lib().oracle_scal_to_SH(self._h, pf, out.view(np.float64).ctypes.data_as(_D),
                                self._lc(lcut))
        return out

    def spat_to_qst(self, f, g, h, lcut=None):
        arrs = [self._r(x) for x in (f, g, h)]
        q, s, t = self._spec(), self._spec(), self._spec()
        lib().oracle_spat_to_qst(self._h, *[p for _, p in arrs],
                                 *[x.view(np.float64).ctypes.data_as(_D) for x in (q, s, t)],
                                 self._lc(lcut))
        return q, s, t

    def spat_to_sphertor(self, f, g, lcut=None):
        arrs = [self._r(x) for x in (f, g)]
        a, b = self._spec(), self._spec()
        lib().oracle_spat_to_sphertor(self._h, *[p for _, p in arrs],
                                      *[x.view(np.float64).ctypes.data_as(_D) for x in (a, b)],
                                      self._lc(lcut))
        return a, b

    def axi_to_spat(self, fl_ax):
        F, pf = self._c(fl_ax)
        out = np.zeros(self.n_theta_max)
        lib().oracle_axi_to_spat(self._h, pf, _p(out))
        return out

    def toraxi_to_spat(self, fl_ax, lcut=None):
        F, pf = self._c(fl_ax)
        a = np.zeros(self.n_theta_max)
        b = np.zeros(self.n_theta_max)
        lib().oracle_toraxi_to_spat(self._h, pf, _p(a), _p(b), self._lc(lcut))
        return a, b


def get_nl(grids: dict, or2, n_theta: int) -> dict:
    """Grid-space nonlinear products (get_nl.f90:213-441 with the Lorentz-force
    addition of rIter.f90:650-655), Boussinesq form (orho1 = 1), curl-form
    advection (get_nl.f90:262-272), unit physical constants, heatTerms = the
    ohmic losses (get_nl.f90:424-429).  Grids are [level][phi][theta] with
    scrambled north/south rows (rows 2j, 2j+1 at colatitudes theta_j and
    pi - theta_j); numpy FP64."""
    theta, _ = gauleg(n_theta)                                # colatitudes, north to south
    sn2 = np.repeat(1.0 / np.sin(theta[: n_theta // 2]) ** 2, 2)  # O_sin_theta_E2 per scrambled row
    o2 = np.asarray(or2, dtype=np.float64)[:, None, None]
    o4 = o2 * o2
    g = {k: np.asarray(v, dtype=np.float64)[..., :n_theta] for k, v in grids.items()}
    vr, vt, vp = g["vrc"], g["vtc"], g["vpc"]
    wr, wt, wp = g["cvrc"], g["cvtc"], g["cvpc"]
    br, bt, bp = g["brc"], g["btc"], g["bpc"]
    jr, jt, jp = g["cbrc"], g["cbtc"], g["cbpc"]
    s = g["sc"]
    LFr = sn2 * (jt * bp - jp * bt)
    LFt = o4 * (jp * br - jr * bp)
    LFp = o4 * (jr * bt - jt * br)
    return {
        "Advr": -sn2 * (wt * vp - wp * vt) + LFr,
        "Advt": -o4 * (wp * vr - wr * vp) + LFt,
        "Advp": -o4 * (wr * vt - wt * vr) + LFp,
        "VSr": vr * s,
        "VSt": o2 * vt * s,
        "VSp": o2 * vp * s,
        "VxBr": sn2 * (vt * bp - vp * bt),
        "VxBt": o4 * (vp * br - vr * bp),
        "VxBp": o4 * (vr * bt - vt * br),
        "heatTerms": o2 * (o2 * jr * jr + sn2 * jt * jt + sn2 * jp * jp),
    }


def get_td(spec: dict, r, cor_fac: float, l_max: int, minc: int = 1, lcut=None, epsc=None) -> dict:
    """Spectral assembly of the explicit time derivatives at interior levels
    (get_td.f90: get_dwdt :133-208, get_dpdt :311-379, get_dzdt :381-457,
    get_dsdt :459-521, get_dbdt :558-619), Boussinesq, Coriolis on, no
    double-curl form; operator coefficients of horizontal.f90:204-229.  Arrays
    [level][lm] complex in the m-major st_map order; numpy FP64."""
    ls, ms = [], []
    for m in range(0, l_max + 1, minc):
        for l in range(m, l_max + 1):
            ls.append(l)
            ms.append(m)
    l = np.array(ls, dtype=np.float64)
    m = np.array(ms, dtype=np.float64)
    li = np.array(ls)
    n = len(np.asarray(r))
    K = len(ls)

    def clm(ll, mm):
        return np.sqrt(np.maximum((ll + mm) * (ll - mm), 0.0) / ((2 * ll - 1) * (2 * ll + 1)))

    hasS = li > np.array(ms)                        # lm2lmS valid (l > m)
    cS = np.where(hasS, clm(l, m), 0.0)
    cA = clm(l + 1, m)
    dLh = l * (l + 1)
    t2S, t2A = (l - 1) * cS, (l + 2) * cA
    t3S, t3A = (l - 1) * (l + 1) * cS, l * (l + 2) * cA
    t4S, t4A = (l + 1) * cS * (l - 1) * l, l * cA * (l + 1) * (l + 2)
    idxS = np.where(hasS, np.arange(K) - 1, np.arange(K))
    idxA = np.minimum(np.arange(K) + 1, K - 1)
    out = {k: np.zeros((n, K), dtype=np.complex128) for k in
           ("dwdt", "dzdt", "dpdt", "dsdt", "dbdt", "djdt", "dVxBhLM")}
    for ir in range(n):
        rr = float(np.asarray(r)[ir])
        or1, or2 = 1.0 / rr, 1.0 / rr ** 2
        or4 = or2 * or2
        lR = l_max if lcut is None else min(int(np.asarray(lcut)[ir]), l_max)
        w, dw, z = (np.asarray(spec[k])[ir] for k in ("w", "dw", "z"))
        A = np.where(li < lR, 1.0, 0.0)                # l+1 terms (l < l_R)
        inside = li <= lR
        zA, zS = z[idxA] * A, z[idxS]
        dwA, dwS = dw[idxA] * A, dw[idxS]
        wA, wS = w[idxA] * A, w[idxS]
        dphi = 1j * m
        cor = 2.0 * cor_fac
        # get_dwdt
        c = dphi * dw + t2A * zA - t2S * zS
        c[0] = t2A[0] * zA[0]                            # lm = 1 (l = 0)
        out["dwdt"][ir] = or2 * np.asarray(spec["AdvrLM"])[ir] + np.where(inside, cor * or1 * c, 0)
        # get_dzdt
        c = dphi * z + t3A * dwA + or1 * t4A * wA + t3S * dwS - or1 * t4S * wS
        dz = dLh * np.asarray(spec["AdvpLM"])[ir] + np.where(inside, cor * or2 * c, 0)
        dz[0] = cor * or2 * (t3A[0] * dwA[0] + or1 * t4A[0] * wA[0])
        out["dzdt"][ir] = dz
        # get_dpdt
        c = -dphi * (dw + or1 * dLh * w) + t3A * zA + t3S * zS
        dp = -dLh * np.asarray(spec["AdvtLM"])[ir] + np.where(inside, cor * or2 * c, 0)
        dp[0] = 0.0
        out["dpdt"][ir] = dp
        # get_dsdt (Boussinesq)
        ds = dLh * np.asarray(spec["VStLM"])[ir]
        ds[0] = 0.0 if epsc is None else float(np.asarray(epsc)[ir])
        out["dsdt"][ir] = ds
        # get_dbdt
        out["dbdt"][ir] = dLh * np.asarray(spec["VxBpLM"])[ir]
        out["dVxBhLM"][ir] = -dLh * np.asarray(spec["VxBtLM"])[ir] * rr * rr
        out["djdt"][ir] = dLh * or4 * np.asarray(spec["VxBrLM"])[ir]
    return out
