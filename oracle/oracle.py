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


def courant(grids: dict, radial: dict, n_theta: int, courfac: float, alffac: float, LFfac: float = 1.0,
            opm: float = 1.0, alf_damp: bool = True, dtrkc=None, dthkc=None):
    """Courant steps per level (courant.f90:54-278, the XSH_COURANT == 0
    branch :193-276): maxima over the grid of the radial and horizontal
    velocity terms, fluid plus damped Alfven velocity when ``brc``, ``btc``,
    ``bpc`` are given (:226-252), fluid only otherwise (:256-268); each
    product rounded in the reference's order; a 0/0 term is left out of the
    maximum.  Grids [level][phi][theta] (scrambled rows); numpy FP64."""
    theta, _ = gauleg(n_theta)
    sn2 = np.repeat(1.0 / np.sin(theta[: n_theta // 2]) ** 2, 2)
    g = {k: np.asarray(v, dtype=np.float64)[..., :n_theta] for k, v in grids.items() if v is not None}
    n = g["vrc"].shape[0]
    rf = {k: np.asarray(radial[k], dtype=np.float64) for k in ("orho1", "orho2", "or2", "or4", "delxr2", "delxh2")}
    dtr = np.full(n, 1e10) if dtrkc is None else np.array(dtrkc, dtype=np.float64)
    dth = np.full(n, 1e10) if dthkc is None else np.array(dthkc, dtype=np.float64)
    cf2, af2 = courfac * courfac, alffac * alffac
    mag = "brc" in g
    with np.errstate(invalid="ignore", divide="ignore"):
        for i in range(n):
            vr, vt, vp = g["vrc"][i], g["vtc"][i], g["vpc"][i]
            vflr2 = rf["orho2"][i] * vr * vr
            vflh2 = (vt * vt + vp * vp) * sn2 * rf["orho2"][i]
            if mag:
                if alf_damp:
                    h = 0.5 * (1.0 + opm)
                    valri2, valhi2 = h * h / rf["delxr2"][i], h * h / rf["delxh2"][i]
                else:
                    valri2 = valhi2 = 0.0
                br, bt, bp = g["brc"][i], g["btc"][i], g["bpc"][i]
                valr = br * br * LFfac * rf["orho1"][i]
                valr2 = valr * valr / (valr + valri2)
                vr2 = rf["or4"][i] * (cf2 * vflr2 + af2 * valr2)
                valh2 = (bt * bt + bp * bp) * LFfac * sn2 * rf["orho1"][i]
                valh2m = valh2 * valh2 / (valh2 + valhi2)
                vh2 = rf["or2"][i] * (cf2 * vflh2 + af2 * valh2m)
            else:
                vr2 = cf2 * rf["or4"][i] * vflr2
                vh2 = cf2 * rf["or2"][i] * vflh2
            vr2max = float(np.fmax.reduce(np.fmax(vr2, 0.0), axis=None))
            vh2max = float(np.fmax.reduce(np.fmax(vh2, 0.0), axis=None))
            if vr2max != 0.0:
                dtr[i] = min(dtr[i], np.sqrt(rf["delxr2"][i] / vr2max))
            if vh2max != 0.0:
                dth[i] = min(dth[i], np.sqrt(rf["delxh2"][i] / vh2max))
    return dtr, dth


def _row_trig(n_theta: int):
    """sin and cos of the colatitude of every scrambled row (horizontal.f90:145-159):
    rows 2j, 2j+1 at theta_j and pi - theta_j."""
    theta, _ = gauleg(n_theta)
    s = np.repeat(np.sin(theta[: n_theta // 2]), 2)
    c = np.repeat(np.cos(theta[: n_theta // 2]), 2)
    c[1::2] *= -1.0
    return s, c


def v_rigid_boundary(n_theta: int, n_phi: int, r2_rho0: float, omega: float, keep_vr: bool, vr):
    """v_rigid_boundary (nonlinear_bcs.f90:120-175) for one level: returns
    vr, vt, vp, cvr, dvrdt, dvrdp, dvtdp, dvpdp as (n_phi, n_theta) arrays."""
    s, c = _row_trig(n_theta)
    z = np.zeros((n_phi, n_theta))
    vr_out = np.array(vr, dtype=np.float64)[:, :n_theta] if keep_vr else z.copy()
    vp = np.broadcast_to(r2_rho0 * (s * s) * omega, (n_phi, n_theta)).copy()
    cvr = np.broadcast_to(r2_rho0 * 2.0 * c * omega, (n_phi, n_theta)).copy()
    return {"vr": vr_out, "vt": z.copy(), "vp": vp, "cvr": cvr, "dvrdt": z.copy(), "dvrdp": z.copy(),
            "dvtdp": z.copy(), "dvpdp": z.copy()}


def v_center_sphere(ddw, minc: int, n_theta: int, n_phi: int):
    """v_center_sphere (nonlinear_bcs.f90:177-224): vr, vt, vp (n_phi, n_theta)
    from ddw(l=1, m=0) (st_map index 1) and ddw(l=1, m=1) (index l_max + 1,
    minc = 1); y10_norm, y11_norm of preCalculations.f90:313-314."""
    ddw = np.asarray(ddw)
    s, c = _row_trig(n_theta)
    y10, y11 = 0.5 * np.sqrt(3.0 / np.pi), 0.5 * np.sqrt(1.5 / np.pi)
    d10 = ddw[1].real
    phi = np.arange(n_phi) * (2.0 * np.pi / (n_phi * minc))
    if minc == 1:
        l_max = (np.sqrt(8 * len(ddw) + 1) - 3) / 2  # lm_max = (L+1)(L+2)/2
        d11 = ddw[int(round(l_max)) + 1]
        cp, sp = np.cos(phi)[:, None], np.sin(phi)[:, None]
        cc = d11.real * cp - d11.imag * sp
        vr = y10 * d10 * c + 2.0 * y11 * s * cc
        vt = s * (-y10 * d10 * s + 2.0 * y11 * c * cc)
        vp = -2.0 * y11 * s * (d11.real * sp + d11.imag * cp)
    else:
        vr = np.broadcast_to(y10 * d10 * c, (n_phi, n_theta)).copy()
        vt = np.broadcast_to(-s * y10 * d10 * s, (n_phi, n_theta)).copy()
        vp = np.zeros((n_phi, n_theta))
    return vr, vt, vp


def get_br_v_bcs(sht: "OracleSHT", br, vt, vp, omega: float, or2: float, orho1: float):
    """get_br_v_bcs (nonlinear_bcs.f90:24-69) with the oracle's spat_to_sphertor."""
    n_theta = sht.n_theta_max
    s, _ = _row_trig(n_theta)
    fac = or2 * orho1
    b = np.asarray(br)[:, :n_theta]
    br_vt = fac * b * np.asarray(vt)[:, :n_theta]
    br_vp = b * (fac * np.asarray(vp)[:, :n_theta] - omega * (s * s))
    return sht.spat_to_sphertor(br_vt, br_vp, sht.l_max)


def lorentz_torque(br, bp, n_theta: int, LFfac: float = 1.0, b0: float = 0.0) -> float:
    """get_lorentz_torque (outRot.f90:423-483) of one level's grids
    [phi][theta] (scrambled rows; gauss is stored scrambled too, horizontal.f90:
    180-184): LFfac 2 pi / n_phi_max sum of gauss (br - b0 cos(theta)) bp."""
    _, w = gauleg(n_theta)
    gauss = np.repeat(w[: n_theta // 2], 2)
    _, c = _row_trig(n_theta)
    br = np.asarray(br, dtype=np.float64)[:, :n_theta]
    bp = np.asarray(bp, dtype=np.float64)[:, :n_theta]
    fac = LFfac * 2.0 * np.pi / br.shape[0]
    return float(np.sum(fac * gauss[None, :] * (br - b0 * c[None, :]) * bp))


def get_b_nl_bcs(fac: float, y):
    """get_b_nl_bcs (nonlinear_bcs.f90:71-118): -fac y, 0 at l = m = 0."""
    x = -fac * np.asarray(y, dtype=np.complex128)
    x[0] = 0.0
    return x


def dt_courant(dtrkc, dthkc, dt: float, dtMax: float):
    """New time step from the Courant steps (courant.f90:280-346, without the
    log lines): returns (l_new_dt, dt_new)."""
    dt_fac = 2.0
    dt_r = min([1000.0 * dtMax] + [float(x) for x in dtrkc])
    dt_h = min([1000.0 * dtMax] + [float(x) for x in dthkc])
    dtMin = min(dt_r, dt_h)
    dt_2 = min(0.5 * (1.0 / dt_fac + 1.0) * dtMin, dtMax)
    if dt > dtMax:
        return True, dtMax
    if dt > dtMin:
        return True, dt_2
    if dt_fac * dt < dtMin and dt < dtMax:
        return True, dt_2
    return False, dt


def get_td(spec: dict, r, cor_fac: float, l_max: int, minc: int = 1, lcut=None, epsc=None, nbc=None) -> dict:
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
        if nbc is not None and int(np.asarray(nbc)[ir]) != 0:
            # boundary level: get_dbdt's dVxBhLM only (get_td.f90:598-612); the
            # reference leaves the other outputs unset (NaN here)
            out["dVxBhLM"][ir] = -dLh * np.asarray(spec["VxBtLM"])[ir] * rr * rr
            for k in ("dwdt", "dzdt", "dpdt", "dsdt", "dbdt", "djdt"):
                out[k][ir] = np.nan
            continue
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


def _row_factors(n_theta: int):
    """O_sin_theta_E2 and cosn_theta_E2 on the scrambled rows (2j: colatitude
    theta_j, 2j+1: pi - theta_j), horizontal.f90:145-157."""
    theta, _ = gauleg(n_theta)
    colat = theta[: n_theta // 2]
    sn2 = np.repeat(1.0 / (np.sin(colat) * np.sin(colat)), 2)
    c = np.cos(colat) / np.sin(colat) / np.sin(colat)
    cn2 = np.empty(n_theta)
    cn2[0::2] = c
    cn2[1::2] = -c
    return sn2, cn2


def get_nl_full(grids: dict, n_theta: int, r, l_conv_nl=True, l_adv_curl=True, l_mag_LF=True,
                l_heat_nl=True, l_chemical_conv=False, l_mag_nl=True, l_anel=False, LFfac=1.0,
                ViscHeatFac=1.0, OhmLossFac=1.0, orho1=None, beta=None, otemp1=None, visc=None,
                lam=None, nbc=None, lcr=None) -> dict:
    """Grid-space nonlinear products with the reference's switches and radial
    functions (get_nl.f90:213-441) and the Lorentz-force combination of
    transform_to_lm_space (rIter.f90:645-662), per level:
      Lorentz force LF (:243-256) where l_mag_LF, nBc = 0 and the level is
      outside the low-conductivity region (lcr = 0, nR > n_r_LCR);
      advection, curl form (:260-272) or u.grad u (:274-302), where l_conv_nl
      and nBc = 0; Adv += LF (rIter.f90:648-652) or Adv = LF / 0 without
      l_conv_nl (:653-661);
      V S (:316-320), V Xi (:323-327) where nBc = 0;
      V x B (:376-395): the full product where nBc = 0 outside the region,
      the stress-free form where nBc = 1 or inside it, the rigid form where
      nBc = 2;
      heatTerms (:398-432): viscous heating plus ohmic losses (outside the
      region, with l_mag_nl) where l_anel and nBc = 0.
    Entries a level does not write are NaN (the reference leaves them as they
    were).  Grids [level][phi][theta] in the scrambled row order; numpy FP64."""
    sn2, cn2 = _row_factors(n_theta)
    nl = len(np.asarray(r))
    one = np.ones(nl)
    rr = np.asarray(r, dtype=np.float64)
    prof = {k: (one if v is None else np.asarray(v, dtype=np.float64))
            for k, v in (("orho1", orho1), ("otemp1", otemp1), ("visc", visc), ("lam", lam))}
    bet = np.zeros(nl) if beta is None else np.asarray(beta, dtype=np.float64)
    nb = np.zeros(nl, dtype=int) if nbc is None else np.asarray(nbc)
    lc = np.zeros(nl, dtype=int) if lcr is None else np.asarray(lcr)
    g = {k: np.asarray(v, dtype=np.float64)[..., :n_theta] for k, v in grids.items() if v is not None}
    shape = next(iter(g.values())).shape
    names = ("Advr", "Advt", "Advp", "VSr", "VSt", "VSp", "VXir", "VXit", "VXip", "VxBr", "VxBt", "VxBp",
             "heatTerms")
    out = {k: np.full(shape, np.nan) for k in names}
    two, third = 2.0, 1.0 / 3.0
    for i in range(nl):
        o1 = 1.0 / rr[i]
        o2 = o1 * o1
        o4 = o2 * o2
        oh, bt_, ot, vi, la = prof["orho1"][i], bet[i], prof["otemp1"][i], prof["visc"][i], prof["lam"][i]
        bulk = nb[i] == 0
        x = {k: v[i] for k, v in g.items()}
        LF = None
        if l_mag_LF and bulk and lc[i] == 0:
            LF = (LFfac * sn2 * (x["cbtc"] * x["bpc"] - x["cbpc"] * x["btc"]),
                  LFfac * o4 * (x["cbpc"] * x["brc"] - x["cbrc"] * x["bpc"]),
                  LFfac * o4 * (x["cbrc"] * x["btc"] - x["cbtc"] * x["brc"]))
        adv = None
        if l_conv_nl and bulk:
            vr, vt, vp = x["vrc"], x["vtc"], x["vpc"]
            if l_adv_curl:
                adv = [-sn2 * (x["cvtc"] * vp - x["cvpc"] * vt),
                       -o4 * (x["cvpc"] * vr - x["cvrc"] * vp),
                       -o4 * (x["cvrc"] * vt - x["cvtc"] * vr)]
            else:
                adv = [-o2 * oh * (vr * (x["dvrdrc"] - (two * o1 + bt_) * vr) +
                                   sn2 * (vt * (x["dvrdtc"] - rr[i] * vt) + vp * (x["dvrdpc"] - rr[i] * vp))),
                       o4 * oh * (-vr * (x["dvtdrc"] - bt_ * vt) +
                                  vt * (cn2 * vt + x["dvpdpc"] + x["dvrdrc"]) +
                                  vp * (cn2 * vp - x["dvtdpc"])),
                       o4 * oh * (-vr * (x["dvpdrc"] - bt_ * vp) - vt * (x["dvtdpc"] + x["cvrc"]) -
                                  vp * x["dvpdpc"])]
        # transform_to_lm_space (rIter.f90:645-662)
        if bulk and (l_conv_nl or l_mag_LF):
            if l_conv_nl and l_mag_LF:
                if lc[i] == 0:
                    adv = [a + b for a, b in zip(adv, LF)]
            elif l_mag_LF:
                adv = list(LF) if lc[i] == 0 else [np.zeros(shape[1:])] * 3
            for k, v in zip(("Advr", "Advt", "Advp"), adv):
                out[k][i] = v
        if l_heat_nl and bulk:
            out["VSr"][i] = x["vrc"] * x["sc"]
            out["VSt"][i] = o2 * x["vtc"] * x["sc"]
            out["VSp"][i] = o2 * x["vpc"] * x["sc"]
        if l_chemical_conv and bulk:
            out["VXir"][i] = x["vrc"] * x["xic"]
            out["VXit"][i] = o2 * x["vtc"] * x["xic"]
            out["VXip"][i] = o2 * x["vpc"] * x["xic"]
        if l_mag_nl:
            if bulk and lc[i] == 0:
                out["VxBr"][i] = oh * sn2 * (x["vtc"] * x["bpc"] - x["vpc"] * x["btc"])
                out["VxBt"][i] = oh * o4 * (x["vpc"] * x["brc"] - x["vrc"] * x["bpc"])
                out["VxBp"][i] = oh * o4 * (x["vrc"] * x["btc"] - x["vtc"] * x["brc"])
            elif nb[i] == 1 or lc[i] != 0:
                out["VxBt"][i] = o4 * oh * x["vpc"] * x["brc"]
                out["VxBp"][i] = -o4 * oh * x["vtc"] * x["brc"]
            elif nb[i] == 2:
                out["VxBt"][i] = o4 * oh * x["vpc"] * x["brc"]
                out["VxBp"][i] = 0.0
        if l_anel and bulk:
            vr, vt, vp = x["vrc"], x["vtc"], x["vpc"]
            h = ViscHeatFac * o4 * oh * ot * vi * (
                two * (x["dvrdrc"] - (two * o1 + bt_) * vr) ** 2 +
                two * (cn2 * vt + x["dvpdpc"] + x["dvrdrc"] - o1 * vr) ** 2 +
                two * (x["dvpdpc"] + cn2 * vt + o1 * vr) ** 2 +
                (two * x["dvtdpc"] + x["cvrc"] - two * cn2 * vp) ** 2 +
                sn2 * ((rr[i] * x["dvtdrc"] - (two + bt_ * rr[i]) * vt + o1 * x["dvrdtc"]) ** 2 +
                       (rr[i] * x["dvpdrc"] - (two + bt_ * rr[i]) * vp + o1 * x["dvrdpc"]) ** 2) -
                two * third * (bt_ * vr) ** 2)
            if l_mag_nl and lc[i] == 0:
                h = h + OhmLossFac * o2 * ot * la * (o2 * x["cbrc"] ** 2 + sn2 * x["cbtc"] ** 2 +
                                                     sn2 * x["cbpc"] ** 2)
            out["heatTerms"][i] = h
    return out


def get_td_full(spec: dict, r, cor_fac: float, l_max: int, minc: int = 1, lcut=None, nbc=None,
                l_conv_nl=True, l_corr=True, l_double_curl=False, l_single_matrix=False, l_anel=False,
                l_anelastic_liquid=False, l_mag_nl=True, orho1=None, beta=None, temp0=None, epsc=None,
                epscXi=0.0, outputs=("dwdt", "dzdt", "dpdt", "dsdt", "dxidt", "dbdt", "djdt", "dVxBhLM",
                                     "dVxVhLM", "dVSrLM", "dVXirLM")) -> dict:
    """The spectral assembly of get_td.f90 with the reference's switches, per
    level (the calls of rIter.f90:410-428; an output is computed when it is
    in ``outputs``, standing for the equation being on):
      get_dwdt (:133-208) or get_dwdt_double_curl (:210-309, with dVxVhLM),
      get_dpdt (:311-379), get_dzdt (:381-457), get_dsdt (:459-521, with the
      anelastic heatTermsLM and temp0), get_dxidt (:523-556), get_dbdt
      (:558-619; l_mag_nl False: zeros).
    Entries the reference does not set at a level are NaN.  Arrays
    [level][lm] complex in the m-major st_map order; numpy FP64."""
    ls, ms = [], []
    for m in range(0, l_max + 1, minc):
        for l in range(m, l_max + 1):
            ls.append(l)
            ms.append(m)
    l = np.array(ls, dtype=np.float64)
    m = np.array(ms, dtype=np.float64)
    li = np.array(ls)
    rr_all = np.asarray(r, dtype=np.float64)
    n = rr_all.size
    K = len(ls)

    def clm(ll, mm):
        return np.sqrt(np.maximum((ll + mm) * (ll - mm), 0.0) / ((2 * ll - 1) * (2 * ll + 1)))

    hasS = li > np.array(ms)
    cS = np.where(hasS, clm(l, m), 0.0)
    cA = clm(l + 1, m)
    dLh = l * (l + 1)
    t2S, t2A = (l - 1) * cS, (l + 2) * cA
    t3S, t3A = (l - 1) * (l + 1) * cS, l * (l + 2) * cA
    t4S, t4A = (l + 1) * cS * (l - 1) * l, l * cA * (l + 1) * (l + 2)
    idxS = np.where(hasS, np.arange(K) - 1, np.arange(K))
    idxA = np.minimum(np.arange(K) + 1, K - 1)
    one = np.ones(n)
    oh_all = one if orho1 is None else np.asarray(orho1, dtype=np.float64)
    be_all = np.zeros(n) if beta is None else np.asarray(beta, dtype=np.float64)
    t0_all = one if temp0 is None else np.asarray(temp0, dtype=np.float64)
    ep_all = np.zeros(n) if epsc is None else np.asarray(epsc, dtype=np.float64)
    nb_all = np.zeros(n, dtype=int) if nbc is None else np.asarray(nbc)
    out = {k: np.full((n, K), np.nan + 0j, dtype=np.complex128) for k in outputs}
    S = {k: (None if spec.get(k) is None else np.asarray(spec[k])) for k in
         ("w", "dw", "ddw", "z", "dz", "AdvrLM", "AdvtLM", "AdvpLM", "VStLM", "heatTermsLM", "VXitLM",
          "VxBrLM", "VxBtLM", "VxBpLM")}
    cor = 2.0 * cor_fac
    dphi = 1j * m
    for ir in range(n):
        rr = rr_all[ir]
        or1, or2 = 1.0 / rr, 1.0 / rr ** 2
        or4 = or2 * or2
        oh, be = oh_all[ir], be_all[ir]
        bulk = int(nb_all[ir]) == 0
        lR = l_max if lcut is None else min(int(np.asarray(lcut)[ir]), l_max)
        A = np.where(li < lR, 1.0, 0.0)
        inside = li <= lR
        lv = {k: (None if v is None else v[ir]) for k, v in S.items()}

        def nb(x):
            return x[idxA] * A, x[idxS]
        if bulk:
            w, dw, z = lv["w"], lv["dw"], lv["z"]
            zA, zS = nb(z)
            dwA, dwS = nb(dw)
            wA, wS = nb(w)
            if "dzdt" in out:
                dz_ = (dLh * lv["AdvpLM"]) if l_conv_nl else np.zeros(K, complex)
                if l_corr:
                    c = dphi * z + t3A * dwA + or1 * t4A * wA + t3S * dwS - or1 * t4S * wS
                    dz_ = dz_ + np.where(inside, cor * or2 * c, 0)
                # lm = 1 (get_td.f90:401-409)
                dz_[0] = cor * or2 * (t3A[0] * dw[idxA[0]] + or1 * t4A[0] * w[idxA[0]]) if l_corr else 0.0
                out["dzdt"][ir] = dz_
            if "dwdt" in out:
                d0 = or2 * lv["AdvrLM"][0] if l_conv_nl else 0.0
                if l_corr and not l_single_matrix:
                    d0 = d0 + cor * or1 * t2A[0] * z[idxA[0]]
                if not l_double_curl:
                    dw_ = (or2 * lv["AdvrLM"]) if l_conv_nl else np.zeros(K, complex)
                    if l_corr:
                        c = dphi * dw + t2A * zA - t2S * zS
                        dw_ = dw_ + np.where(inside, cor * or1 * c, 0)
                else:
                    ddw, dzz = lv["ddw"], lv["dz"]
                    dzA, dzS = nb(dzz)
                    if l_conv_nl:
                        dw_ = dLh * or4 * oh * lv["AdvrLM"]
                        vh = -oh * rr * rr * dLh * lv["AdvtLM"]
                    else:
                        dw_ = np.zeros(K, complex)
                        vh = np.zeros(K, complex)
                    if l_corr:
                        c = (dphi * (-ddw + be * dw + (be * or1 + or2) * dLh * w) +
                             t3A * (dzA - be * zA) + t3S * (dzS - be * zS) + or1 * (t4A * zA - t4S * zS))
                        dw_ = dw_ + np.where(inside, cor * or2 * oh * c, 0)
                    if "dVxVhLM" in out:
                        vh = vh.copy()
                        vh[0] = out["dVxVhLM"][ir][0]  # lm = 1 left as it was
                        out["dVxVhLM"][ir] = vh
                dw_ = dw_.copy()
                dw_[0] = d0
                out["dwdt"][ir] = dw_
            if "dpdt" in out:
                dp = (-dLh * lv["AdvtLM"]) if l_conv_nl else np.zeros(K, complex)
                if l_corr:
                    c = -dphi * (dw + or1 * dLh * w) + t3A * zA + t3S * zS
                    dp = dp + np.where(inside, cor * or2 * c, 0)
                dp = dp.copy()
                dp[0] = np.nan  # get_dpdt leaves lm = 1
                out["dpdt"][ir] = dp
            if "dsdt" in out:
                ds = dLh * lv["VStLM"]
                if l_anel:
                    ds = ds + (t0_all[ir] if l_anelastic_liquid else 1.0) * lv["heatTermsLM"]
                ds = ds.copy()
                ds[0] = ep_all[ir] + ((t0_all[ir] if l_anelastic_liquid else 1.0) * lv["heatTermsLM"][0]
                                      if l_anel else 0.0)
                out["dsdt"][ir] = ds
            if "dxidt" in out:
                dx = dLh * lv["VXitLM"]
                dx = dx.copy()
                dx[0] = epscXi
                out["dxidt"][ir] = dx
            if l_mag_nl:
                for k, v in (("dbdt", dLh * lv["VxBpLM"]), ("dVxBhLM", -dLh * lv["VxBtLM"] * rr * rr),
                             ("djdt", dLh * or4 * lv["VxBrLM"])):
                    if k in out:
                        out[k][ir] = v
            else:
                for k in ("dbdt", "djdt", "dVxBhLM"):
                    if k in out:
                        out[k][ir] = 0.0
        else:
            if l_double_curl and "dVxVhLM" in out:
                out["dVxVhLM"][ir] = 0.0
            if "dsdt" in out and "dVSrLM" in out:
                out["dVSrLM"][ir] = 0.0
            if "dxidt" in out and "dVXirLM" in out:
                out["dVXirLM"][ir] = 0.0
            if "dVxBhLM" in out:
                if l_mag_nl:
                    v = -dLh * lv["VxBtLM"] * rr * rr
                    v[0] = 0.0
                    out["dVxBhLM"][ir] = v
                else:
                    out["dVxBhLM"][ir] = 0.0
    return out
