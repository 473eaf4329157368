"""The radial loop's explicit stage on the device, over all radial levels.

``RadialLoop.step`` runs what ``radialLoop`` (src/rIter.f90:94-464) does for
every level nR of a spherical shell, batched over the levels instead of one
level at a time: the synthesis set (transform_to_grid_space), the boundary
overrides of the two boundary levels (rIter.f90:548-597 with
v_rigid_boundary, nonlinear_bcs.f90:120-175), the grid-space products
(get_nl, interior levels, and the boundaries when lMagNlBc), the Courant
steps (courant.f90:54-278), the analysis set (transform_to_lm_space), the
conducting-boundary products (get_br_v_bcs, rIter.f90:263-277) and the
spectral assembly (get_td with the boundary flags nBc).

Configuration of the device kernels: Boussinesq (rho0 = 1), curl-form
advection, magnetic field with Lorentz force, heat equation, Coriolis force,
unit physical constants in get_nl.  Level 0 is the outer boundary (n_r_cmb,
nBc = ktopv), level n-1 the inner boundary (n_r_icb, nBc = kbotv), as in
MagIC's radial ordering.  Every array is a CUDA tensor ([level][lm] complex
spectra, [level][phi][theta] grids) and the stage runs on the current torch
stream; the per-level arrays (radii, or2, lcut, nBc, the Courant radial
functions) live on the device, so no call of the stage waits for the
stream, and the Courant steps come back to the host (numpy) at the end, as
dt_courant (courant.f90:280-346) needs them there: the stage's one
synchronisation.
The two boundary levels run the bulk synthesis set and are then overwritten
(vrc = 0 at a stress-free boundary, v_rigid_boundary at a rigid one); the
grids the reference does not compute there are not read afterwards.
"""
from __future__ import annotations

from typing import Dict, Optional

import numpy as np

from . import _lib
from .sht import SHT


def delx2(r, lcut) -> tuple:
    """Courant grid intervals of preCalculations.f90:303-310: delxr2 (squared
    smallest neighbouring radial spacing) and delxh2 = r^2 / (l_R (l_R + 1))."""
    r = np.asarray(r, dtype=np.float64)
    lc = np.asarray(lcut, dtype=np.float64)
    delxh2 = r ** 2 / (lc * (lc + 1.0))
    n = len(r)
    delxr2 = np.empty(n)
    delxr2[0] = (r[0] - r[1]) ** 2
    delxr2[n - 1] = (r[n - 2] - r[n - 1]) ** 2
    for i in range(1, n - 1):
        d = min(r[i - 1] - r[i], r[i] - r[i + 1])
        delxr2[i] = d * d
    return delxr2, delxh2


class RadialLoop:
    """One explicit stage of the radial loop over levels r[0] (outer) .. r[n-1]
    (inner) with the handle ``sht`` (any precision form).

    Boundary kinds (ktopv, kbotv): 1 stress-free, 2 rigid (rotating at
    omega_ma / omega_ic).  l_vr_cmb / l_vr_icb keep the radial velocity at a
    rigid boundary (special.f90).  The conducting-mantle / inner-core terms
    (get_br_v_bcs) run when l_b_nl_cmb / l_b_nl_icb hold (Namelists.f90:713-729:
    stress-free and conducting)."""

    def __init__(self, sht: SHT, r, cor_fac: float, courfac: float = 2.5, alffac: float = 1.0,
                 LFfac: float = 1.0, opm: float = 1.0, l_cour_alf_damp: bool = True, lcut=None, epsc=None,
                 ktopv: int = 2, kbotv: int = 2, l_vr_cmb: bool = False, l_vr_icb: bool = False,
                 omega_ma: float = 0.0, omega_ic: float = 0.0, l_rot_ma: bool = False, l_rot_ic: bool = False,
                 l_cond_ma: bool = False, l_cond_ic: bool = False):
        if ktopv not in (1, 2) or kbotv not in (1, 2):
            raise ValueError("ktopv and kbotv are 1 (stress-free) or 2 (rigid)")
        self.s = sht
        self.r = np.ascontiguousarray(r, dtype=np.float64)
        self.n = n = len(self.r)
        if n < 3:
            raise ValueError("the radial loop needs two boundary levels and at least one interior level")
        self.lcut = None if lcut is None else np.ascontiguousarray(lcut, dtype=np.int32)
        self.epsc = epsc
        self.cor_fac = float(cor_fac)
        self.courfac, self.alffac, self.LFfac, self.opm = float(courfac), float(alffac), float(LFfac), float(opm)
        self.l_cour_alf_damp = bool(l_cour_alf_damp)
        self.ktopv, self.kbotv = ktopv, kbotv
        self.l_vr_cmb, self.l_vr_icb = bool(l_vr_cmb), bool(l_vr_icb)
        self.omega_ma, self.omega_ic = float(omega_ma), float(omega_ic)
        self.or2 = 1.0 / self.r ** 2
        lc = np.full(n, sht.l_max) if self.lcut is None else self.lcut
        delxr2, delxh2 = delx2(self.r, lc)
        self.radial = {"orho1": np.ones(n), "orho2": np.ones(n), "or2": self.or2, "or4": self.or2 ** 2,
                       "delxr2": delxr2, "delxh2": delxh2}
        # rIter.f90:180-187 (Fortran precedence: .and. before .or.)
        self.lMagNlBc = ((ktopv == 1 or l_cond_ma or (ktopv == 2 and l_rot_ma))
                         or (kbotv == 1 or l_cond_ic or (kbotv == 2 and l_rot_ic)))
        self.l_b_nl_cmb = ktopv == 1 and l_cond_ma
        self.l_b_nl_icb = kbotv == 1 and l_cond_ic
        self.nbc = np.zeros(n, dtype=np.int32)
        self.nbc[0], self.nbc[n - 1] = ktopv, kbotv
        self._dev = {}

    def _on(self, device):
        """The per-level arrays as CUDA tensors on `device` (made once): every
        call of the stage then takes device pointers, so none of them waits
        for the stream."""
        if device not in self._dev:
            import torch
            f = lambda x: torch.as_tensor(np.ascontiguousarray(x), device=device)  # noqa: E731
            d = {"or2": f(self.or2), "r": f(self.r), "nbc": f(self.nbc),
                 "lcut": None if self.lcut is None else f(self.lcut),
                 "epsc": None if self.epsc is None else f(np.asarray(self.epsc, dtype=np.float64)),
                 "radial": {k: f(v) for k, v in self.radial.items()}}
            self._dev[device] = d
        return self._dev[device]

    def _boundary_grids(self, g: Dict, i: int, kind: int, omega: float, keep_vr: bool):
        if kind == 1:  # stress-free: vrc = 0 (rIter.f90:552-556)
            g["vrc"][i].zero_()
        else:          # rigid (rIter.f90:570-592, lDeriv off: cvr untouched)
            self.s.v_rigid_boundary({"vr": g["vrc"][i], "vt": g["vtc"][i], "vp": g["vpc"][i]},
                                    self.r[i] ** 2, omega, keep_vr)

    def step(self, spec: Dict, out: Optional[Dict] = None) -> Dict:
        """One stage from the spectra of transform_to_grid_space (``s``, ``p``,
        ``xi``, ``w`` .. ``dj``; [level][lm] complex CUDA tensors).  Returns
        the get_td outputs (``dwdt`` .. ``dVxBhLM``), ``VSrLM`` (dVSrLM, 0 at
        the boundaries), numpy ``dtrkc`` / ``dthkc``, and at conducting
        boundaries ``br_vt_lm_cmb`` / ``br_vp_lm_cmb`` (or ``_icb``)."""
        import torch
        s, n = self.s, self.n
        dv = self._on(spec["w"].device)
        g = s.transform_to_grid_space(spec, or2=dv["or2"], lcut=dv["lcut"])
        self._boundary_grids(g, 0, self.ktopv, self.omega_ma, self.l_vr_cmb)
        self._boundary_grids(g, n - 1, self.kbotv, self.omega_ic, self.l_vr_icb)
        lo, hi = (0, n) if self.lMagNlBc else (1, n - 1)
        gs = {k: v[lo:hi] for k, v in g.items()}
        nl = s.get_nl(gs, or2=dv["or2"][lo:hi])
        lc = None if dv["lcut"] is None else dv["lcut"][lo:hi]
        # analysis outputs at all levels, written in place into rows lo..hi-1;
        # boundary levels without lMagNlBc have zero VxBt / VxBp
        # (rIter.f90:256-259) and every level's dVSrLM is zero at the
        # boundaries (get_td.f90:501-507)
        dev = g["vrc"].device
        full = {k: torch.empty((n, s.lm_max), dtype=torch.complex128, device=dev) for k in _lib.LM_SPACE_OUT}
        s.transform_to_lm_space(nl, lcut=lc, out={k: v[lo:hi] for k, v in full.items()})
        for k, v in full.items():
            if lo > 0:
                v[:lo].zero_()
            if hi < n:
                v[hi:].zero_()
        full["VSrLM"][0].zero_()
        full["VSrLM"][n - 1].zero_()
        res = dict(out or {})
        dtrkc, dthkc = s.courant({k: g[k] for k in ("vrc", "vtc", "vpc", "brc", "btc", "bpc")}, dv["radial"],
                                 self.courfac, self.alffac, self.LFfac, self.opm, self.l_cour_alf_damp,
                                 dtrkc=torch.full((n,), 1e10, dtype=torch.float64, device=dev),
                                 dthkc=torch.full((n,), 1e10, dtype=torch.float64, device=dev))
        if self.l_b_nl_cmb:
            res["br_vt_lm_cmb"], res["br_vp_lm_cmb"] = s.get_br_v_bcs(g["brc"][0], g["vtc"][0], g["vpc"][0],
                                                                      self.omega_ma, self.or2[0], 1.0)
        if self.l_b_nl_icb:
            res["br_vt_lm_icb"], res["br_vp_lm_icb"] = s.get_br_v_bcs(g["brc"][n - 1], g["vtc"][n - 1],
                                                                      g["vpc"][n - 1], self.omega_ic,
                                                                      self.or2[n - 1], 1.0)
        tdin = {k: spec[k] for k in ("w", "dw", "z")}
        tdin.update({k: full[k] for k in ("AdvrLM", "AdvtLM", "AdvpLM", "VStLM", "VxBrLM", "VxBtLM", "VxBpLM")})
        td = s.get_td(tdin, dv["r"], self.cor_fac, lcut=dv["lcut"], epsc=dv["epsc"], nbc=dv["nbc"],
                      out={k: res[k] for k in _lib.TD_OUT if k in res} or None)
        res.update(td)
        res["VSrLM"] = full["VSrLM"]
        # the stage's one synchronisation: dt_courant wants the steps on the host
        res["dtrkc"], res["dthkc"] = dtrkc.cpu().numpy(), dthkc.cpu().numpy()
        res["grids"] = g
        return res
