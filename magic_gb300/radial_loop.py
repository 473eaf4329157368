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

Configuration of the device kernels: by default Boussinesq (rho0 = 1),
curl-form advection, magnetic field with Lorentz force, heat equation,
Coriolis force, unit physical constants in get_nl (magic_sht_get_nl /
magic_sht_get_td); with ``physics`` the reference's switches, constants and
radial profiles through the general routines (magic_sht_get_nl_opts /
magic_sht_get_td_opts): density and temperature profiles, composition,
double-curl dwdt, the anelastic-liquid dsdt, the physical constants.  Level 0 is the outer boundary (n_r_cmb,
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
    stress-free and conducting).

    ``physics`` (optional) selects the general get_nl / get_td: the
    keyword arguments of SHT.get_nl_opts (``ViscHeatFac``, ``OhmLossFac``,
    the profiles ``orho1``, ``beta``, ``otemp1``, ``visc``, ``lam``, the
    low-conductivity flags ``lcr``, and the switches ``l_conv_nl``,
    ``l_adv_curl``, ``l_mag_LF``, ``l_heat_nl``, ``l_chemical_conv``,
    ``l_mag_nl``, ``l_anel``; the u.grad u form and the viscous heating
    take the velocity-derivative grids of the synthesis set,
    rIter.f90:527-545) and of SHT.get_td_opts (``temp0``, ``epscXi``, ``l_corr``,
    ``l_double_curl``, ``l_single_matrix``, ``l_anelastic_liquid``);
    profiles are per level (numpy).  LFfac is the loop's own.  The Courant
    condition then takes orho1 and orho2 = orho1^2 from the profile."""

    def __init__(self, sht: SHT, r, cor_fac: float, courfac: float = 2.5, alffac: float = 1.0,
                 LFfac: float = 1.0, opm: float = 1.0, l_cour_alf_damp: bool = True, lcut=None, epsc=None,
                 ktopv: int = 2, kbotv: int = 2, l_vr_cmb: bool = False, l_vr_icb: bool = False,
                 omega_ma: float = 0.0, omega_ic: float = 0.0, l_rot_ma: bool = False, l_rot_ic: bool = False,
                 l_cond_ma: bool = False, l_cond_ic: bool = False, BIC: float = 0.0,
                 physics: Optional[dict] = None):
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
        self.physics = self._physics(physics)
        orho1 = np.ones(n) if self.physics is None or self.physics["profiles"].get("orho1") is None \
            else self.physics["profiles"]["orho1"]
        self.radial = {"orho1": orho1, "orho2": orho1 ** 2, "or2": self.or2, "or4": self.or2 ** 2,
                       "delxr2": delxr2, "delxh2": delxh2}
        # rIter.f90:180-187 (Fortran precedence: .and. before .or.)
        self.lMagNlBc = ((ktopv == 1 or l_cond_ma or (ktopv == 2 and l_rot_ma))
                         or (kbotv == 1 or l_cond_ic or (kbotv == 2 and l_rot_ic)))
        self.l_b_nl_cmb = ktopv == 1 and l_cond_ma
        self.l_b_nl_icb = kbotv == 1 and l_cond_ic
        # Lorentz torques on a rotating, conducting mantle / inner core
        # (rIter.f90:278-292; the Lorentz force is on); b0 of the Grenoble
        # setup's imposed dipole (outRot.f90:466-472), 0 without it
        self.torque_ma = bool(l_rot_ma and l_cond_ma)
        self.torque_ic = bool(l_rot_ic and l_cond_ic)
        r_icb, r_cmb = float(self.r[-1]), float(self.r[0])
        self.b0_ic = 2.0 * BIC * r_icb ** 2
        self.b0_ma = 2.0 * BIC * r_icb ** 2 * (r_icb / r_cmb)
        self.nbc = np.zeros(n, dtype=np.int32)
        self.nbc[0], self.nbc[n - 1] = ktopv, kbotv
        self._dev = {}

    NL_FLAGS = ("l_conv_nl", "l_adv_curl", "l_mag_LF", "l_heat_nl", "l_chemical_conv", "l_mag_nl", "l_anel")
    NL_CONST = ("ViscHeatFac", "OhmLossFac")
    TD_FLAGS = ("l_corr", "l_double_curl", "l_single_matrix", "l_anelastic_liquid")
    PROFILES = ("orho1", "beta", "otemp1", "visc", "lam", "temp0")

    def _physics(self, physics: Optional[dict]):
        """The general routines' arguments, split into switches, constants and
        per-level profiles (or None for the default configuration)."""
        if physics is None:
            return None
        p = dict(physics)
        known = set(self.NL_FLAGS + self.NL_CONST + self.TD_FLAGS + self.PROFILES + ("lcr", "epscXi"))
        unknown = set(p) - known
        if unknown:
            raise ValueError("unknown physics keys: %s" % sorted(unknown))
        flags = {k: bool(p.get(k, d)) for k, d in (("l_conv_nl", True), ("l_adv_curl", True),
                                                  ("l_mag_LF", True), ("l_heat_nl", True),
                                                  ("l_chemical_conv", False), ("l_mag_nl", True), ("l_anel", False),
                                                  ("l_corr", True), ("l_double_curl", False),
                                                  ("l_single_matrix", False), ("l_anelastic_liquid", False))}
        prof = {}
        for k in self.PROFILES:
            if p.get(k) is not None:
                a = np.ascontiguousarray(p[k], dtype=np.float64)
                if a.shape != (self.n,):
                    raise ValueError("%s needs %d levels" % (k, self.n))
                prof[k] = a
        lcr = None if p.get("lcr") is None else np.ascontiguousarray(p["lcr"], dtype=np.int32)
        return {"flags": flags, "const": {k: float(p[k]) for k in self.NL_CONST if k in p},
                "epscXi": float(p.get("epscXi", 0.0)), "profiles": prof, "lcr": lcr}

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
            if self.physics is not None:
                d["profiles"] = {k: f(v) for k, v in self.physics["profiles"].items()}
                d["lcr"] = None if self.physics["lcr"] is None else f(self.physics["lcr"])
            self._dev[device] = d
        return self._dev[device]

    def _boundary_grids(self, g: Dict, i: int, kind: int, omega: float, keep_vr: bool):
        if kind == 1:  # stress-free: vrc = 0 (rIter.f90:552-556)
            g["vrc"][i].zero_()
        else:          # rigid (rIter.f90:570-592, lDeriv off: cvr untouched)
            self.s.v_rigid_boundary({"vr": g["vrc"][i], "vt": g["vtc"][i], "vp": g["vpc"][i]},
                                    self.r[i] ** 2 / self.radial["orho1"][i], omega, keep_vr)

    def _lohi(self):
        return (0, self.n) if self.lMagNlBc else (1, self.n - 1)

    def _alloc(self, spec: Dict, out: Optional[Dict] = None) -> Dict:
        """Every output of one stage: the synthesis grids, the analysis inputs
        of the get_nl levels, the analysis outputs, the get_td outputs (from
        ``out`` where given), the Courant steps and the conducting-boundary
        spectra."""
        import torch
        s, n = self.s, self.n
        dev = spec["w"].device
        f64 = dict(dtype=torch.float64, device=dev)
        c128 = dict(dtype=torch.complex128, device=dev)
        src = {"sc": "s", "pc": "p", "xic": "xi", "vrc": "w", "vtc": "w", "vpc": "w", "cvrc": "ddw", "cvtc": "ddw",
               "cvpc": "ddw", "brc": "b", "btc": "b", "bpc": "b", "cbrc": "ddb", "cbtc": "ddb", "cbpc": "ddb"}
        grids = {k: torch.empty((n, s.n_phi_max, s.nlat_padded), **f64) for k in _lib.GRID_SPACE_OUT
                 if spec.get(src[k]) is not None}
        grid_out = dict(grids)
        if self._derivatives():
            # the u.grad u advection and the viscous heating (rIter.f90:527-545);
            # the u.grad u form takes cvrc alone (pol_to_curlr_spat(z), :540)
            for k in _lib.GRID_SPACE_OUT_DV:
                grids[k] = grid_out[k] = torch.empty((n, s.n_phi_max, s.nlat_padded), **f64)
            if not self.physics["flags"]["l_adv_curl"]:
                for k in ("cvtc", "cvpc"):
                    grids.pop(k, None)
                    grid_out[k] = None
        lo, hi = self._lohi()
        out = out or {}
        if self.physics is None:
            nl_names, lm_names, td_names = _lib.LM_SPACE_IN, _lib.LM_SPACE_OUT, _lib.TD_OUT
            nl_alloc = torch.empty
        else:
            # the general get_nl / get_td leave what a level does not form
            # untouched (get_dpdt the l = 0 entry, get_td.f90:311-379):
            # zero-filled once, those entries stay zero
            xi = self.physics["flags"]["l_chemical_conv"]
            nl_names = [k for k in _lib.NLF_OUT if xi or not k.startswith("VXi")]
            lm_names = _lib.LM_SPACE_OUT + (_lib.LM_SPACE_OUT_XI if xi else [])
            td_names = self._td_outputs()
            nl_alloc = torch.zeros
        b = {"device": dev, "grids": grids, "grid_out": grid_out,
             "nl": {k: nl_alloc((hi - lo, s.n_phi_max, s.nlat_padded), **f64) for k in nl_names},
             "lm": {k: torch.empty((n, s.lm_max), **c128) for k in lm_names},
             "td": {k: out[k] if k in out else nl_alloc((n, s.lm_max), **c128) for k in td_names},
             "dtrkc": torch.empty(n, **f64), "dthkc": torch.empty(n, **f64)}
        for flag, key in ((self.l_b_nl_cmb, "cmb"), (self.l_b_nl_icb, "icb")):
            if flag:
                b[key] = (torch.empty(s.lm_max, **c128), torch.empty(s.lm_max, **c128))
        if self._rigid_kept_vr():
            b["zero_grid"] = torch.zeros((1, s.n_phi_max, s.nlat_padded), **f64)
        for flag, key in ((self.torque_ma, "torque_ma"), (self.torque_ic, "torque_ic")):
            if flag:
                b[key] = torch.empty(1, **f64)
        return b

    def _derivatives(self):
        """Whether the stage needs the velocity-derivative grids (the u.grad u
        advection or the anelastic viscous heating)."""
        if self.physics is None:
            return False
        fl = self.physics["flags"]
        return (fl["l_conv_nl"] and not fl["l_adv_curl"]) or fl["l_anel"]

    def _td_outputs(self):
        """The outputs of the general get_td the switches call for
        (rIter.f90:410-428: get_dwdt, get_dsdt, get_dxidt, get_dbdt)."""
        fl = self.physics["flags"]
        names = []
        if fl["l_conv_nl"] or fl["l_corr"]:
            names += ["dwdt", "dzdt"] + (["dVxVhLM"] if fl["l_double_curl"] else ["dpdt"])
        if fl["l_heat_nl"]:
            names += ["dsdt", "dVSrLM"]
        if fl["l_chemical_conv"]:
            names += ["dxidt", "dVXirLM"]
        if fl["l_mag_nl"]:
            names += ["dbdt", "djdt", "dVxBhLM"]
        return names

    def _rigid_kept_vr(self):
        """Boundary levels whose products get_nl forms at all (lMagNlBc) and
        whose grid keeps a radial velocity at a rigid boundary (l_vr_cmb /
        l_vr_icb)."""
        if not self.lMagNlBc:
            return []
        return [i for i, kind, keep in ((0, self.ktopv, self.l_vr_cmb), (self.n - 1, self.kbotv, self.l_vr_icb))
                if kind == 2 and keep]

    def _enqueue(self, spec: Dict, b: Dict):
        """Launch one stage into the buffers ``b`` on the current stream: no
        allocation and no synchronisation (so it can be captured)."""
        s, n = self.s, self.n
        dv = self._on(b["device"])
        g = s.transform_to_grid_space(spec, or2=dv["or2"], lcut=dv["lcut"], out=b["grid_out"])
        self._boundary_grids(g, 0, self.ktopv, self.omega_ma, self.l_vr_cmb)
        self._boundary_grids(g, n - 1, self.kbotv, self.omega_ic, self.l_vr_icb)
        lo, hi = self._lohi()
        if self.physics is not None:
            self._nl_td_general(spec, b, g, dv, lo, hi)
            self._boundary_outputs(b, g, dv)
            return
        nl = s.get_nl({k: v[lo:hi] for k, v in g.items()}, or2=dv["or2"][lo:hi], out=b["nl"])
        # at a rigid boundary the reference forms V x B with vr = vt = 0 (nBc = 2
        # branch of get_nl.f90:391-395: VxBt = or4 vp br, VxBp = 0); where the grid
        # keeps its radial velocity, that level's products come from a zero vr grid
        # (the other products of a boundary level are not used)
        for i in self._rigid_kept_vr():
            gi = {k: v[i:i + 1] for k, v in g.items()}
            gi["vrc"] = b["zero_grid"]
            s.get_nl(gi, or2=dv["or2"][i:i + 1], out={k: v[i - lo:i - lo + 1] for k, v in b["nl"].items()})
        lc = None if dv["lcut"] is None else dv["lcut"][lo:hi]
        # analysis outputs at all levels, written in place into rows lo..hi-1;
        # boundary levels without lMagNlBc have zero VxBt / VxBp
        # (rIter.f90:256-259) and every level's dVSrLM is zero at the
        # boundaries (get_td.f90:501-507)
        full = b["lm"]
        s.transform_to_lm_space(nl, lcut=lc, out={k: v[lo:hi] for k, v in full.items()})
        for v in full.values():
            if lo > 0:
                v[:lo].zero_()
            if hi < n:
                v[hi:].zero_()
        full["VSrLM"][0].zero_()
        full["VSrLM"][n - 1].zero_()
        self._boundary_outputs(b, g, dv)
        tdin = {k: spec[k] for k in ("w", "dw", "z")}
        tdin.update({k: full[k] for k in ("AdvrLM", "AdvtLM", "AdvpLM", "VStLM", "VxBrLM", "VxBtLM", "VxBpLM")})
        s.get_td(tdin, dv["r"], self.cor_fac, lcut=dv["lcut"], epsc=dv["epsc"], nbc=dv["nbc"], out=b["td"])

    def _nl_td_general(self, spec: Dict, b: Dict, g: Dict, dv: Dict, lo: int, hi: int):
        """get_nl, the analysis set and get_td through the general routines:
        get_nl_opts on the levels lo..hi-1 with their nBc (the boundary forms
        of V x B at a rigid or stress-free boundary come from the kernel),
        get_td_opts with the boundary flags of every level."""
        s, n, ph = self.s, self.n, self.physics
        fl, prof = ph["flags"], dv["profiles"]
        sl = lambda t: None if t is None else t[lo:hi]  # noqa: E731
        nl = s.get_nl_opts({k: v[lo:hi] for k, v in g.items()}, dv["r"][lo:hi], out=b["nl"], LFfac=self.LFfac,
                           orho1=sl(prof.get("orho1")), beta=sl(prof.get("beta")), otemp1=sl(prof.get("otemp1")),
                           visc=sl(prof.get("visc")), lam=sl(prof.get("lam")), nbc=dv["nbc"][lo:hi],
                           lcr=sl(dv["lcr"]), **ph["const"],
                           **{k: fl[k] for k in self.NL_FLAGS})
        lc = None if dv["lcut"] is None else dv["lcut"][lo:hi]
        full = b["lm"]
        s.transform_to_lm_space(nl, lcut=lc, out={k: v[lo:hi] for k, v in full.items()})
        for v in full.values():
            if lo > 0:
                v[:lo].zero_()
            if hi < n:
                v[hi:].zero_()
        tdin = {k: spec[k] for k in ("w", "dw", "ddw", "z", "dz") if spec.get(k) is not None}
        tdin.update({k: full[k] for k in ("AdvrLM", "AdvtLM", "AdvpLM", "VStLM", "heatTermsLM", "VXitLM", "VxBrLM",
                                          "VxBtLM", "VxBpLM") if k in full})
        s.get_td_opts(tdin, dv["r"], self.cor_fac, outputs=list(b["td"]), out=b["td"], lcut=dv["lcut"],
                      nbc=dv["nbc"], orho1=prof.get("orho1"), beta=prof.get("beta"), temp0=prof.get("temp0"),
                      epsc=dv["epsc"], epscXi=ph["epscXi"], l_conv_nl=fl["l_conv_nl"], l_anel=fl["l_anel"],
                      l_mag_nl=fl["l_mag_nl"], **{k: fl[k] for k in self.TD_FLAGS})

    def _boundary_outputs(self, b: Dict, g: Dict, dv: Dict):
        """The Courant steps, the Lorentz torques and the conducting-boundary
        products of the stage."""
        s, n = self.s, self.n
        b["dtrkc"].fill_(1e10)
        b["dthkc"].fill_(1e10)
        s.courant({k: g[k] for k in ("vrc", "vtc", "vpc", "brc", "btc", "bpc")}, dv["radial"],
                  self.courfac, self.alffac, self.LFfac, self.opm, self.l_cour_alf_damp,
                  dtrkc=b["dtrkc"], dthkc=b["dthkc"])
        if self.torque_ic:
            s.lorentz_torque(g["brc"][n - 1], g["bpc"][n - 1], self.LFfac, self.b0_ic, out=b["torque_ic"])
        if self.torque_ma:
            s.lorentz_torque(g["brc"][0], g["bpc"][0], self.LFfac, self.b0_ma, out=b["torque_ma"])
        if self.l_b_nl_cmb:
            s.get_br_v_bcs(g["brc"][0], g["vtc"][0], g["vpc"][0], self.omega_ma, self.or2[0], 1.0, out=b["cmb"])
        if self.l_b_nl_icb:
            s.get_br_v_bcs(g["brc"][n - 1], g["vtc"][n - 1], g["vpc"][n - 1], self.omega_ic, self.or2[n - 1], 1.0,
                           out=b["icb"])

    @staticmethod
    def _result(b: Dict) -> Dict:
        res = dict(b["td"])
        res["VSrLM"] = b["lm"]["VSrLM"]
        # the stage's one synchronisation: dt_courant wants the steps on the host
        res["dtrkc"], res["dthkc"] = b["dtrkc"].cpu().numpy(), b["dthkc"].cpu().numpy()
        for key in ("cmb", "icb"):
            if key in b:
                res["br_vt_lm_" + key], res["br_vp_lm_" + key] = b[key]
        # the mantle's torque is computed with the inward normal: the radial
        # loop negates it (rIter.f90:462)
        if "torque_ic" in b:
            res["lorentz_torque_ic"] = float(b["torque_ic"].item())
        if "torque_ma" in b:
            res["lorentz_torque_ma"] = -float(b["torque_ma"].item())
        res["grids"] = b["grids"]
        return res

    def step(self, spec: Dict, out: Optional[Dict] = None) -> Dict:
        """One stage from the spectra of transform_to_grid_space (``s``, ``p``,
        ``xi``, ``w`` .. ``dj``; [level][lm] complex CUDA tensors).  Returns
        the get_td outputs (``dwdt`` .. ``dVxBhLM``, into ``out`` where
        given), ``VSrLM`` (dVSrLM, 0 at the boundaries), numpy ``dtrkc`` /
        ``dthkc``, the synthesis ``grids``, at conducting boundaries
        ``br_vt_lm_cmb`` / ``br_vp_lm_cmb`` (or ``_icb``), and with a
        rotating, conducting mantle / inner core ``lorentz_torque_ma`` /
        ``lorentz_torque_ic``."""
        b = self._alloc(spec, out)
        self._enqueue(spec, b)
        return self._result(b)

    def capture(self, spec: Dict) -> "StageGraph":
        """The stage on ``spec`` captured once as a CUDA graph (see StageGraph)."""
        return StageGraph(self, spec)


class StageGraph:
    """One explicit stage captured as a CUDA graph over fixed buffers: every
    replay reads the spectra ``spec`` given at capture (update them in place
    between replays) and rewrites the same output tensors, so a stage costs
    one graph launch and the one synchronisation that brings the Courant
    steps to the host.  The loop's handle must not be captured elsewhere
    meanwhile; replay() binds it to the graph's own stream and returns once
    the stage is complete."""

    def __init__(self, loop: RadialLoop, spec: Dict):
        import torch
        s = loop.s
        for k, v in spec.items():
            if v is None:
                continue
            if not (isinstance(v, torch.Tensor) and v.is_cuda and v.is_contiguous() and v.dtype == torch.complex128
                    and tuple(v.shape) == (loop.n, s.lm_max)):
                raise ValueError("captured spectra must be contiguous complex128 CUDA tensors of shape "
                                 "(%d, %d): %r" % (loop.n, s.lm_max, k))
        self.graph = None
        self.loop, self.spec = loop, spec
        self.b = loop._alloc(spec)
        s.reserve(loop.n)
        self.stream = torch.cuda.Stream(device=spec["w"].device)
        self.stream.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(self.stream):
            loop._enqueue(spec, self.b)   # sizes the workspace, binds the handle to this stream
            self.stream.synchronize()
            s.graph_begin()
            try:
                loop._enqueue(spec, self.b)
            finally:
                self.graph = s.graph_end()

    def replay(self) -> Dict:
        import torch
        with torch.cuda.stream(self.stream):
            # the handle may have been bound to another stream since the capture
            self.loop.s._bind_torch_stream()
            self.loop.s.graph_launch(self.graph)
            return RadialLoop._result(self.b)

    def close(self):
        if self.graph is not None:
            self.loop.s.graph_destroy(self.graph)
            self.graph = None
