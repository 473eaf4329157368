"""ctypes binding of ``libmagic_sht.so`` (C ABI declared in include/magic_sht.h).

The library is built in-tree by ``magic_gb300.build.build()``.  There is no
CPU fallback: if the shared library is missing, importing the transform
layer raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmagic_sht.so")

OK = 0
ERR_ARG, ERR_SIZE, ERR_LCUT, ERR_CUDA, ERR_UNSUPPORTED, ERR_NOMEM, ERR_TIMEOUT = range(1, 8)
FP64, FP32, BF16X3, TF32X2, FP64TC, BF16X5 = 0, 1, 2, 3, 4, 5
PRECISIONS = {"fp64": FP64, "fp32": FP32, "bf16x3": BF16X3, "tf32x2": TF32X2, "fp64tc": FP64TC, "bf16x5": BF16X5}
PHASES = ["inv_leg_scalar", "inv_leg_vector", "fft_inv", "fft_fwd", "fwd_leg_scalar",
          "fwd_leg_vector", "nl", "courant", "td", "bcs"]

_D = ctypes.POINTER(ctypes.c_double)
_I = ctypes.POINTER(ctypes.c_int)
_V = ctypes.c_void_p


class Desc(ctypes.Structure):
    _fields_ = [("l_max", ctypes.c_int), ("m_max", ctypes.c_int), ("minc", ctypes.c_int),
                ("n_theta_max", ctypes.c_int), ("n_phi_max", ctypes.c_int),
                ("nlat_padded", ctypes.c_int), ("precision", ctypes.c_int),
                ("device", ctypes.c_int)]


# grids read and written by magic_sht_get_nl (nl.cu)
NL_IN = ["vrc", "vtc", "vpc", "cvrc", "cvtc", "cvpc", "brc", "btc", "bpc", "cbrc", "cbtc", "cbpc", "sc"]
GRID_SPACE_IN = ["s", "p", "xi", "w", "dw", "ddw", "z", "dz", "b", "db", "ddb", "aj", "dj"]
GRID_SPACE_OUT = ["sc", "pc", "xic", "vrc", "vtc", "vpc", "cvrc", "cvtc", "cvpc",
                  "brc", "btc", "bpc", "cbrc", "cbtc", "cbpc"]
LM_SPACE_IN = ["Advr", "Advt", "Advp", "VSr", "VSt", "VSp", "VxBr", "VxBt", "VxBp", "heatTerms"]
LM_SPACE_OUT = ["AdvrLM", "AdvtLM", "AdvpLM", "VSrLM", "VStLM", "VSpLM", "VxBrLM", "VxBtLM",
                "VxBpLM", "heatTermsLM"]


# velocity derivatives of the u.grad u advection and the anelastic viscous heating
GRID_SPACE_OUT_DV = ["dvrdrc", "dvtdrc", "dvpdrc", "dvrdtc", "dvrdpc", "dvtdpc", "dvpdpc"]


class GridSpaceArgs(ctypes.Structure):
    _fields_ = ([(n, _V) for n in GRID_SPACE_IN] + [("spec_ld", ctypes.c_longlong)] +
                [(n, _V) for n in GRID_SPACE_OUT] + [("grid_ld", ctypes.c_longlong)] +
                [(n, _V) for n in GRID_SPACE_OUT_DV])


TD_IN = ["w", "dw", "z", "AdvrLM", "AdvtLM", "AdvpLM", "VStLM", "VxBrLM", "VxBtLM", "VxBpLM"]
TD_OUT = ["dwdt", "dzdt", "dpdt", "dsdt", "dbdt", "djdt", "dVxBhLM"]


class TdArgs(ctypes.Structure):
    _fields_ = [(n, _V) for n in TD_IN + TD_OUT] + [("spec_ld", ctypes.c_longlong)]


class CourantArgs(ctypes.Structure):
    _fields_ = ([(n, _V) for n in ["vr", "vt", "vp", "br", "bt", "bp"]] + [("grid_ld", ctypes.c_longlong)] +
                [(n, _V) for n in ["orho1", "orho2", "or2", "or4", "delxr2", "delxh2"]] +
                [(n, ctypes.c_double) for n in ["courfac", "alffac", "LFfac", "opm"]] +
                [("l_cour_alf_damp", ctypes.c_int)])


RIGID = ["vr", "vt", "vp", "cvr", "dvrdt", "dvrdp", "dvtdp", "dvpdp"]


class RigidArgs(ctypes.Structure):
    _fields_ = [(n, _V) for n in RIGID]


class Tuning(ctypes.Structure):
    _fields_ = [(n, ctypes.c_int) for n in ("tc_kernel", "tc_order", "pipe_chunk", "fft_rows")]


# the composition flux of l_chemical_conv, at the end of magic_sht_lm_space_args
LM_SPACE_IN_XI = ["VXir", "VXit", "VXip"]
LM_SPACE_OUT_XI = ["VXirLM", "VXitLM", "VXipLM"]


class LmSpaceArgs(ctypes.Structure):
    _fields_ = ([(n, _V) for n in LM_SPACE_IN] + [("grid_ld", ctypes.c_longlong)] +
                [(n, _V) for n in LM_SPACE_OUT] + [("spec_ld", ctypes.c_longlong)] +
                [(n, _V) for n in LM_SPACE_IN_XI + LM_SPACE_OUT_XI])


# the general get_nl (magic_sht_get_nl_opts): switches, constants, per-level arrays
NL_SWITCHES = ["l_conv_nl", "l_adv_curl", "l_mag_LF", "l_heat_nl", "l_chemical_conv", "l_mag_nl", "l_anel"]
NL_PROFILES = ["r", "orho1", "beta", "otemp1", "visc", "lambda"]


class NlOpts(ctypes.Structure):
    _fields_ = ([(n, ctypes.c_int) for n in NL_SWITCHES + ["pad_"]] +
                [(n, ctypes.c_double) for n in ("LFfac", "ViscHeatFac", "OhmLossFac")] +
                [(n, _V) for n in NL_PROFILES + ["nbc", "lcr"]])


NLF_IN = ["vrc", "vtc", "vpc", "cvrc", "cvtc", "cvpc", "dvrdrc", "dvtdrc", "dvpdrc", "dvrdtc", "dvrdpc",
          "dvtdpc", "dvpdpc", "brc", "btc", "bpc", "cbrc", "cbtc", "cbpc", "sc", "xic"]
NLF_OUT = ["Advr", "Advt", "Advp", "VSr", "VSt", "VSp", "VXir", "VXit", "VXip", "VxBr", "VxBt", "VxBp",
           "heatTerms"]


class NlGrids(ctypes.Structure):
    _fields_ = [(n, _V) for n in NLF_IN] + [("grid_ld", ctypes.c_longlong)]


class NlOut(ctypes.Structure):
    _fields_ = [(n, _V) for n in NLF_OUT] + [("grid_ld", ctypes.c_longlong)]


# the general get_td (magic_sht_get_td_opts)
TD_SWITCHES = ["l_conv_nl", "l_corr", "l_double_curl", "l_single_matrix", "l_anel", "l_anelastic_liquid",
               "l_mag_nl"]
TDF_IN = ["w", "dw", "ddw", "z", "dz", "AdvrLM", "AdvtLM", "AdvpLM", "VStLM", "heatTermsLM", "VXitLM",
          "VxBrLM", "VxBtLM", "VxBpLM"]
TDF_OUT = ["dwdt", "dzdt", "dpdt", "dsdt", "dxidt", "dbdt", "djdt", "dVxBhLM", "dVxVhLM", "dVSrLM", "dVXirLM"]


class TdOpts(ctypes.Structure):
    _fields_ = ([(n, ctypes.c_int) for n in TD_SWITCHES + ["pad_"]] +
                [(n, ctypes.c_double) for n in ("cor_fac", "epscXi")] +
                [(n, _V) for n in ("r", "orho1", "beta", "temp0", "epsc", "lcut", "nbc")])


class TdIn(ctypes.Structure):
    _fields_ = [(n, _V) for n in TDF_IN] + [("spec_ld", ctypes.c_longlong)]


class TdOut(ctypes.Structure):
    _fields_ = [(n, _V) for n in TDF_OUT] + [("spec_ld", ctypes.c_longlong)]


# batched facade jobs (magic_sht_inv_batch / magic_sht_fwd_batch): routine
# name -> (MAGIC_SHT_JOB_* code, number of array inputs, number of outputs)
JOBS = {
    "scal_to_spat": (1, 1, 1), "scal_to_grad_spat": (2, 1, 2), "pol_to_grad_spat": (3, 1, 2),
    "torpol_to_spat": (4, 3, 3), "sphtor_to_spat": (5, 2, 2), "torpol_to_curl_spat": (6, 4, 3),
    "pol_to_curlr_spat": (7, 1, 1), "torpol_to_dphspat": (8, 2, 2),
    "scal_to_SH": (101, 1, 1), "spat_to_qst": (102, 3, 3), "spat_to_sphertor": (103, 2, 2),
}


class Job(ctypes.Structure):
    _fields_ = [("routine", ctypes.c_int), ("pad_", ctypes.c_int), ("in", _V * 4), ("out", _V * 3)]


# every entry point of include/magic_sht.h with its argument types
SIGNATURES = {
    "magic_sht_init": [ctypes.POINTER(Desc), ctypes.POINTER(_V)],
    "magic_sht_finalize": [_V],
    "magic_sht_last_error": [],
    "magic_sht_scrambled_theta": [_V, _I],
    "magic_sht_get_sizes": [_V, _I],
    "magic_sht_gauss_grid": [_V, _V, _V],
    "magic_sht_set_stream": [_V, _V],
    "magic_sht_synchronize": [_V],
    "magic_sht_reserve": [_V, ctypes.c_int],
    "magic_sht_scal_to_spat": [_V, _V, _V, ctypes.c_int],
    "magic_sht_scal_to_spat_noalloc": [_V, _V, _V, ctypes.c_int],
    "magic_sht_scal_to_grad_spat": [_V, _V, _V, _V, ctypes.c_int],
    "magic_sht_pol_to_grad_spat": [_V, _V, _V, _V, ctypes.c_int],
    "magic_sht_torpol_to_spat": [_V, _V, _V, _V, _V, _V, _V, ctypes.c_int],
    "magic_sht_sphtor_to_spat": [_V, _V, _V, _V, _V, ctypes.c_int],
    "magic_sht_torpol_to_curl_spat_IC": [_V, ctypes.c_double, ctypes.c_double, _V, _V, _V, _V,
                                         _V, _V, _V],
    "magic_sht_torpol_to_spat_IC": [_V, ctypes.c_double, ctypes.c_double, _V, _V, _V, _V, _V, _V],
    "magic_sht_torpol_to_dphspat": [_V, _V, _V, _V, _V, ctypes.c_int],
    "magic_sht_pol_to_curlr_spat": [_V, _V, _V, ctypes.c_int],
    "magic_sht_torpol_to_curl_spat": [_V, ctypes.c_double, _V, _V, _V, _V, _V, _V, _V,
                                      ctypes.c_int],
    "magic_sht_axi_to_spat": [_V, _V, _V],
    "magic_sht_toraxi_to_spat": [_V, _V, _V, _V, ctypes.c_int],
    "magic_sht_scal_to_SH": [_V, _V, _V, ctypes.c_int],
    "magic_sht_spat_to_qst": [_V, _V, _V, _V, _V, _V, _V, ctypes.c_int],
    "magic_sht_spat_to_sphertor": [_V, _V, _V, _V, _V, ctypes.c_int],
    "magic_sht_transform_to_grid_space": [_V, ctypes.c_int, _V, _V,
                                          ctypes.POINTER(GridSpaceArgs)],
    "magic_sht_transform_to_lm_space": [_V, ctypes.c_int, _V, ctypes.POINTER(LmSpaceArgs)],
    "magic_sht_inv_batch": [_V, ctypes.c_int, _V, _V, ctypes.c_longlong, ctypes.c_longlong, ctypes.POINTER(Job),
                            ctypes.c_int],
    "magic_sht_fwd_batch": [_V, ctypes.c_int, _V, ctypes.c_longlong, ctypes.c_longlong, ctypes.POINTER(Job),
                            ctypes.c_int],
    "magic_sht_set_host_async": [_V, ctypes.c_int],
    "magic_sht_set_tuning": [_V, ctypes.POINTER(Tuning)],
    "magic_sht_get_tuning": [_V, ctypes.POINTER(Tuning)],
    "magic_sht_get_td": [_V, ctypes.c_int, _V, _V, ctypes.c_double, _V, ctypes.POINTER(TdArgs)],
    "magic_sht_get_td_nbc": [_V, ctypes.c_int, _V, _V, ctypes.c_double, _V, _V, ctypes.POINTER(TdArgs)],
    "magic_sht_get_nl": [_V, ctypes.c_int, _V, ctypes.POINTER(GridSpaceArgs), ctypes.POINTER(LmSpaceArgs)],
    "magic_sht_get_td_opts": [_V, ctypes.c_int, ctypes.POINTER(TdOpts), ctypes.POINTER(TdIn),
                              ctypes.POINTER(TdOut)],
    "magic_sht_get_nl_opts": [_V, ctypes.c_int, ctypes.POINTER(NlOpts), ctypes.POINTER(NlGrids),
                              ctypes.POINTER(NlOut)],
    "magic_sht_courant": [_V, ctypes.c_int, ctypes.POINTER(CourantArgs), _V, _V],
    "magic_sht_dt_courant": [ctypes.c_int, _V, _V, ctypes.c_double, ctypes.c_double, _I, _D],
    "magic_sht_v_rigid_boundary": [_V, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.POINTER(RigidArgs)],
    "magic_sht_v_center_sphere": [_V, _V, _V, _V, _V],
    "magic_sht_get_br_v_bcs": [_V, _V, _V, _V, ctypes.c_double, ctypes.c_double, ctypes.c_double, _V, _V],
    "magic_sht_get_b_nl_bcs": [_V, ctypes.c_double, _V, _V, _V, _V],
    "magic_sht_lorentz_torque": [_V, _V, _V, ctypes.c_double, ctypes.c_double, _V],
    "magic_sht_graph_begin": [_V],
    "magic_sht_graph_end": [_V, ctypes.POINTER(_V)],
    "magic_sht_graph_launch": [_V, _V],
    "magic_sht_graph_destroy": [_V],
    "magic_sht_group_create": [_V, ctypes.c_int, ctypes.POINTER(_V)],
    "magic_sht_group_destroy": [_V],
    "magic_sht_group_transform_to_grid_space": [_V, _V, _V, _V, ctypes.POINTER(GridSpaceArgs)],
    "magic_sht_group_transform_to_lm_space": [_V, _V, _V, ctypes.POINTER(LmSpaceArgs)],
    "magic_sht_measure_gflops": [ctypes.c_int, ctypes.c_int, _D],
    "magic_sht_set_profiling": [_V, ctypes.c_int],
    "magic_sht_phase_times": [_V, _V, _V, ctypes.c_int],
    "magic_sht_launch_count": [_V, ctypes.POINTER(ctypes.c_longlong)],
    "magic_sht_device_status": [_V, ctypes.c_int],
    "magic_sht_tc_selftest": [ctypes.c_int, ctypes.c_int, ctypes.c_int, _D],
    "magic_sht_tc_selftest_tf32": [ctypes.c_int, ctypes.c_int, ctypes.c_int, _D],
    "magic_sht_wait_selftest": [ctypes.c_int, ctypes.c_longlong, ctypes.c_int],
}

_lib = None


class ShtError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("magic_sht error %d: %s" % (code, msg))
        self.code = code


def load(path: str = LIB_PATH):
    """Load the CUDA library; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError(
            "libmagic_sht.so is missing (%s); build it with "
            "`python -c 'import __graft_entry__ as g; g.build()'`" % path)
    lib = ctypes.CDLL(path)
    for name, args in SIGNATURES.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = ctypes.c_char_p if name == "magic_sht_last_error" else ctypes.c_int
    _lib = lib
    return lib


def check(rc: int):
    if rc != OK:
        msg = load().magic_sht_last_error()
        raise ShtError(rc, msg.decode() if msg else "")
    return rc
