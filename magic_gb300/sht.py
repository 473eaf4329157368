"""Host-side mirror of MagIC's ``module sht`` (src/sht_native.f90:16-20) over
the GB300 CUDA library.

Arrays follow the reference layouts:
  * spectral: complex128, shape (lm_max,) in st_map order (m-major, l inner);
    batched: (n_levels, lm_max) like the R-distributed ``f_Rloc(lm_max, nR)``;
  * grid: float64, shape (n_phi_max, nlat_padded) in C order, i.e. Fortran
    ``f(nlat_padded, n_phi_max)`` with theta fastest and the theta rows
    scrambled north/south (row 2j north, 2j+1 south); batched:
    (n_levels, n_phi_max, nlat_padded).
Inputs may be numpy arrays (host memory: the call stages them through the
GPU and returns numpy results) or CUDA torch tensors (device memory: the call
runs asynchronously on the current torch stream and returns CUDA tensors).
"""
from __future__ import annotations

import ctypes
from typing import Dict, Optional

import numpy as np

from . import _lib
from ._lib import check


def prime_decomposition(nlon: int) -> int:
    """Closest 2^i 3^j 5^k >= nlon (src/truncation.f90:162-192)."""
    best, dist_min = nlon, 100.0
    for i in range(13):
        for j in range(7):
            for k in range(7):
                res = 2 ** i * 3 ** j * 5 ** k
                dist = res - nlon
                if 0 <= dist < dist_min:
                    best, dist_min = res, dist
    return best


def truncation(l_max: int, nalias: int = 20, minc: int = 1) -> Dict[str, int]:
    """Grid sizes from l_max (src/truncation.f90:50-124, the l_max /= 0 branch)."""
    n_theta = (30 * l_max) // nalias
    n_phi_tot = prime_decomposition(2 * n_theta)
    n_phi_max = n_phi_tot // minc
    n_theta = n_phi_tot // 2
    m_max = min((l_max // minc) * minc, l_max)
    n_m_max = m_max // minc + 1
    lm_max = sum(l_max - m + 1 for m in range(0, m_max + 1, minc))
    return dict(n_theta_max=n_theta, n_phi_tot=n_phi_tot, n_phi_max=n_phi_max, m_max=m_max,
                n_m_max=n_m_max, lm_max=lm_max)


def _torch():
    try:
        import torch
        return torch
    except Exception:  # pragma: no cover
        return None


def _is_torch(x) -> bool:
    t = _torch()
    return t is not None and isinstance(x, t.Tensor)


def _per_level(x, np_dtype, n: int, name: str):
    """(keep-alive object, pointer) of a per-level array (or2, r, lcut, ...):
    a CUDA tensor is passed as it is (device pointer); anything else as a
    contiguous numpy array (host pointer, which the library copies through
    pinned memory without synchronising the stream)."""
    if x is None:
        return None, None
    if _is_torch(x) and x.is_cuda:
        torch = _torch()
        t = x.to(dtype=torch.float64 if np_dtype == np.float64 else torch.int32).contiguous()
        if t.numel() != n:
            raise ValueError("%s needs %d levels, got %d" % (name, n, t.numel()))
        return t, t.data_ptr()
    a = np.ascontiguousarray(x, dtype=np_dtype)
    if a.size != n:
        raise ValueError("%s needs %d levels, got %d" % (name, n, a.size))
    return a, a.ctypes.data


class SHT:
    """One transform instance (grid + truncation), the drop-in for ``module sht``."""

    def __init__(self, l_max: int, minc: int = 1, n_theta_max: Optional[int] = None,
                 n_phi_max: Optional[int] = None, m_max: int = 0, nlat_padded: int = 0,
                 precision: str = "fp64", device: int = -1):
        if n_theta_max is None or n_phi_max is None:
            tr = truncation(l_max, minc=minc)
            n_theta_max = n_theta_max or tr["n_theta_max"]
            n_phi_max = n_phi_max or tr["n_phi_max"]
        self._lib = _lib.load()
        d = _lib.Desc(l_max, m_max, minc, n_theta_max, n_phi_max, nlat_padded,
                      _lib.PRECISIONS[precision], device)
        h = ctypes.c_void_p()
        check(self._lib.magic_sht_init(ctypes.byref(d), ctypes.byref(h)))
        self._h = h
        sz = (ctypes.c_int * 8)()
        check(self._lib.magic_sht_get_sizes(h, sz))
        (self.l_max, self.m_max, self.minc, self.n_theta_max, self.n_phi_max,
         self.nlat_padded, self.n_m_max, self.lm_max) = list(sz)
        self.precision = precision
        self.lm2l = np.array([l for m in range(0, self.m_max + 1, self.minc)
                              for l in range(m, self.l_max + 1)], dtype=np.int64)
        self.lm2m = np.array([m for m in range(0, self.m_max + 1, self.minc)
                              for l in range(m, self.l_max + 1)], dtype=np.int64)
        self._stream = -1  # the handle's own stream until bound to torch's
        self._device = None

    # ---------------------------------------------------------------- life
    def close(self):
        if getattr(self, "_h", None):
            self._lib.magic_sht_finalize(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def initialize_sht(self) -> bool:
        """l_scrambled_theta of the reference (src/sht_native.f90:24-32)."""
        v = ctypes.c_int()
        check(self._lib.magic_sht_scrambled_theta(self._h, ctypes.byref(v)))
        return bool(v.value)

    def gauss_grid(self):
        th = np.zeros(self.n_theta_max)
        w = np.zeros(self.n_theta_max)
        check(self._lib.magic_sht_gauss_grid(self._h, th.ctypes.data, w.ctypes.data))
        return th, w

    def synchronize(self):
        check(self._lib.magic_sht_synchronize(self._h))

    def reserve(self, n_levels: int):
        check(self._lib.magic_sht_reserve(self._h, int(n_levels)))

    def set_stream(self, stream_ptr: Optional[int]):
        check(self._lib.magic_sht_set_stream(self._h, stream_ptr))
        self._stream = stream_ptr

    # ------------------------------------------------------------- helpers
    def _bind_torch_stream(self):
        torch = _torch()
        s = torch.cuda.current_stream().cuda_stream
        if s != self._stream:
            self.set_stream(s)

    def _spec_in(self, x, n=None):
        if _is_torch(x):
            torch = _torch()
            assert x.dtype == torch.complex128, "spectral tensors: complex128"
            x = x.contiguous()
            if x.is_cuda:
                self._bind_torch_stream()
            return x, x.data_ptr()
        a = np.ascontiguousarray(x, dtype=np.complex128)
        return a, a.ctypes.data

    def _grid_in(self, x):
        if _is_torch(x):
            torch = _torch()
            assert x.dtype == torch.float64, "grid tensors: float64"
            x = x.contiguous()
            if x.is_cuda:
                self._bind_torch_stream()
            return x, x.data_ptr()
        a = np.ascontiguousarray(x, dtype=np.float64)
        return a, a.ctypes.data

    def _new(self, like, shape, complex_=False):
        if _is_torch(like):
            torch = _torch()
            dt = torch.complex128 if complex_ else torch.float64
            if like.is_cuda:
                t = torch.zeros(shape, dtype=dt, device=like.device)
            else:
                t = torch.zeros(shape, dtype=dt, pin_memory=True)
            return t, t.data_ptr()
        a = np.zeros(shape, dtype=np.complex128 if complex_ else np.float64)
        return a, a.ctypes.data

    def _grid(self, like, n=None):
        shape = (self.n_phi_max, self.nlat_padded) if n is None else (n, self.n_phi_max, self.nlat_padded)
        return self._new(like, shape)

    def _spec(self, like, n=None):
        shape = (self.lm_max,) if n is None else (n, self.lm_max)
        return self._new(like, shape, complex_=True)

    def _lc(self, lcut):
        return self.l_max if lcut is None else int(lcut)

    # ------------------------------------- spectral -> grid (one level)
    def scal_to_spat(self, Slm, lcut=None):
        S, ps = self._spec_in(Slm)
        f, pf = self._grid(S)
        check(self._lib.magic_sht_scal_to_spat(self._h, ps, pf, self._lc(lcut)))
        return f

    def scal_to_grad_spat(self, Slm, lcut=None):
        S, ps = self._spec_in(Slm)
        a, pa = self._grid(S)
        b, pb = self._grid(S)
        check(self._lib.magic_sht_scal_to_grad_spat(self._h, ps, pa, pb, self._lc(lcut)))
        return a, b

    def pol_to_grad_spat(self, Slm, lcut=None):
        S, ps = self._spec_in(Slm)
        a, pa = self._grid(S)
        b, pb = self._grid(S)
        check(self._lib.magic_sht_pol_to_grad_spat(self._h, ps, pa, pb, self._lc(lcut)))
        return a, b

    def torpol_to_spat(self, Wlm, dWlm, Zlm, lcut=None):
        (W, pw), (dW, pdw), (Z, pz) = self._spec_in(Wlm), self._spec_in(dWlm), self._spec_in(Zlm)
        a, pa = self._grid(W)
        b, pb = self._grid(W)
        c, pc = self._grid(W)
        check(self._lib.magic_sht_torpol_to_spat(self._h, pw, pdw, pz, pa, pb, pc, self._lc(lcut)))
        return a, b, c

    def sphtor_to_spat(self, dWlm, Zlm, lcut=None):
        (dW, pdw), (Z, pz) = self._spec_in(dWlm), self._spec_in(Zlm)
        a, pa = self._grid(dW)
        b, pb = self._grid(dW)
        check(self._lib.magic_sht_sphtor_to_spat(self._h, pdw, pz, pa, pb, self._lc(lcut)))
        return a, b

    def torpol_to_curl_spat_IC(self, r, r_ICB, dBlm, ddBlm, Jlm, dJlm):
        ins = [self._spec_in(x) for x in (dBlm, ddBlm, Jlm, dJlm)]
        outs = [self._grid(ins[0][0]) for _ in range(3)]
        check(self._lib.magic_sht_torpol_to_curl_spat_IC(self._h, float(r), float(r_ICB),
                                                        *[p for _, p in ins], *[p for _, p in outs]))
        return tuple(o for o, _ in outs)

    def torpol_to_spat_IC(self, r, r_ICB, Wlm, dWlm, Zlm):
        ins = [self._spec_in(x) for x in (Wlm, dWlm, Zlm)]
        outs = [self._grid(ins[0][0]) for _ in range(3)]
        check(self._lib.magic_sht_torpol_to_spat_IC(self._h, float(r), float(r_ICB),
                                                   *[p for _, p in ins], *[p for _, p in outs]))
        return tuple(o for o, _ in outs)

    def torpol_to_dphspat(self, dWlm, Zlm, lcut=None):
        (dW, pdw), (Z, pz) = self._spec_in(dWlm), self._spec_in(Zlm)
        a, pa = self._grid(dW)
        b, pb = self._grid(dW)
        check(self._lib.magic_sht_torpol_to_dphspat(self._h, pdw, pz, pa, pb, self._lc(lcut)))
        return a, b

    def pol_to_curlr_spat(self, Qlm, lcut=None):
        Q, pq = self._spec_in(Qlm)
        f, pf = self._grid(Q)
        check(self._lib.magic_sht_pol_to_curlr_spat(self._h, pq, pf, self._lc(lcut)))
        return f

    def torpol_to_curl_spat(self, or2, Blm, ddBlm, Jlm, dJlm, lcut=None):
        ins = [self._spec_in(x) for x in (Blm, ddBlm, Jlm, dJlm)]
        outs = [self._grid(ins[0][0]) for _ in range(3)]
        check(self._lib.magic_sht_torpol_to_curl_spat(self._h, float(or2), *[p for _, p in ins],
                                                     *[p for _, p in outs], self._lc(lcut)))
        return tuple(o for o, _ in outs)

    def axi_to_spat(self, fl_ax):
        F, pf = self._spec_in(fl_ax)
        out, po = self._new(F, (self.n_theta_max,))
        check(self._lib.magic_sht_axi_to_spat(self._h, pf, po))
        return out

    def toraxi_to_spat(self, fl_ax, lcut=None):
        F, pf = self._spec_in(fl_ax)
        a, pa = self._new(F, (self.n_theta_max,))
        b, pb = self._new(F, (self.n_theta_max,))
        check(self._lib.magic_sht_toraxi_to_spat(self._h, pf, pa, pb, self._lc(lcut)))
        return a, b

    # ------------------------------------- grid -> spectral (one level)
    def scal_to_SH(self, f, lcut=None):
        F, pf = self._grid_in(f)
        o, po = self._spec(F)
        check(self._lib.magic_sht_scal_to_SH(self._h, pf, po, self._lc(lcut)))
        return o

    def spat_to_qst(self, f, g, h, lcut=None):
        ins = [self._grid_in(x) for x in (f, g, h)]
        outs = [self._spec(ins[0][0]) for _ in range(3)]
        check(self._lib.magic_sht_spat_to_qst(self._h, *[p for _, p in ins], *[p for _, p in outs],
                                             self._lc(lcut)))
        return tuple(o for o, _ in outs)

    def spat_to_sphertor(self, f, g, lcut=None):
        ins = [self._grid_in(x) for x in (f, g)]
        outs = [self._spec(ins[0][0]) for _ in range(2)]
        check(self._lib.magic_sht_spat_to_sphertor(self._h, *[p for _, p in ins],
                                                  *[p for _, p in outs], self._lc(lcut)))
        return tuple(o for o, _ in outs)

    # ------------------------------------- the radial loop's transform set
    def _levels(self, arr, n, lcut):
        return _per_level(lcut, np.int32, n, "lcut")

    def _grid_space_call(self, spec: dict, or2, lcut, out, derivatives=False):
        """The argument block of one transform_to_grid_space call: (n, args,
        outputs, or2 pointer, lcut pointer, arrays to keep alive)."""
        keys = [k for k in _lib.GRID_SPACE_IN if spec.get(k) is not None]
        first = spec[keys[0]]
        n = int(first.shape[0])
        a = _lib.GridSpaceArgs()
        keep = []
        for k in keys:
            arr, p = self._spec_in(spec[k])
            assert tuple(arr.shape) == (n, self.lm_max), k
            keep.append(arr)
            setattr(a, k, p)
        a.spec_ld = self.lm_max
        produced = {
            "sc": "s", "pc": "p", "xic": "xi",
            "vrc": "w", "vtc": "w", "vpc": "w", "cvrc": "ddw", "cvtc": "ddw", "cvpc": "ddw",
            "brc": "b", "btc": "b", "bpc": "b", "cbrc": "ddb", "cbtc": "ddb", "cbpc": "ddb",
        }
        outs = {} if out is None else dict(out)
        skip = {k for k, v in outs.items() if v is None}  # outputs the caller does not want
        for k in skip:
            del outs[k]
        for k in _lib.GRID_SPACE_OUT:
            if k in skip or (spec.get(produced[k]) is None and k not in outs):
                continue
            if k not in outs:
                outs[k], _ = self._grid(first, n)
            setattr(a, k, outs[k].data_ptr() if _is_torch(outs[k]) else outs[k].ctypes.data)
        # velocity derivatives (rIter.f90:527-545) on request or when given in `out`
        need = {"dvrdrc": ("dw", "ddw", "dz"), "dvtdrc": ("dw", "ddw", "dz"), "dvpdrc": ("dw", "ddw", "dz"),
                "dvrdtc": ("w",), "dvrdpc": ("w",), "dvtdpc": ("dw", "z"), "dvpdpc": ("dw", "z")}
        for k in _lib.GRID_SPACE_OUT_DV:
            if k in skip or (k not in outs and not (derivatives and all(spec.get(x) is not None for x in need[k]))):
                continue
            if k not in outs:
                outs[k], _ = self._grid(first, n)
            setattr(a, k, outs[k].data_ptr() if _is_torch(outs[k]) else outs[k].ctypes.data)
        a.grid_ld = self.n_phi_max * self.nlat_padded
        or2_arr, por2 = _per_level(or2, np.float64, n, "or2")
        lc_arr, plc = self._levels(first, n, lcut)
        keep += [or2_arr, lc_arr]
        return n, a, outs, por2, plc, keep

    def transform_to_grid_space(self, spec: dict, or2=None, lcut=None, out: Optional[dict] = None,
                                derivatives: bool = False):
        """rIter.f90:466-622 for many radial levels; `spec` maps the names of
        _lib.GRID_SPACE_IN to (n_levels, lm_max) arrays; returns the grid dict.
        ``derivatives``: also the velocity derivatives of the u.grad u
        advection and the anelastic viscous heating (``dvrdrc`` ..
        ``dvpdpc``, rIter.f90:527-545).  An entry None in ``out`` leaves that
        output out (``cvtc`` and ``cvpc`` None: the u.grad u set's
        pol_to_curlr_spat(z) alone, rIter.f90:540)."""
        n, a, outs, por2, plc, keep = self._grid_space_call(spec, or2, lcut, out, derivatives)
        check(self._lib.magic_sht_transform_to_grid_space(self._h, n, por2, plc, ctypes.byref(a)))
        return outs

    def _lm_space_call(self, grids: dict, lcut, out):
        """The argument block of one transform_to_lm_space call: (n, args,
        outputs, lcut pointer, arrays to keep alive)."""
        names_in = _lib.LM_SPACE_IN + _lib.LM_SPACE_IN_XI
        names_out = _lib.LM_SPACE_OUT + _lib.LM_SPACE_OUT_XI
        keys = [k for k in names_in if grids.get(k) is not None]
        first = grids[keys[0]]
        n = int(first.shape[0])
        a = _lib.LmSpaceArgs()
        keep = []
        for k in keys:
            arr, p = self._grid_in(grids[k])
            keep.append(arr)
            setattr(a, k, p)
        a.grid_ld = self.n_phi_max * self.nlat_padded
        outs = {} if out is None else dict(out)
        for kin, kout in zip(names_in, names_out):
            if grids.get(kin) is None:
                continue
            if kout not in outs:
                outs[kout], _ = self._spec(first, n)
            setattr(a, kout, outs[kout].data_ptr() if _is_torch(outs[kout]) else outs[kout].ctypes.data)
        a.spec_ld = self.lm_max
        lc_arr, plc = self._levels(first, n, lcut)
        keep.append(lc_arr)
        return n, a, outs, plc, keep

    def transform_to_lm_space(self, grids: dict, lcut=None, out: Optional[dict] = None):
        """rIter.f90:624-712 for many radial levels (also V Xi -> VXirLM,
        VXitLM, VXipLM when ``VXir`` .. ``VXip`` are given)."""
        n, a, outs, plc, keep = self._lm_space_call(grids, lcut, out)
        check(self._lib.magic_sht_transform_to_lm_space(self._h, n, plc, ctypes.byref(a)))
        return outs

    def _batch(self, jobs, inverse: bool, lcut, or2=None):
        """(n, Job array, outputs per job, keep-alive list, lcut / or2 pointers)
        of magic_sht_inv_batch / magic_sht_fwd_batch."""
        if not jobs:
            raise ValueError("no jobs")
        n = None
        arr = (_lib.Job * len(jobs))()
        outs, keep = [], []
        for j, job in enumerate(jobs):
            name, ins = job[0], job[1:]
            code, n_in, n_out = _lib.JOBS[name]
            if (code < 100) != inverse:
                raise ValueError("%s is not a %s routine" % (name, "synthesis" if inverse else "analysis"))
            if len(ins) != n_in:
                raise ValueError("%s takes %d arrays, got %d" % (name, n_in, len(ins)))
            arr[j].routine = code
            for k, x in enumerate(ins):
                t, p = self._spec_in(x) if inverse else self._grid_in(x)
                if n is None:
                    n = int(t.shape[0])
                if int(t.shape[0]) != n:
                    raise ValueError("every array needs the same number of levels")
                keep.append(t)
                getattr(arr[j], "in")[k] = p
            o = []
            for k in range(n_out):
                t, p = self._grid(keep[-1], n) if inverse else self._spec(keep[-1], n)
                o.append(t)
                arr[j].out[k] = p
            outs.append(tuple(o))
        lc_arr, plc = self._levels(None, n, lcut)
        or2_arr, por2 = _per_level(or2, np.float64, n, "or2")
        keep += [lc_arr, or2_arr]
        return n, arr, outs, keep, plc, por2

    def inv_batch(self, jobs, or2=None, lcut=None):
        """Facade synthesis routines over many levels in one call
        (magic_sht_inv_batch): ``jobs`` is a list of (routine name, array
        inputs...) in the routine's argument order, each input (n_levels,
        lm_max); ``or2`` per level for torpol_to_curl_spat jobs.  Returns one
        tuple of (n_levels, n_phi_max, nlat_padded) outputs per job."""
        n, arr, outs, keep, plc, por2 = self._batch(jobs, True, lcut, or2)
        check(self._lib.magic_sht_inv_batch(self._h, n, por2, plc, self.lm_max, self.n_phi_max * self.nlat_padded,
                                            arr, len(jobs)))
        return outs

    def fwd_batch(self, jobs, lcut=None):
        """Facade analysis routines over many levels in one call
        (magic_sht_fwd_batch): ``jobs`` = [(routine name, grids...)], each grid
        (n_levels, n_phi_max, nlat_padded); returns one tuple of (n_levels,
        lm_max) spectra per job."""
        n, arr, outs, keep, plc, _ = self._batch(jobs, False, lcut)
        check(self._lib.magic_sht_fwd_batch(self._h, n, plc, self.n_phi_max * self.nlat_padded, self.lm_max,
                                            arr, len(jobs)))
        return outs

    def tuning(self) -> Dict[str, int]:
        """Runtime tuning of this handle (magic_sht_get_tuning): tc_kernel,
        tc_order, pipe_chunk, fft_rows."""
        t = _lib.Tuning()
        check(self._lib.magic_sht_get_tuning(self._h, ctypes.byref(t)))
        return {n: getattr(t, n) for n, _ in _lib.Tuning._fields_}

    def set_tuning(self, **kw):
        """Change some of tc_kernel, tc_order, pipe_chunk, fft_rows
        (magic_sht_set_tuning); returns the previous settings."""
        old = self.tuning()
        bad = set(kw) - set(old)
        if bad:
            raise ValueError("unknown tuning keys %s" % sorted(bad))
        new = dict(old, **kw)
        t = _lib.Tuning(*[int(new[n]) for n, _ in _lib.Tuning._fields_])
        check(self._lib.magic_sht_set_tuning(self._h, ctypes.byref(t)))
        return old

    def set_host_async(self, on: bool):
        """Batched calls on host arrays return once queued; results are valid
        after ``synchronize()`` (magic_sht_set_host_async)."""
        check(self._lib.magic_sht_set_host_async(self._h, 1 if on else 0))

    def get_nl(self, grids: dict, or2=None, out: Optional[dict] = None):
        """Grid-space nonlinear products between the two transform sets
        (get_nl.f90:213-441, rIter.f90:650-655): from the synthesis grids
        (``vrc`` .. ``cbpc``, ``sc``; CUDA tensors [level][phi][theta]) the
        analysis inputs ``Advr`` .. ``heatTerms`` (Boussinesq, curl-form
        advection, unit constants, heatTerms = ohmic losses).  ``or2``: per
        level, numpy or CUDA.  FP64 arithmetic on an FP64 handle, FP32 on the
        reduced forms."""
        import torch
        missing = [k for k in _lib.NL_IN if grids.get(k) is None]
        if missing:
            raise ValueError("get_nl needs the grids %s" % missing)
        first = grids[_lib.NL_IN[0]]
        if not (_is_torch(first) and first.is_cuda):
            raise ValueError("get_nl takes CUDA tensors")
        n = int(first.shape[0])
        g = _lib.GridSpaceArgs()
        keep = []
        for k in _lib.NL_IN:
            t = grids[k].contiguous()
            keep.append(t)
            setattr(g, k, t.data_ptr())
        g.grid_ld = self.n_phi_max * self.nlat_padded
        outs = {} if out is None else dict(out)
        nl = _lib.LmSpaceArgs()
        for k in _lib.LM_SPACE_IN:
            if k not in outs:
                outs[k] = torch.empty_like(keep[0])
            setattr(nl, k, outs[k].data_ptr())
        nl.grid_ld = self.n_phi_max * self.nlat_padded
        or2_arr, por2 = _per_level(or2, np.float64, n, "or2")
        self._bind_torch_stream()
        check(self._lib.magic_sht_get_nl(self._h, n, por2, ctypes.byref(g), ctypes.byref(nl)))
        return outs

    def get_nl_opts(self, grids: dict, r, out: Optional[dict] = None, LFfac: float = 1.0,
                    ViscHeatFac: float = 1.0, OhmLossFac: float = 1.0, orho1=None, beta=None, otemp1=None,
                    visc=None, lam=None, nbc=None, lcr=None, l_conv_nl=True, l_adv_curl=True, l_mag_LF=True,
                    l_heat_nl=True, l_chemical_conv=False, l_mag_nl=True, l_anel=False):
        """The grid-space nonlinear products with the reference's switches and
        radial functions (get_nl.f90:213-441, rIter.f90:645-662;
        magic_sht_get_nl_opts).  ``grids``: CUDA tensors [level][phi][theta]
        named as in the reference (``vrc`` .. ``cvpc``, ``dvrdrc`` ..
        ``dvpdpc``, ``brc`` .. ``cbpc``, ``sc``, ``xic``; the ones the switches
        need).  ``r`` and the profiles: per level, numpy or CUDA.  Returns the
        outputs ``Advr`` .. ``heatTerms`` (new zero-filled tensors unless given
        in ``out``; entries a level does not produce keep their values)."""
        import torch
        first = next(v for v in grids.values() if v is not None)
        if not (_is_torch(first) and first.is_cuda):
            raise ValueError("get_nl_opts takes CUDA tensors")
        n = int(first.shape[0])
        g = _lib.NlGrids()
        keep = []
        for k in _lib.NLF_IN:
            t = grids.get(k)
            if t is not None:
                t = t.contiguous()
                keep.append(t)
                setattr(g, k, t.data_ptr())
        g.grid_ld = self.n_phi_max * self.nlat_padded
        outs = {} if out is None else dict(out)
        o = _lib.NlOut()
        for k in _lib.NLF_OUT:
            if k not in outs:
                outs[k] = torch.zeros_like(first)
            setattr(o, k, outs[k].data_ptr())
        o.grid_ld = self.n_phi_max * self.nlat_padded
        opt = _lib.NlOpts()
        for k, v in (("l_conv_nl", l_conv_nl), ("l_adv_curl", l_adv_curl), ("l_mag_LF", l_mag_LF),
                     ("l_heat_nl", l_heat_nl), ("l_chemical_conv", l_chemical_conv), ("l_mag_nl", l_mag_nl),
                     ("l_anel", l_anel)):
            setattr(opt, k, 1 if v else 0)
        opt.LFfac, opt.ViscHeatFac, opt.OhmLossFac = LFfac, ViscHeatFac, OhmLossFac
        held = []
        for k, v in (("r", r), ("orho1", orho1), ("beta", beta), ("otemp1", otemp1), ("visc", visc),
                     ("lambda", lam)):
            arr, ptr = _per_level(v, np.float64, n, k)
            held.append(arr)
            setattr(opt, k, ptr)
        for k, v in (("nbc", nbc), ("lcr", lcr)):
            arr, ptr = _per_level(v, np.int32, n, k)
            held.append(arr)
            setattr(opt, k, ptr)
        self._bind_torch_stream()
        check(self._lib.magic_sht_get_nl_opts(self._h, n, ctypes.byref(opt), ctypes.byref(g), ctypes.byref(o)))
        return outs

    def get_td_opts(self, spec: dict, r, cor_fac: float, outputs=None, out: Optional[dict] = None,
                    lcut=None, nbc=None, orho1=None, beta=None, temp0=None, epsc=None, epscXi: float = 0.0,
                    l_conv_nl=True, l_corr=True, l_double_curl=False, l_single_matrix=False, l_anel=False,
                    l_anelastic_liquid=False, l_mag_nl=True):
        """The spectral assembly with the reference's switches
        (magic_sht_get_td_opts, get_td.f90 as rIter.f90:410-428 calls it).
        ``spec``: CUDA tensors [level][lm] named as in the reference (``w``,
        ``dw``, ``ddw``, ``z``, ``dz``, ``AdvrLM`` .. ``VxBpLM``, ``VXitLM``,
        ``heatTermsLM``; the ones the outputs need).  ``outputs``: the names
        to compute (default: all of dwdt, dzdt, dpdt, dsdt, dxidt, dbdt, djdt,
        dVxBhLM, dVxVhLM, dVSrLM, dVXirLM); tensors not given in ``out`` are
        new and zero-filled, and entries not produced keep their values."""
        import torch
        first = next(v for v in spec.values() if v is not None)
        if not (_is_torch(first) and first.is_cuda):
            raise ValueError("get_td_opts takes CUDA tensors")
        n = int(first.shape[0])
        names = list(_lib.TDF_OUT) if outputs is None else list(outputs)
        a = _lib.TdIn()
        keep = []
        for k in _lib.TDF_IN:
            t = spec.get(k)
            if t is not None:
                t = t.contiguous()
                keep.append(t)
                setattr(a, k, t.data_ptr())
        a.spec_ld = self.lm_max
        outs = {} if out is None else dict(out)
        b = _lib.TdOut()
        for k in names:
            if k not in outs:
                outs[k] = torch.zeros((n, self.lm_max), dtype=torch.complex128, device=first.device)
            setattr(b, k, outs[k].data_ptr())
        b.spec_ld = self.lm_max
        o = _lib.TdOpts()
        for k, v in (("l_conv_nl", l_conv_nl), ("l_corr", l_corr), ("l_double_curl", l_double_curl),
                     ("l_single_matrix", l_single_matrix), ("l_anel", l_anel),
                     ("l_anelastic_liquid", l_anelastic_liquid), ("l_mag_nl", l_mag_nl)):
            setattr(o, k, 1 if v else 0)
        o.cor_fac, o.epscXi = cor_fac, epscXi
        held = []
        for k, v in (("r", r), ("orho1", orho1), ("beta", beta), ("temp0", temp0), ("epsc", epsc)):
            arr, ptr = _per_level(v, np.float64, n, k)
            held.append(arr)
            setattr(o, k, ptr)
        for k, v in (("lcut", lcut), ("nbc", nbc)):
            arr, ptr = _per_level(v, np.int32, n, k)
            held.append(arr)
            setattr(o, k, ptr)
        self._bind_torch_stream()
        check(self._lib.magic_sht_get_td_opts(self._h, n, ctypes.byref(o), ctypes.byref(a), ctypes.byref(b)))
        return outs

    def get_td(self, spec: dict, r, cor_fac: float, lcut=None, epsc=None, out: Optional[dict] = None,
               nbc=None):
        """Spectral assembly of the explicit time derivatives (get_td.f90):
        from CUDA tensors ``w``, ``dw``, ``z`` and the analysis outputs
        (``AdvrLM`` .. ``VxBpLM``) the outputs ``dwdt``, ``dzdt``, ``dpdt``,
        ``dsdt``, ``dbdt``, ``djdt``, ``dVxBhLM`` ([level][lm] complex).
        ``nbc`` (per level, nBc of the radial loop): at a level with nbc != 0
        only ``dVxBhLM`` is written.  Per-level arrays (``r``, ``lcut``,
        ``epsc``, ``nbc``): numpy or CUDA.  FP64 arithmetic on an FP64 handle,
        FP32 on the reduced forms."""
        import torch
        missing = [k for k in _lib.TD_IN if spec.get(k) is None]
        if missing:
            raise ValueError("get_td needs %s" % missing)
        first = spec[_lib.TD_IN[0]]
        if not (_is_torch(first) and first.is_cuda):
            raise ValueError("get_td takes CUDA tensors")
        n = int(first.shape[0])
        a = _lib.TdArgs()
        keep = []
        for k in _lib.TD_IN:
            t = spec[k].contiguous()
            keep.append(t)
            setattr(a, k, t.data_ptr())
        outs = {} if out is None else dict(out)
        for k in _lib.TD_OUT:
            if k not in outs:
                outs[k] = torch.empty_like(keep[0])
            setattr(a, k, outs[k].data_ptr())
        a.spec_ld = self.lm_max
        r_arr, pr = _per_level(r, np.float64, n, "r")
        lc, plc = _per_level(lcut, np.int32, n, "lcut")
        ep, pep = _per_level(epsc, np.float64, n, "epsc")
        bc, pbc = _per_level(nbc, np.int32, n, "nbc")
        self._bind_torch_stream()
        check(self._lib.magic_sht_get_td_nbc(self._h, n, pr, plc, float(cor_fac), pep, pbc, ctypes.byref(a)))
        return outs

    def courant(self, grids: dict, radial: dict, courfac: float, alffac: float, LFfac: float = 1.0,
                opm: float = 1.0, alf_damp: bool = True, dtrkc=None, dthkc=None):
        """Courant condition of the radial loop (courant.f90:54-278) on CUDA
        grids ``vrc``, ``vtc``, ``vpc`` (and ``brc``, ``btc``, ``bpc`` for the
        Lorentz-force term; leave them out when it is off), [level][phi][theta].
        ``radial`` holds per-level arrays ``orho1``, ``orho2``, ``or2``,
        ``or4``, ``delxr2``, ``delxh2`` (numpy or CUDA tensors).  Returns
        (dtrkc, dthkc), each the minimum of its start value (1e10 by default,
        as in the radial loop) and the level's Courant step: numpy arrays, or
        the given CUDA tensors updated in place (then nothing synchronises)."""
        v = grids["vrc"]
        if not (_is_torch(v) and v.is_cuda):
            raise ValueError("courant takes CUDA grids")
        n = int(v.shape[0])
        a = _lib.CourantArgs()
        keep = []
        for k, f in (("vrc", "vr"), ("vtc", "vt"), ("vpc", "vp"), ("brc", "br"), ("btc", "bt"), ("bpc", "bp")):
            t = grids.get(k)
            if t is None:
                continue
            t = t.contiguous()
            keep.append(t)
            setattr(a, f, t.data_ptr())
        a.grid_ld = int(v[0].numel())
        rf = {}
        for k in ("orho1", "orho2", "or2", "or4", "delxr2", "delxh2"):
            rf[k], p = _per_level(radial[k], np.float64, n, "radial[%r]" % k)
            setattr(a, k, p)
        a.courfac, a.alffac, a.LFfac, a.opm = float(courfac), float(alffac), float(LFfac), float(opm)
        a.l_cour_alf_damp = 1 if alf_damp else 0

        def start(x):
            if _is_torch(x) and x.is_cuda:
                if x.dtype != _torch().float64 or not x.is_contiguous() or x.numel() != n:
                    raise ValueError("dtrkc / dthkc tensors: contiguous float64, %d levels (updated in place)" % n)
                return x, x.data_ptr()
            arr = np.full(n, 1e10) if x is None else np.array(x, dtype=np.float64)
            return arr, arr.ctypes.data
        dr, pdr = start(dtrkc)
        dh, pdh = start(dthkc)
        self._bind_torch_stream()
        check(self._lib.magic_sht_courant(self._h, n, ctypes.byref(a), pdr, pdh))
        return dr, dh

    # ------------------------------------------------ boundary pieces
    def v_rigid_boundary(self, grids: dict, r2_rho0: float, omega: float, keep_vr: bool = False):
        """v_rigid_boundary (nonlinear_bcs.f90:120-175) in place on one level's
        grids: ``vr``, ``vt``, ``vp`` and, when given (lDeriv), ``cvr``,
        ``dvrdt``, ``dvrdp``, ``dvtdp``, ``dvpdp`` (numpy or CUDA, each
        (n_phi_max, nlat_padded))."""
        a = _lib.RigidArgs()
        keep = []
        for k in _lib.RIGID:
            x = grids.get(k)
            if x is None:
                continue
            if _is_torch(x) and not x.is_contiguous():
                raise ValueError("%s must be contiguous (written in place)" % k)
            if not _is_torch(x) and not (isinstance(x, np.ndarray) and x.flags.c_contiguous
                                         and x.dtype == np.float64):
                raise ValueError("%s must be a contiguous float64 array (written in place)" % k)
            keep.append(x)
            setattr(a, k, x.data_ptr() if _is_torch(x) else x.ctypes.data)
        self._bind_torch_stream()
        check(self._lib.magic_sht_v_rigid_boundary(self._h, float(r2_rho0), float(omega), 1 if keep_vr else 0,
                                                   ctypes.byref(a)))
        return grids

    def v_center_sphere(self, ddw):
        """v_center_sphere (nonlinear_bcs.f90:177-224): (vr, vt, vp) of the l = 1
        flow at the centre of a full sphere from the spectrum ``ddw``."""
        x, px = self._spec_in(ddw)
        outs = [self._grid(x) for _ in range(3)]
        check(self._lib.magic_sht_v_center_sphere(self._h, px, *[p for _, p in outs]))
        return tuple(o for o, _ in outs)

    def get_br_v_bcs(self, br, vt, vp, omega: float, or2: float, orho1: float, out=None):
        """get_br_v_bcs (nonlinear_bcs.f90:24-69): (br_vt_lm, br_vp_lm), into
        the two spectra of ``out`` when given."""
        ins = [self._grid_in(x) for x in (br, vt, vp)]
        if out is None:
            outs = [self._spec(ins[0][0]) for _ in range(2)]
        else:
            outs = [(o, o.data_ptr() if _is_torch(o) else o.ctypes.data) for o in out]
        check(self._lib.magic_sht_get_br_v_bcs(self._h, *[p for _, p in ins], float(omega), float(or2),
                                               float(orho1), *[p for _, p in outs]))
        return tuple(o for o, _ in outs)

    def lorentz_torque(self, br, bp, LFfac: float = 1.0, b0: float = 0.0, out=None):
        """get_lorentz_torque (outRot.f90:423-483) of one boundary level's
        grids br, bp (numpy or CUDA): LFfac 2 pi / n_phi_max times the
        Gauss-weighted sum of (br - b0 cos(theta)) bp.  Returns the torque as
        a float, or writes it into the one-element float64 CUDA tensor
        ``out`` (then nothing synchronises)."""
        (a, pa), (b, pb) = self._grid_in(br), self._grid_in(bp)
        if out is not None:
            if not (_is_torch(out) and out.is_cuda and out.dtype == _torch().float64 and out.numel() == 1):
                raise ValueError("out: a one-element float64 CUDA tensor")
            pt, res = out.data_ptr(), None
        else:
            res = np.zeros(1)
            pt = res.ctypes.data
        check(self._lib.magic_sht_lorentz_torque(self._h, pa, pb, float(LFfac), float(b0), pt))
        return out if res is None else float(res[0])

    def get_b_nl_bcs(self, bc: str, fac: float, br_vt_lm, br_vp_lm):
        """get_b_nl_bcs (nonlinear_bcs.f90:71-118): (b_nl_bc, aj_nl_bc) at the
        'CMB' (fac = conductance_ma prmag), (None, aj_nl_bc) at the 'ICB'
        (fac = sigma_ratio prmag)."""
        if bc not in ("CMB", "ICB"):
            raise ValueError("bc must be 'CMB' or 'ICB'")
        vp_, pvp = self._spec_in(br_vp_lm)
        vt_, pvt = self._spec_in(br_vt_lm) if bc == "CMB" else (None, None)
        aj, paj = self._spec(vp_)
        b, pb = self._spec(vp_) if bc == "CMB" else (None, None)
        check(self._lib.magic_sht_get_b_nl_bcs(self._h, float(fac), pvt, pvp, pb, paj))
        return b, aj

    # ---------------------------------------------------------- profiling
    def set_profiling(self, on: bool):
        check(self._lib.magic_sht_set_profiling(self._h, 1 if on else 0))

    def phase_times(self, reset: bool = True):
        n = len(_lib.PHASES)
        ms = (ctypes.c_double * n)()
        cnt = (ctypes.c_longlong * n)()
        check(self._lib.magic_sht_phase_times(self._h, ms, cnt, 1 if reset else 0))
        return {k: (float(ms[i]), int(cnt[i])) for i, k in enumerate(_lib.PHASES)}

    def device_status(self, clear: bool = True):
        """Raise if a bounded device wait of an earlier tensor-core kernel gave up."""
        check(self._lib.magic_sht_device_status(self._h, 1 if clear else 0))

    def launch_count(self) -> int:
        v = ctypes.c_longlong()
        check(self._lib.magic_sht_launch_count(self._h, ctypes.byref(v)))
        return int(v.value)

    # ------------------------------------------------------------- graphs
    def graph_begin(self):
        """Start capturing on the current torch stream (must not be the default stream)."""
        if _torch() is not None and _torch().cuda.is_available():
            self._bind_torch_stream()
        check(self._lib.magic_sht_graph_begin(self._h))

    def graph_end(self):
        g = ctypes.c_void_p()
        check(self._lib.magic_sht_graph_end(self._h, ctypes.byref(g)))
        return g

    def graph_launch(self, g):
        check(self._lib.magic_sht_graph_launch(self._h, g))

    def graph_destroy(self, g):
        check(self._lib.magic_sht_graph_destroy(g))


class SHTGroup:
    """Several independent instances (SHT handles of different l_max, minc and
    grids, all precision="fp64tc", all "bf16x5" or all "bf16x3") transformed together
    (magic_sht_group_*): the Legendre sums of every instance run as one pack
    and one persistent tensor-core launch per direction and field kind, with
    results equal to the instances' own calls bit for bit.  Spectra and grids
    are CUDA tensors; every call runs on torch's current stream, to which all
    instances are bound."""

    def __init__(self, shts):
        self.shts = list(shts)
        self._lib = _lib.load()
        arr = (ctypes.c_void_p * len(self.shts))(*[s._h.value for s in self.shts])
        g = ctypes.c_void_p()
        check(self._lib.magic_sht_group_create(arr, len(self.shts), ctypes.byref(g)))
        self._g = g

    def close(self):
        if getattr(self, "_g", None):
            self._lib.magic_sht_group_destroy(self._g)
            self._g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _bind(self):
        for s in self.shts:
            s._bind_torch_stream()

    def transform_to_grid_space(self, specs, or2s=None, lcuts=None, outs=None, derivatives=False):
        """specs[i] (and or2s[i], lcuts[i], outs[i], ``derivatives``) as
        SHT.transform_to_grid_space of instance i; returns the list of grid dicts."""
        k = len(self.shts)
        or2s = or2s or [None] * k
        lcuts = lcuts or [None] * k
        outs = outs or [None] * k
        calls = [s._grid_space_call(specs[i], or2s[i], lcuts[i], outs[i], derivatives)
                 for i, s in enumerate(self.shts)]
        self._bind()
        n = (ctypes.c_int * k)(*[c[0] for c in calls])
        args = (_lib.GridSpaceArgs * k)(*[c[1] for c in calls])
        por2 = (ctypes.c_void_p * k)(*[c[3] for c in calls])
        plc = (ctypes.c_void_p * k)(*[c[4] for c in calls])
        check(self._lib.magic_sht_group_transform_to_grid_space(self._g, n, por2, plc, args))
        return [c[2] for c in calls]

    def transform_to_lm_space(self, grids, lcuts=None, outs=None):
        """grids[i] (and lcuts[i], outs[i]) as SHT.transform_to_lm_space of
        instance i; returns the list of spectral dicts."""
        k = len(self.shts)
        lcuts = lcuts or [None] * k
        outs = outs or [None] * k
        calls = [s._lm_space_call(grids[i], lcuts[i], outs[i]) for i, s in enumerate(self.shts)]
        self._bind()
        n = (ctypes.c_int * k)(*[c[0] for c in calls])
        args = (_lib.LmSpaceArgs * k)(*[c[1] for c in calls])
        plc = (ctypes.c_void_p * k)(*[c[3] for c in calls])
        check(self._lib.magic_sht_group_transform_to_lm_space(self._g, n, plc, args))
        return [c[2] for c in calls]


def dt_courant(dtrkc, dthkc, dt: float, dtMax: float):
    """New time step from the Courant steps of all levels (dt_courant,
    courant.f90:280-346): returns (l_new_dt, dt_new).  Host only."""
    lib = _lib.load()
    r = np.ascontiguousarray(dtrkc, dtype=np.float64)
    h = np.ascontiguousarray(dthkc, dtype=np.float64)
    if r.shape != h.shape or r.ndim != 1:
        raise ValueError("dtrkc and dthkc need the same 1-d shape")
    flag = ctypes.c_int(0)
    new = ctypes.c_double(0.0)
    check(lib.magic_sht_dt_courant(int(r.shape[0]), r.ctypes.data, h.ctypes.data, float(dt), float(dtMax),
                                   ctypes.byref(flag), ctypes.byref(new)))
    return bool(flag.value), new.value


def measure_gflops(precision: str = "fp64", device: int = 0) -> float:
    """FMA throughput of the device (GFLOP/s) for "fp64" or "fp32"."""
    lib = _lib.load()
    v = ctypes.c_double()
    check(lib.magic_sht_measure_gflops(int(device), _lib.PRECISIONS[precision], ctypes.byref(v)))
    return float(v.value)
