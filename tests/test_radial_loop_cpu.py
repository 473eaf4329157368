"""Host logic of the device radial-loop stage (magic_gb300/radial_loop.py),
no GPU: the Courant grid intervals of preCalculations.f90:303-310, the
lMagNlBc rule of rIter.f90:180-187 (Fortran precedence) and the boundary
flags of the levels."""
import itertools

import numpy as np
import pytest

from magic_gb300.radial_loop import RadialLoop, delx2


class _Handle:  # the loop only reads l_max at construction
    l_max = 63


def test_delx2_matches_the_reference_formulas():
    r = np.array([1.5, 1.4, 1.25, 1.0, 0.9, 0.6])
    lc = np.array([63, 63, 60, 63, 63, 10])
    dr2, dh2 = delx2(r, lc)
    assert dr2[0] == (r[0] - r[1]) ** 2 and dr2[-1] == (r[-2] - r[-1]) ** 2
    for i in range(1, len(r) - 1):
        assert dr2[i] == min(r[i - 1] - r[i], r[i] - r[i + 1]) ** 2
    np.testing.assert_array_equal(dh2, r ** 2 / (lc * (lc + 1.0)))


@pytest.mark.parametrize("ktopv,kbotv,cma,cic,rma,ric",
                         list(itertools.product((1, 2), (1, 2), (False, True), (False, True), (False, True),
                                                (False, True))))
def test_lMagNlBc_and_boundary_flags(ktopv, kbotv, cma, cic, rma, ric):
    loop = RadialLoop(_Handle(), np.linspace(1.5, 0.5, 5), cor_fac=1.0, ktopv=ktopv, kbotv=kbotv,
                      l_cond_ma=cma, l_cond_ic=cic, l_rot_ma=rma, l_rot_ic=ric)
    # rIter.f90:180-187 with l_mag_nl on: .and. binds before .or.
    top = ktopv == 1 or cma or (ktopv == 2 and rma)
    bot = kbotv == 1 or cic or (kbotv == 2 and ric)
    assert loop.lMagNlBc == (top or bot)
    assert loop.l_b_nl_cmb == (ktopv == 1 and cma)      # Namelists.f90:722-729
    assert loop.l_b_nl_icb == (kbotv == 1 and cic)      # Namelists.f90:713-720
    assert list(loop.nbc) == [ktopv, 0, 0, 0, kbotv]


def test_rejects_bad_boundaries_and_too_few_levels():
    with pytest.raises(ValueError):
        RadialLoop(_Handle(), np.linspace(1.5, 0.5, 5), cor_fac=1.0, ktopv=3)
    with pytest.raises(ValueError):
        RadialLoop(_Handle(), np.array([1.5, 0.5]), cor_fac=1.0)


class _Sized(_Handle):  # sizes _alloc reads
    n_phi_max, nlat_padded, lm_max = 8, 6, 10


@pytest.mark.parametrize("ktopv,cond", [(2, False), (1, True)])
def test_stage_buffers(ktopv, cond):
    """Every output buffer of a stage, allocated once per stage (and once for
    a captured stage): synthesis grids of the given spectra, analysis inputs
    of the get_nl levels (interior only unless lMagNlBc), analysis and get_td
    outputs at all levels, Courant steps, conducting-boundary spectra; get_td
    outputs given by the caller are used as they are."""
    import torch
    from magic_gb300._lib import GRID_SPACE_IN, GRID_SPACE_OUT, LM_SPACE_IN, LM_SPACE_OUT, TD_OUT
    n = 5
    loop = RadialLoop(_Sized(), np.linspace(1.5, 0.5, n), cor_fac=1.0, ktopv=ktopv, l_cond_ma=cond)
    spec = {k: torch.zeros((n, 10), dtype=torch.complex128) for k in GRID_SPACE_IN if k != "xi"}
    mine = torch.zeros((n, 10), dtype=torch.complex128)
    b = loop._alloc(spec, out={"dwdt": mine})
    assert set(b["grids"]) == set(GRID_SPACE_OUT) - {"xic"}
    assert all(v.shape == (n, 8, 6) and v.dtype == torch.float64 for v in b["grids"].values())
    lo, hi = loop._lohi()
    assert (lo, hi) == ((0, n) if loop.lMagNlBc else (1, n - 1))
    assert set(b["nl"]) == set(LM_SPACE_IN) and all(v.shape == (hi - lo, 8, 6) for v in b["nl"].values())
    assert set(b["lm"]) == set(LM_SPACE_OUT) and set(b["td"]) == set(TD_OUT)
    assert b["td"]["dwdt"] is mine
    assert b["dtrkc"].shape == (n,) and b["dthkc"].shape == (n,)
    assert ("cmb" in b) == loop.l_b_nl_cmb and "icb" not in b


def test_per_level_arrays():
    """Per-level arguments: numpy (and CPU tensors) pass as host pointers of
    the right type, a wrong length is refused."""
    import torch
    from magic_gb300.sht import _per_level
    a, p = _per_level([1, 2, 3], np.int32, 3, "lcut")
    assert a.dtype == np.int32 and a.flags.c_contiguous and p == a.ctypes.data
    a, p = _per_level(torch.arange(4, dtype=torch.float32), np.float64, 4, "or2")
    assert a.dtype == np.float64 and list(a) == [0.0, 1.0, 2.0, 3.0]
    assert _per_level(None, np.float64, 3, "epsc") == (None, None)
    with pytest.raises(ValueError):
        _per_level(np.ones(4), np.float64, 3, "r")


def test_capture_refuses_spectra_it_cannot_read_in_place():
    """A captured stage reads the spectra by address at every replay: host,
    non-contiguous or wrongly shaped spectra are refused before any launch."""
    import torch
    from magic_gb300.radial_loop import StageGraph
    n = 5
    loop = RadialLoop(_Sized(), np.linspace(1.5, 0.5, n), cor_fac=1.0)
    with pytest.raises(ValueError):
        StageGraph(loop, {"w": torch.zeros((n, 10), dtype=torch.complex128)})  # host tensor
