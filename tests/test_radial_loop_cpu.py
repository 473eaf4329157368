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
