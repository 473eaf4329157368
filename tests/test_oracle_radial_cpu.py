"""Known answers of the oracle's restatements of the radial-loop pieces that
have closed forms (no GPU)."""
import numpy as np
import pytest

from oracle import oracle as orc


@pytest.mark.parametrize("N,P", [(48, 96), (96, 192)])
@pytest.mark.parametrize("LFfac", [1.0, 2.5])
def test_lorentz_torque_known_answers(N, P, LFfac):
    """get_lorentz_torque (outRot.f90:423-483) is LFfac 2 pi / n_phi times a
    Gauss-quadrature sum over the sphere: for br = bp = 1 it is
    LFfac 2 pi * 2, for br = bp = cos(theta) LFfac 2 pi * 2/3, and the Grenoble
    term -b0 cos(theta) bp with bp = cos(theta) adds -b0 LFfac 2 pi * 2/3
    (the quadrature is exact for these polynomials)."""
    _, c = orc._row_trig(N)
    one = np.ones((P, N))
    cg = np.broadcast_to(c, (P, N))
    assert abs(orc.lorentz_torque(one, one, N, LFfac) - LFfac * 4.0 * np.pi) < 1e-12
    assert abs(orc.lorentz_torque(cg, cg, N, LFfac) - LFfac * 4.0 * np.pi / 3.0) < 1e-12
    b0 = 0.7
    got = orc.lorentz_torque(np.zeros((P, N)), cg, N, LFfac, b0)
    assert abs(got + b0 * LFfac * 4.0 * np.pi / 3.0) < 1e-12
    # only the phi average of br bp matters: a cos(phi) modulation of bp integrates to 0
    phi = 2.0 * np.pi * np.arange(P) / P
    assert abs(orc.lorentz_torque(one, np.cos(phi)[:, None] * one, N, LFfac)) < 1e-12
