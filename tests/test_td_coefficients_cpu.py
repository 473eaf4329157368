"""The operator coefficients of get_td (horizontal.f90:204-229: clm,
dTheta1..4) pinned to the Legendre functions the transforms use (the
oracle's plm_theta, plms.f90): clm(l, m) = sqrt((l+m)(l-m)/((2l-1)(2l+1)))
is the coefficient of the orthonormal three-term recurrence
    cos(theta) P_lm = clm(l+1, m) P_l+1,m + clm(l, m) P_l-1,m,
and the tabulated sin(theta) dP_lm/dtheta is
    l clm(l+1, m) P_l+1,m - (l+1) clm(l, m) P_l-1,m
(dTheta1A, dTheta1S); dTheta2A P_l+1,m - dTheta2S P_l-1,m is then
(sin(theta) d/dtheta + 2 cos(theta)) P_lm."""
import numpy as np
import pytest

from oracle import oracle as orc


def clm(l, m):
    return np.sqrt(max((l + m) * (l - m), 0) / ((2 * l - 1) * (2 * l + 1)))


@pytest.mark.parametrize("L,minc", [(12, 1), (40, 1), (33, 3)])
@pytest.mark.parametrize("theta", [0.05, 0.7, 1.5, 2.9])
def test_clm_and_dtheta_against_plm(L, minc, theta):
    p, dp = orc.plm_theta(theta, L + 1, ((L + 1) // minc) * minc, minc)
    idx, k = {}, 0
    for m in range(0, ((L + 1) // minc) * minc + 1, minc):
        for l in range(m, L + 2):
            idx[(l, m)] = k
            k += 1
    c = np.cos(theta)
    scale = np.max(np.abs(p))
    for (l, m), i in idx.items():
        if l > L:
            continue
        P = lambda ll: p[idx[(ll, m)]] if ll >= m else 0.0  # noqa: E731
        assert abs(c * P(l) - (clm(l + 1, m) * P(l + 1) + clm(l, m) * P(l - 1))) < 1e-13 * scale, (l, m)
        d1 = l * clm(l + 1, m) * P(l + 1) - (l + 1) * clm(l, m) * P(l - 1)
        assert abs(dp[i] - d1) < 1e-12 * scale * (l + 1), (l, m)
        d2 = (l + 2) * clm(l + 1, m) * P(l + 1) - (l - 1) * clm(l, m) * P(l - 1)
        assert abs(dp[i] + 2 * c * P(l) - d2) < 1e-12 * scale * (l + 1), (l, m)
