"""Mie amplitudes (nmc_mie, host code): checked against an independent
evaluation of the Lorenz-Mie coefficients from scipy's spherical Bessel
functions, and against the identities every sphere obeys: the optical
theorem Q_ext = 4/x^2 Re S(0), S1(0) = S2(0), S1(pi) = -S2(pi), Q_ext = Q_sca
without absorption, the tabulated phase function's mean cosine equal to g,
and the Rayleigh limit Q_sca -> 8/3 x^4 |(m^2-1)/(m^2+2)|^2."""
import math

import numpy as np
import pytest

from nmc_gb300 import efield

special = pytest.importorskip("scipy.special")


def _scipy_q(x, m):
    n = np.arange(1, int(x + 4 * x ** (1 / 3) + 2) + 1)
    mx = m * x
    jx, jxp = special.spherical_jn(n, x), special.spherical_jn(n, x, derivative=True)
    yx, yxp = special.spherical_yn(n, x), special.spherical_yn(n, x, derivative=True)
    jm, jmp = special.spherical_jn(n, mx), special.spherical_jn(n, mx, derivative=True)
    psi_x, dpsi_x = x * jx, jx + x * jxp
    psi_m, dpsi_m = mx * jm, jm + mx * jmp
    h, hp = jx + 1j * yx, jxp + 1j * yxp
    xi, dxi = x * h, h + x * hp
    a = (m * psi_m * dpsi_x - psi_x * dpsi_m) / (m * psi_m * dxi - xi * dpsi_m)
    b = (psi_m * dpsi_x - m * psi_x * dpsi_m) / (psi_m * dxi - m * xi * dpsi_m)
    qs = 2 / x ** 2 * np.sum((2 * n + 1) * (abs(a) ** 2 + abs(b) ** 2))
    qe = 2 / x ** 2 * np.sum((2 * n + 1) * (a + b).real)
    return qe, qs


@pytest.mark.parametrize("x,m", [(0.5, 1.33), (3.0, 1.55), (2 * math.pi * 1.33 * 0.5 / 0.633, 1.59 / 1.33),
                                 (2 * math.pi * 1.33 * 0.5 / 0.700, 1.59 / 1.33), (20.0, 1.2)])
def test_mie_against_independent_bessel_evaluation(x, m):
    r = efield.mie(x, complex(m, 0.0))
    qe, qs = _scipy_q(x, m)
    assert r["q_ext"] == pytest.approx(qe, rel=1e-9)
    assert r["q_sca"] == pytest.approx(qs, rel=1e-9)


def test_mie_identities():
    x, m = 2 * math.pi * 1.33 * 0.5 / 0.633, 1.59 / 1.33  # the C5 spheres
    r = efield.mie(x, complex(m, 0.0), 1801)
    S1, S2, th = r["S1"], r["S2"], r["theta"]
    assert r["q_ext"] == pytest.approx(r["q_sca"], rel=1e-9)  # no absorption
    assert r["q_ext"] == pytest.approx(4 / x ** 2 * S1[0].real, rel=1e-5)  # optical theorem
    assert abs(S1[0] - S2[0]) <= 1e-5 * abs(S1[0])
    assert abs(S1[-1] + S2[-1]) <= 1e-4 * max(abs(S1[-1]), 1e-6)
    p = 0.5 * (abs(S1) ** 2 + abs(S2) ** 2) * np.sin(th)
    g_tab = np.trapezoid(p * np.cos(th), th) / np.trapezoid(p, th)
    assert g_tab == pytest.approx(r["g"], abs=2e-4)
    assert 0.85 < r["g"] < 0.95


def test_mie_rayleigh_limit_and_absorption():
    x, m = 0.02, 1.5
    r = efield.mie(x, complex(m, 0.0), 3)
    k = (m * m - 1) / (m * m + 2)
    assert r["q_sca"] == pytest.approx(8 / 3 * x ** 4 * k * k, rel=1e-3)
    a = efield.mie(2.0, complex(1.5, 0.1), 181)
    assert a["q_ext"] > a["q_sca"] > 0  # an absorbing sphere extinguishes more than it scatters


def test_mie_rejects_bad_input():
    with pytest.raises(Exception):
        efield.mie(-1.0, complex(1.5, 0.0))
    with pytest.raises(Exception):
        efield.mie(1.0, complex(1.5, -0.1))
