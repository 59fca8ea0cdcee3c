"""The oracle's restatement of the polarised E-field model (orc_efield_run)
on the CPU:
  * the scalar limit: with S1 = S2 = sqrt(p_HG) the escaped weight equals the
    oracle's mcsub restatement for the same medium within 3 combined
    standard errors;
  * FP32 and FP64 follow the same photons on short paths, so their sums agree
    to 1e-3 of the escaped weight;
  * reciprocity: the co-polarised interference term equals the co-polarised
    multiple-scattering intensity.
"""
import math

import numpy as np
import pytest

from nmc_gb300 import abi
import nmc_cases as cases


def test_scalar_limit_matches_mcsub(oracle):
    n = 20_000
    g, mua, mus, n1, n2 = 0.9, 1.0, 100.0, 1.37, 1.0
    cfg = abi.EfieldConfig(mua=mua, mus=mus, wavelength_cm=633e-7, mu_raman=0.0, n_medium=n1, n_outside=n2,
                           n_angles=1801, cone_n=2, cone_half_angle=1e-3, sep_n=2, sep_half_width=1.0, map_n=1,
                           map_dx=1.0, depth_bins=1, depth_dz=1.0, seed=3)
    st = [abi.EfieldSetting(pol_angle=0.0, theta_in=0.0, phi_in=0.0, photons=n)]
    r = oracle.efield(cfg, cases.hg_amplitude_table(g), st)
    rd_e = r["Rd"][0] / n
    se_e = math.sqrt(max(r["Rd2"][0] / n - rd_e ** 2, 0) / n)
    rp, tp, ext = cases.mcsub_case(g=g, mua=mua, mus=mus, n1=n1, n2=n2, seed=9)
    m = oracle.run(abi.SIM_MCSUB, rp, tp, ext=ext, n=n, tallies=False)
    rd_m = m["E"] / n
    se_m = math.sqrt(max(m["rd_sumsq"] / n - rd_m ** 2, 0) / n)
    assert abs(rd_e - rd_m) <= 3 * math.hypot(se_e, se_m), (rd_e, se_e, rd_m, se_m)
    assert r["co"][0] + r["cross"][0] == pytest.approx(r["Rd"][0], rel=0.05)


def test_fp32_follows_fp64_on_short_paths(oracle):
    cfg, s633, s700, st = cases.cbs_case(n_settings=4, photons=20_000, mu_raman=2.0, sep_half_width=0.05)
    cfg.mua, cfg.raman_mua = 30.0, 30.0
    a = oracle.efield(cfg, s633, st, S_raman=s700, cone=True, real_bits=64)
    b = oracle.efield(cfg, s633, st, S_raman=s700, cone=True, real_bits=32)
    scale = a["Rd"] + a["raman_Rd"]
    for k in abi.EF_FIELDS:
        if k in ("photons", "raman_n", "scatters", "Rd2"):
            continue
        assert np.all(np.abs(a[k] - b[k]) <= 1e-3 * scale + 1e-3), (k, a[k], b[k])
    np.testing.assert_array_equal(a["photons"], b["photons"])
    assert np.all(np.abs(a["raman_n"] - b["raman_n"]) <= 2e-3 * a["raman_n"] + 2)
    # reciprocity: the time-reversed partner of a co-polarised path has the same amplitude
    np.testing.assert_allclose(a["interf_co"], a["multi_co"], rtol=1e-9)
    assert np.all(a["interf_cross"] < a["multi_cross"])


def test_separation_overflow_shrinks_with_the_histogram_width(oracle):
    # CBS partners farther apart than the separation histogram reaches are
    # counted in sep_outside: almost all of the co-polarised interference for
    # a tiny histogram, less as it widens, almost none once it spans the
    # walk (mua 10 /cm: paths of ~0.1 cm)
    out = []
    for w in (1e-5, 0.005, 0.05, 0.5):
        cfg, s633, _, st = cases.cbs_case(n_settings=1, photons=5_000, mu_raman=0.0, sep_half_width=w)
        cfg.mua = 10.0
        r = oracle.efield(cfg, s633, st, cone=True)
        out.append(r["sep_outside"][0])
        interf = r["interf_co"][0]
    assert out[0] >= 0.99 * interf
    assert all(a > b for a, b in zip(out, out[1:]))
    assert out[-1] <= 1e-3 * interf
