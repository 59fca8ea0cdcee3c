"""The polarised E-field kernel (efield.cu) against its CPU restatement
(oracle orc_efield_run) on the same Philox streams.

The reference's E-field kernels are empty, so this pins the CUDA kernel to
the model it implements, not to the reference:
  * short paths (mua 30 /cm, mus 100 /cm, mu_raman 2 /cm: about 29
    scatterings per photon, most of them Raman-converted): with precise math
    the kernel follows the FP32 restatement photon for photon, so every
    per-setting sum agrees to 1e-3 of the escaped weight and the counts to
    0.2 %;
  * long paths (the CBS suspension, about 5000 scatterings per photon): FP32
    and FP64 rounding separate the trajectories, so the sums agree with the
    FP64 restatement within 4 sqrt(2) standard errors of the escaped weight
    (every channel's per-photon contribution is bounded by that photon's
    escaped weight).
"""
import math

import numpy as np
import pytest

from nmc_gb300 import abi
import nmc_cases as cases

pytestmark = pytest.mark.gpu

_SUMS = ("specular", "Rd", "co", "cross", "multi_co", "multi_cross", "interf_co", "interf_cross", "sep_outside",
         "raman_Rd", "raman_co", "raman_cross")


def _short_case():
    cfg, s633, s700, st = cases.cbs_case(n_settings=8, photons=50_000, mu_raman=2.0, sep_half_width=0.05)
    cfg.mua, cfg.raman_mua = 30.0, 30.0
    cfg.flags = abi.FLAG_PRECISE_MATH
    return cfg, s633, s700, st


def test_short_paths_track_fp32_oracle(gpu, oracle):
    from nmc_gb300 import efield
    from oracle import bindings as ob

    cfg, s633, s700, st = _short_case()
    g = efield.run(cfg, s633, st, S_raman=s700, cone=True, pol_vs_scatt=False, maps=False, raman_depth=False)
    o = ob.efield(cfg, s633, st, S_raman=s700, cone=True, real_bits=32)
    np.testing.assert_array_equal(g["photons"], o["photons"])
    scale = o["Rd"] + o["raman_Rd"]
    for k in _SUMS:
        d = np.abs(g[k] - o[k])
        assert np.all(d <= 1e-3 * scale + 1e-3), (k, g[k], o[k])
    for k in ("raman_n", "scatters"):
        assert np.all(np.abs(g[k] - o[k]) <= 2e-3 * o[k] + 2), (k, g[k], o[k])
    assert np.all(o["raman_n"] > 0.2 * o["photons"]) and np.all(o["sep_outside"] > 0)


def test_long_paths_match_fp64_oracle(gpu, oracle):
    from nmc_gb300 import efield
    from oracle import bindings as ob

    n = 16_000
    cfg, s633, s700, st = cases.cbs_case(n_settings=2, photons=n)
    g = efield.run(cfg, s633, st, S_raman=s700, cone=True, pol_vs_scatt=False, maps=False, raman_depth=False)
    o = ob.efield(cfg, s633, st, S_raman=s700, cone=True, real_bits=64)
    np.testing.assert_array_equal(g["photons"], o["photons"])
    np.testing.assert_allclose(g["specular"], o["specular"], rtol=1e-5)
    se = np.sqrt(np.maximum(o["Rd2"] / n - (o["Rd"] / n) ** 2, 0) / n) * n
    for k in _SUMS[1:]:
        assert np.all(np.abs(g[k] - o[k]) <= 4 * math.sqrt(2) * se + 1e-6), (k, g[k], o[k], se)
    assert np.all(np.abs(g["raman_n"] - o["raman_n"]) <= 4 * np.sqrt(g["raman_n"] + o["raman_n"]) + 2)
    np.testing.assert_allclose(g["scatters"], o["scatters"], rtol=0.05)
