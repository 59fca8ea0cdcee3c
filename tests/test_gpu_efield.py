"""Polarised E-field transport, CBS cone and Raman conversion (efield.cu).

No reference semantics exist (the reference's kernels are empty), so parity
against the reference is unpinned (test_gpu_efield_oracle.py pins the kernel
to its CPU restatement); these tests check what the physics fixes:
  * the scalar limit: with S1 = S2 = sqrt(p_HG) the escaped weight equals the
    mcsub kernel's for the same medium within 3 combined standard errors;
  * reciprocity: the co-polarised channel's interference term equals its
    incoherent multiple-scattering intensity (enhancement exactly 2), the
    cross channel's lies between 1 and 2;
  * the cone: peaked at exact backscattering with the interference sum
    there, symmetric, of a width set by lambda / (2 pi l*);
  * isotropy: the incident polarisation angle does not change the
    co/cross split beyond noise;
  * batching: a setting of a batch equals a run of that setting alone with
    seed + (s << 32).
"""
import math

import numpy as np
import pytest

from nmc_gb300 import abi
import nmc_cases as cases

pytestmark = pytest.mark.gpu


def test_scalar_limit_matches_mcsub(gpu):
    from nmc_gb300 import efield

    n = 400_000
    g, mua, mus, n1, n2 = 0.9, 1.0, 100.0, 1.37, 1.0
    cfg = abi.EfieldConfig(mua=mua, mus=mus, wavelength_cm=633e-7, mu_raman=0.0, n_medium=n1, n_outside=n2,
                           n_angles=1801, cone_n=2, cone_half_angle=1e-3, sep_n=2, sep_half_width=1.0, map_n=1,
                           map_dx=1.0, depth_bins=1, depth_dz=1.0, seed=3)
    st = [abi.EfieldSetting(pol_angle=0.0, theta_in=0.0, phi_in=0.0, photons=n)]
    r = efield.run(cfg, cases.hg_amplitude_table(g), st, cone=False, maps=False, raman_depth=False)
    rd_e = r["Rd"][0] / n
    se_e = math.sqrt(max(r["Rd2"][0] / n - rd_e ** 2, 0) / n)
    rp, tp, ext = cases.mcsub_case(g=g, mua=mua, mus=mus, n1=n1, n2=n2, seed=9)
    with gpu.Engine(abi.SIM_MCSUB, 0, ext) as e:
        e.prepare_data(rp, tp)
        e.run(0, n)
        sm = e.summary()
    rd_m = sm["E"] / n
    se_m = math.sqrt(max(sm["rd_sumsq"] / n - rd_m ** 2, 0) / n)
    z = (rd_e - rd_m) / math.hypot(se_e, se_m)
    print(f"escaped weight: E-field {rd_e:.5f} +- {se_e:.5f}, mcsub {rd_m:.5f} +- {se_m:.5f}, z={z:.2f}")
    assert abs(z) <= 3.0
    # co + cross of an x-polarised input = its intensity; both inputs average the weight
    assert r["co"][0] + r["cross"][0] == pytest.approx(r["Rd"][0], rel=0.05)


@pytest.fixture(scope="module")
def cbs(gpu):
    from nmc_gb300 import efield

    cfg, S633, S700, settings = cases.cbs_case(n_settings=2, photons=1_000_000, cone_n=64, cone_half_angle=4e-4,
                                               sep_n=512, sep_half_width=0.512)
    settings[1].pol_angle = math.pi / 4
    return cfg, settings, efield.run(cfg, S633, settings, S_raman=S700)


def test_cbs_reciprocity(cbs):
    cfg, settings, r = cbs
    for s in range(2):
        assert r["interf_co"][s] == pytest.approx(r["multi_co"][s], rel=1e-5)
        e_cross = 1 + r["interf_cross"][s] / r["multi_cross"][s]
        frac_co = r["co"][s] / (r["co"][s] + r["cross"][s])
        print(f"setting {s}: Rd {r['Rd'][s] / r['photons'][s]:.4f} co fraction {frac_co:.3f} "
              f"cross enhancement {e_cross:.3f}")
        assert 1.0 < e_cross < 2.0
        assert 0.5 < frac_co < 1.0
    f0 = r["co"][0] / (r["co"][0] + r["cross"][0])
    f1 = r["co"][1] / (r["co"][1] + r["cross"][1])
    assert f0 == pytest.approx(f1, rel=0.05)  # isotropy of the medium


def test_cbs_cone_shape(cbs):
    cfg, settings, r = cbs
    cone = r["cone"][0, 0].real  # co channel interference, setting 0
    n = cfg.cone_n
    c = cone[n // 2 - 1:n // 2 + 1, n // 2 - 1:n // 2 + 1].mean()
    binned = r["interf_co"][0] - r["sep_outside"][0]
    print(f"cone centre {c:.4g}, binned interference {binned:.4g}, edge {cone[0].mean():.4g}")
    assert 0.7 * binned < c <= 1.001 * binned
    assert abs(cone[0].mean()) < 0.1 * c and abs(cone[:, 0].mean()) < 0.1 * c
    np.testing.assert_allclose(cone, cone[::-1, ::-1], atol=0.05 * c)  # q -> -q
    # half width at half maximum along theta_x vs lambda / (2 pi l*)
    th = -cfg.cone_half_angle + (np.arange(n) + 0.5) * 2 * cfg.cone_half_angle / n
    prof = cone[:, n // 2 - 1:n // 2 + 1].mean(1)
    half = th[(th > 0) & (prof < 0.5 * prof.max())]
    from nmc_gb300 import efield
    g = efield.sphere_suspension(0.5, 1.59, 1.33, 633.0, 100.0)["g"]
    lstar = 1.0 / (cfg.mus * (1 - g) + cfg.mua)
    scale = cfg.wavelength_cm / (2 * math.pi * lstar)
    print(f"HWHM {half.min() * 1e3 if half.size else float('nan'):.4f} mrad, lambda/(2 pi l*) {scale * 1e3:.4f} mrad")
    assert half.size and 0.2 * scale < half.min() < 5 * scale


def test_cbs_outputs_consistent(cbs):
    cfg, settings, r = cbs
    pvs, maps = r["pol_vs_scatt"], r["maps"]
    # intensity by scattering order and the exit maps hold the same photons
    assert pvs[0, 0].sum() + pvs[0, 1].sum() == pytest.approx(r["co"][0] + r["cross"][0], rel=1e-4)
    assert maps["Det"][0].sum() <= r["photons"][0]
    assert maps["Rd"][0].sum() <= r["Rd"][0] * (1 + 1e-5)
    assert r["raman_n"].sum() >= 0


def test_raman_conversion(gpu):
    from nmc_gb300 import efield

    cfg, S633, S700, settings = cases.cbs_case(n_settings=1, photons=200_000, mu_raman=0.5, cone_n=8, sep_n=8)
    r = efield.run(cfg, S633, settings, S_raman=S700)
    print({k: float(r[k][0]) for k in ("raman_n", "raman_Rd", "raman_co", "raman_cross", "Rd")})
    assert r["raman_n"][0] > 1000
    assert 0 < r["raman_Rd"][0] < r["raman_n"][0]
    assert r["raman_co"][0] == pytest.approx(r["raman_cross"][0], rel=0.15)  # depolarised re-emission
    assert r["raman_depth"][0].sum() > 0


def test_batched_setting_equals_alone(gpu):
    from nmc_gb300 import efield

    cfg, S633, S700, settings = cases.cbs_case(n_settings=3, photons=50_000, cone_n=8, sep_n=8)
    r = efield.run(cfg, S633, settings, S_raman=S700)
    cfg1, _, _, st1 = cases.cbs_case(n_settings=3, photons=50_000, cone_n=8, sep_n=8)
    cfg1.seed = cfg.seed + (2 << 32)
    a = efield.run(cfg1, S633, [st1[2]], S_raman=S700)
    for k in ("photons", "Rd", "co", "cross", "scatters", "raman_n"):
        assert a[k][0] == pytest.approx(r[k][2], rel=1e-9, abs=1e-9), k


def test_speckle_mutual_matches_oracle(gpu, oracle):
    # the reference's post-processing (MetalMC.m:628-742) on synthetic maps
    # and records: GPU kernel against the oracle's restatement
    from nmc_gb300 import efield

    rng = np.random.default_rng(17)
    nx, ny, kmax = 24, 20, 40
    maps = np.zeros((len(abi.EF_MAPS), nx, ny), np.float32)
    det = rng.integers(0, 60, (nx, ny)).astype(np.float32)
    maps[abi.EF_MAPS.index("Det")] = det
    for k in ("XX", "XY", "YX", "YY", "Rd"):
        maps[abi.EF_MAPS.index(k)] = rng.uniform(0, 1, (nx, ny)) * det
    for k in ("Phase0", "Phase1", "Phase2", "Phase3"):
        maps[abi.EF_MAPS.index(k)] = rng.uniform(-math.pi, math.pi, (nx, ny)) * det
    rec = np.zeros((kmax, nx, ny), abi.SPECKLE_DTYPE)
    for f in ("Phase", "Path", "Scatt", "Total"):
        rec[f] = rng.uniform(-math.pi, math.pi, rec.shape)
    for f in ("XX", "XY", "Ryx"):
        rec[f] = rng.uniform(0, 0.2, rec.shape)
    rec["XX"][0, 0, 0] = np.nan  # the reference's sanitising of non-finite values
    counts = rng.integers(0, kmax + 5, (nx, ny)).astype(np.int32)
    for lam, lc in ((633e-6, 0.05), (633e-6, 0.005)):  # lc <= 0.01 switches the envelope off
        base = rng.uniform(0, 1, maps.shape).astype(np.float32)
        got = efield.speckle_mutual(maps, rec, counts, lam, lc, out=base.copy())
        want = oracle.speckle_mutual(maps, rec, counts, lam, lc, base.copy().reshape(len(abi.EF_MAPS), -1))
        np.testing.assert_allclose(got.reshape(want.shape), want, rtol=2e-6, atol=2e-6)


def test_efield_speckle_records(gpu):
    from nmc_gb300 import efield

    cfg, S633, S700, settings = cases.cbs_case(n_settings=1, photons=20_000, cone_n=8, sep_n=8)
    cfg.speckle_max = 16
    cfg.map_n, cfg.map_dx = 64, 0.05  # outer pixels see fewer than 16 photons
    r = efield.run(cfg, S633, settings, S_raman=S700)
    spk, cnt, maps = r["speckles"][0], r["speckle_counts"][0], r["maps"]
    assert cnt.max() <= 16 and cnt.sum() > 0
    det = maps["Det"][0]
    full = (det < 16) & (det > 0)  # every arrival recorded
    assert full.any()
    k = np.arange(16)[:, None, None] < cnt[None]
    for f, m in (("XX", "XX"), ("XY", "XY"), ("Ryx", "Rd")):
        s = np.where(k, spk[f], 0).sum(0)
        np.testing.assert_allclose(s[full], maps[m][0][full], rtol=1e-4)
    np.testing.assert_array_equal(cnt[full], det[full].astype(np.int32))
