"""The oracle pinned against known answers and against the reference itself.

Known answers: Random123's Philox4x32-10 test vectors; analytic Fresnel and
phase-function identities.  Reference pins (where the reference sources are
present): the reference kernels compiled from their own files behind the
host shim, run on the same photon streams (the reference's generator).
"""
import math

import numpy as np
import pytest

from nmc_gb300 import abi
import nmc_cases as cases


# Random123 kat_vectors, philox4x32 10 rounds
PHILOX_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,want", PHILOX_KAT)
def test_philox_known_answers(oracle, ctr, key, want):
    assert tuple(int(x) for x in oracle.philox(ctr, key)) == want


def test_philox_uniforms_open_interval(oracle):
    u = oracle.uniforms(abi.ext_defaults(seed=7), abi.SIM_MCXYZ, 123, 4096)
    assert (u > 0).all() and (u < 1).all()
    k = (u * 2 ** 24 - 1) / 2
    assert np.allclose(k, np.round(k))  # u = (2k+1) 2^-24 exactly
    assert abs(u.mean() - 0.5) < 0.02


def test_reference_generator_matches_reference(oracle):
    if not oracle.ref_available():
        pytest.skip("reference sources not present")
    ext = abi.ext_defaults(rng=abi.RNG_TAUS_REF)
    # photon (run 1, index 5): seeds of kernels.metal:339-343 with numRuns = 2
    nr, idx = 2, 5
    s1 = ((nr ^ (idx * 2654435761)) + 12345) & 0xFFFFFFFF
    s2 = ((nr * 1103515245) ^ (idx * 1013904223)) & 0xFFFFFFFF
    s3 = (((idx ^ nr) * 1664525) + 1013904223) & 0xFFFFFFFF
    ref = oracle.ref_taus(s1, s2, s3, 16)
    ours = oracle.uniforms(ext, abi.SIM_MCXYZ, idx, 16)
    assert np.array_equal(ref.astype(np.float64), ours)


def test_fresnel_limits(oracle):
    n1, n2 = 1.37, 1.0
    r, ca2 = oracle.rfresnel(n1, n2, 1.0)  # normal incidence
    assert r == pytest.approx(((n2 - n1) / (n2 + n1)) ** 2, rel=1e-12) and ca2 == 1.0
    r, ca2 = oracle.rfresnel(n1, n2, 1e-7)  # grazing
    assert r == 1.0 and ca2 == 0.0
    r, _ = oracle.rfresnel(n1, n2, math.cos(math.asin(1 / n1) + 0.01))  # beyond the critical angle
    assert r == 1.0
    r, _ = oracle.rfresnel(1.4, 1.4, 0.3)  # matched
    assert r == 0.0
    r, ca2 = oracle.rfresnel(1.0, 1.5, 0.7)  # general: compare with s/p average
    ci, ct = 0.7, ca2
    rs = ((1.0 * ci - 1.5 * ct) / (1.0 * ci + 1.5 * ct)) ** 2
    rpp = ((1.0 * ct - 1.5 * ci) / (1.0 * ct + 1.5 * ci)) ** 2
    assert r == pytest.approx(0.5 * (rs + rpp), rel=1e-10)


@pytest.mark.parametrize("g", [0.0, 0.5, 0.9, -0.3])
def test_hg_mean_cosine_is_g(oracle, g):
    u = (np.arange(200000) + 0.5) / 200000
    c = np.array([oracle.hg_costheta(g, x) for x in u])
    assert c.mean() == pytest.approx(g, abs=2e-4)
    assert c.min() >= -1 - 1e-12 and c.max() <= 1 + 1e-12


def test_two_term_reduces_to_hg_at_alpha_half(oracle):
    for g in (0.9, 0.3):
        for u in (0.01, 0.3, 0.77, 0.999):
            tt = oracle.tt_costheta(g, 0.5, 0.3, 0.5, 1.0, 0.5, u)  # forward branch
            assert tt == pytest.approx(oracle.hg_costheta(g, u), abs=1e-12)
        # backward branch samples HG(gb) and negates it (kernels.metal:1064-1068)
        tt = oracle.tt_costheta(0.9, 0.5, g, 0.5, 0.0, 0.5, 0.4)
        assert tt == pytest.approx(-oracle.hg_costheta(g, 0.4), abs=1e-12)


def test_mcsub_weight_conservation_and_specular(oracle):
    rp, tp, ext = cases.mcsub_case()
    n = 5000
    r = oracle.run(abi.SIM_MCSUB, rp, tp, ext=ext, n=n)
    # roulette conserves weight in expectation only (kernels.metal:289-294)
    assert (r["S"] + r["A"] + r["E"]) / n == pytest.approx(1.0, abs=1e-4)
    assert r["S"] / n == pytest.approx(((1.37 - 1.0) / 2.37) ** 2, rel=1e-6)  # kernels.metal:118-120
    assert r["J"].sum() == pytest.approx(r["E"], rel=1e-9)
    assert r["F"].sum() == pytest.approx(r["A"], rel=1e-9)


def test_mcsub_oracle_replays_reference_per_photon(oracle):
    """With the reference's generator and isotropic sampling, the FP64 oracle
    follows each reference photon (escaped and absorbed weight)."""
    if not oracle.ref_available():
        pytest.skip("reference sources not present")
    rp, tp, _ = cases.mcsub_case()
    ext = abi.ext_defaults(rng=abi.RNG_TAUS_REF, phase=abi.PHASE_ISOTROPIC_REF)  # BINS 101, dr 0.002
    r = oracle.ref_mcsub(rp, tp, 1, 2, 10000, per_photon=True)
    o = oracle.run(abi.SIM_MCSUB, rp, tp, ext=ext, n=20000, trace=True)
    pp = r["per_photon"]
    ok = (np.abs(pp[:, 2] - o["recs"]["detected"]) < 1e-5) & (np.abs(pp[:, 1] - o["recs"]["absorbed"]) < 1e-5)
    assert ok.mean() >= 0.999
    assert np.allclose(r["SAE"], [o["S"], o["A"], o["E"]], rtol=1e-5)
    assert np.abs(r["J"] - o["J"]).sum() <= 1e-3 * r["J"].sum()


def test_mcxyz_fp32_oracle_replays_reference(oracle):
    """FP32 restatement with the reference's generator against the reference
    on the notebook's homogeneous cube (scaled to 60^3)."""
    if not oracle.ref_available():
        pytest.skip("reference sources not present")
    rp, tp, v, ext = cases.homogeneous_case(N=60, d=0.02, rng=abi.RNG_TAUS_REF)
    r = oracle.ref_mcxyz(rp, tp, v, 1, 1, 4000, per_photon=True)
    o = oracle.run(abi.SIM_MCXYZ, rp, tp, v, ext=ext, n=4000, trace=True, real_bits=32)
    d = np.abs(r["per_photon"] - o["recs"]["detected"])
    assert np.mean(d < 1e-5) >= 0.8
    assert o["rd_sum"] == pytest.approx(r["rd_slots"].sum(), rel=0.02)


def test_two_term_fp32_oracle_replays_reference(oracle):
    """MCXYZKernelTT (kernels.metal:757-1118): the FP32 restatement with the
    reference's generator, seeded from run 1 as the reference's TT kernel
    is, against the reference kernel itself on a 60^3 skin-vessel map with
    two-term tissues (g_f 0.9, g_b 0.3, a 0.5, C 0.9)."""
    if not oracle.ref_available():
        pytest.skip("reference sources not present")
    rp, tp, v, _ = cases.skin_vessel_case(N=60, d=0.005)
    rp.mckernelflag = abi.SIM_MCXYZ_TT
    rp.boundaryflag = 1  # the reference's two-term Rd2D index is unclamped (kernels.metal:984)
    for t in range(1, 5):
        tp.gf[t], tp.af[t], tp.gb[t], tp.ab[t], tp.CC[t] = 0.9, 0.5, 0.3, 0.5, 0.9
    ext = abi.ext_defaults(rng=abi.RNG_TAUS_REF, flags=abi.FLAG_TT_REPLAY_RUN1)
    r = oracle.ref_mcxyz_tt(rp, tp, v, 1, 1, 4000, replay_run1=True, per_photon=True)
    o = oracle.run(abi.SIM_MCXYZ_TT, rp, tp, v, ext=ext, n=4000, trace=True, real_bits=32)
    d = np.abs(r["per_photon"] - o["recs"]["detected"])
    print(f"two-term per-photon agreement {np.mean(d < 1e-5):.3f}, Rd ref {r['rd_slots'].sum() / 4000:.5f} "
          f"oracle {o['rd_sum'] / 4000:.5f}")
    assert np.mean(d < 1e-5) >= 0.8
    assert o["rd_sum"] == pytest.approx(r["rd_slots"].sum(), rel=0.02)


@pytest.mark.parametrize("mode", list(cases.PARITY_MODES))
def test_fp32_oracle_replays_reference_in_every_mode(oracle, mode):
    """The oracle's FP32 restatement against the reference's MCXYZKernel
    compiled here, on the reference's own streams, over its launch modes
    (kernels.metal:366-463), boundary modes (:646-672) and detection modes
    (:556-637), and an odd, non-cubic grid: photon for photon on the detected
    weight, and the total Rd."""
    if not oracle.ref_available():
        pytest.skip("reference sources not present")
    rp, tp, v = cases.modes_medium(**cases.PARITY_MODES[mode])
    n = 4000
    ext = abi.ext_defaults(rng=abi.RNG_TAUS_REF, photons_per_dispatch=n)
    r = oracle.ref_mcxyz(rp, tp, v, 1, 1, n, per_photon=True)
    o = oracle.run(abi.SIM_MCXYZ, rp, tp, v, ext=ext, n=n, trace=True, real_bits=32)
    d = np.abs(r["per_photon"] - o["recs"]["detected"])
    agree = np.mean(d <= 1e-5 + 1e-4 * np.abs(r["per_photon"]))
    rd_ref, rd_orc = r["rd_slots"].sum() / n, o["rd_sum"] / n
    print(f"{mode}: per-photon agreement {agree:.4f}, Rd reference {rd_ref:.5f} oracle {rd_orc:.5f}")
    assert agree >= 0.8
    assert abs(rd_orc - rd_ref) <= 0.02 * rd_ref + 1e-4


@pytest.mark.parametrize("mode", [m for m in cases.PARITY_MODES if m != "gaussian-beam"])
def test_two_term_fp32_oracle_replays_reference_in_every_mode(oracle, mode):
    """MCXYZKernelTT (kernels.metal:757-1118, whose launch has no Gaussian
    branch) compiled here against the oracle's FP32 restatement, in each
    launch and detection mode, with boundaryflag 1: beyond the grid's sides
    the reference writes Rd2D at an unclamped index (kernels.metal:984)."""
    if not oracle.ref_available():
        pytest.skip("reference sources not present")
    kw = dict(cases.PARITY_MODES[mode])
    kw["boundaryflag"] = 1
    rp, tp, v = cases.modes_medium(**kw)
    rp.mckernelflag = abi.SIM_MCXYZ_TT
    for t in range(1, 4):
        tp.gf[t], tp.af[t], tp.gb[t], tp.ab[t], tp.CC[t] = 0.9, 0.5, 0.3, 0.5, 0.9
    n = 4000
    ext = abi.ext_defaults(rng=abi.RNG_TAUS_REF, photons_per_dispatch=n, flags=abi.FLAG_TT_REPLAY_RUN1)
    r = oracle.ref_mcxyz_tt(rp, tp, v, 1, 1, n, replay_run1=True, per_photon=True)
    o = oracle.run(abi.SIM_MCXYZ_TT, rp, tp, v, ext=ext, n=n, trace=True, real_bits=32)
    d = np.abs(r["per_photon"] - o["recs"]["detected"])
    agree = np.mean(d <= 1e-5 + 1e-4 * np.abs(r["per_photon"]))
    rd_ref, rd_orc = r["rd_slots"].sum() / n, o["rd_sum"] / n
    print(f"two-term {mode}: per-photon agreement {agree:.4f}, Rd reference {rd_ref:.5f} oracle {rd_orc:.5f}")
    assert agree >= 0.8
    assert abs(rd_orc - rd_ref) <= 0.02 * rd_ref + 1e-4


def test_notebook_rd_reproduced_by_reference_build(oracle):
    """example0.ipynb cell 5 records Rd = 0.26601276 for 1e5 photons of its
    homogeneous cube (Metal, AMD Radeon Pro 5500 XT).  The reference kernel
    compiled here on the same photon streams reproduces it."""
    if not oracle.ref_available():
        pytest.skip("reference sources not present")
    rp, tp, v, _ = cases.homogeneous_case(N=200, d=0.02)
    r = oracle.ref_mcxyz(rp, tp, v, 1, 10, 10000)
    rd = r["rd_slots"].sum() / 1e5
    assert rd == pytest.approx(0.26601276, abs=5e-4)  # SE of the run is ~1e-3


def test_fp64_oracle_agrees_across_generators(oracle):
    """Same physics, different streams: Philox and the reference generator
    give the same Rd within 3 standard errors (FP64)."""
    rp, tp, v, _ = cases.skin_vessel_case(N=40)
    out = []
    for rng in (abi.RNG_PHILOX, abi.RNG_TAUS_REF):
        ext = abi.ext_defaults(rng=rng)
        r = oracle.run(abi.SIM_MCXYZ, rp, tp, v, ext=ext, n=20000)
        m = r["rd_sum"] / 20000
        se = math.sqrt((r["rd_sumsq"] / 20000 - m * m) / 20000)
        out.append((m, se))
    (m1, s1), (m2, s2) = out
    assert abs(m1 - m2) <= 3 * math.hypot(s1, s2)


def test_invalid_tissue_map_rejected(oracle):
    rp, tp, v, ext = cases.skin_vessel_case(N=16)
    v = v.copy()
    v[17] = 40  # > Ntiss - 1
    with pytest.raises(RuntimeError):
        oracle.run(abi.SIM_MCXYZ, rp, tp, v, ext=ext, n=10)
