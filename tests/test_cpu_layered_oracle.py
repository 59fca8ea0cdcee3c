"""The oracle's restatement of the layered model (orc_layered_run) against
closed forms, on the CPU: a clear absorbing slab transmits exp(-mua d) of
the weight (Beer-Lambert), a clear non-absorbing slab between two index
steps transmits (1 - r)/(1 + r) (incoherent multiple reflections), weight
is conserved up to Russian roulette, and one semi-infinite layer gives the
mcsub restatement's Rd; on the reference's streams one semi-infinite layer
is, photon for photon, the reference's own mcsub kernel compiled here."""
import math

import numpy as np
import pytest


def test_beer_lambert_slab(oracle):
    n = 40_000
    r = oracle.layered([(2.0, 0.0, 0.0, 1.0, 0.3)], n, n_above=1.0, n_below=1.0, seed=3)
    t = math.exp(-2.0 * 0.3)
    se = math.sqrt(t * (1 - t) / n)
    assert r["specular"] == 0.0 and r["rd"] == 0.0
    assert abs(r["tt"] - t) <= 4 * se
    assert abs(r["A"] / n - (1 - t)) <= 4 * se


def test_fresnel_slab(oracle):
    # normal incidence; the photon never turns, so every pass is a Fresnel
    # draw: T = (1 - r)^2 / (1 - r^2) of the launched unit weight
    n = 40_000
    r = oracle.layered([(0.0, 0.0, 0.0, 1.5, 0.1)], n, n_above=1.0, n_below=1.0, seed=4)
    rf = (0.5 / 2.5) ** 2
    w0 = 1 - rf
    t = (1 - rf) / (1 + rf)  # of the incident weight, specular included
    assert abs(r["specular"] / n - rf) <= 1e-12
    p = t / w0  # probability that a launched photon leaves through the bottom
    se = math.sqrt(p * (1 - p) / n) * w0
    assert abs(r["tt"] - t) <= 4 * se
    assert abs(r["rd"] + r["tt"] - w0) <= 1e-6


def test_weight_conserved(oracle):
    n = 20_000
    lay = [(3.0, 200.0, 0.8, 1.4, 0.01), (0.3, 150.0, 0.85, 1.4, 0.2), (0.1, 100.0, 0.9, 1.44, math.inf)]
    r = oracle.layered(lay, n, nr=20, dr=0.05, nz=20, dz=0.02, seed=9)
    total = (r["specular"] + r["Rd"] + r["Tt"] + r["A"]) / n
    assert abs(total - 1.0) <= 0.01  # roulette is unbiased, not exact
    assert np.isclose(r["rd_r"].sum(), r["Rd"]) and np.isclose(r["a_z"].sum(), r["A"])
    assert np.isclose(r["a_layer"].sum(), r["A"]) and r["tt"] == 0.0


def test_one_semi_infinite_layer_is_mcsub(oracle):
    # one semi-infinite layer is the mcsub medium: the same specular weight
    # exactly, and Rd within 3 combined standard errors of the oracle's
    # mcsub restatement (independent streams)
    import nmc_cases as cases
    from nmc_gb300 import abi

    n = 50_000
    r = oracle.layered([(1.0, 100.0, 0.9, 1.37, math.inf)], n, n_above=1.0, seed=3)
    rp, tp, ext = cases.mcsub_case(seed=9)
    m = oracle.run(abi.SIM_MCSUB, rp, tp, ext=ext, n=n, tallies=False)
    rd_m = m["E"] / n
    se_m = math.sqrt(max(m["rd_sumsq"] / n - rd_m ** 2, 0) / n)
    assert r["specular"] == pytest.approx(m["S"], rel=1e-12)
    assert abs(r["rd"] - rd_m) <= 3 * math.hypot(r["rd_se"], se_m), (r["rd"], r["rd_se"], rd_m, se_m)


def test_one_layer_on_reference_streams_is_the_reference_mcsub_kernel(oracle):
    # One semi-infinite layer on the reference's generator, in MCSubKernel's
    # draw order and with its isotropic scattering (kernels.metal:252),
    # against MCSubKernel itself compiled from the reference's sources
    # (kernels.metal:59-319), photon for photon: photons (run 1..2, index
    # 0..9999) of the reference's dispatch loop.  Escaped and absorbed weight
    # per photon within 1e-3 relative (+1e-6), J(r) within 1e-3 of its total.
    if not oracle.ref_available():
        pytest.skip("reference sources not present on this machine")
    import nmc_cases as cases
    from nmc_gb300 import abi

    rp, tp, _ = cases.mcsub_case(phase=abi.PHASE_ISOTROPIC_REF, rng=abi.RNG_TAUS_REF, dr=0.002, dz=0.002)
    batch = 10_000
    ref = oracle.ref_mcsub(rp, tp, run_lo=1, run_hi=2, batch=batch, per_photon=True)
    n = 2 * batch
    lay = oracle.layered([(tp.muav[1], tp.musv[1], 0.9, rp.n1, math.inf)], n, n_above=rp.n2, nr=100, dr=0.002,
                         seed=batch, flags=abi.FLAG_LAYERED_REF_STREAMS | abi.FLAG_LAYERED_ISOTROPIC,
                         per_photon=True)
    pr, pl = ref["per_photon"].astype(np.float64), lay["per_photon"]
    esc = np.isclose(pl[:, 0], pr[:, 2], rtol=1e-3, atol=1e-6)
    ab = np.isclose(pl[:, 2], pr[:, 1], rtol=1e-3, atol=1e-6)
    both = float(np.mean(esc & ab))
    J = ref["J"][1:]  # J[ir], ir = 1..BINS (BINS = overflow) <-> rd_r[ir - 1]
    dJ = np.abs(J - lay["rd_r"]).sum() / J.sum()
    print(f"per-photon agreement {both:.5f}; E {ref['SAE'][2]:.6f} vs {lay['Rd']:.6f}; J L1 {dJ:.2e}")
    assert both >= 0.99
    assert abs(lay["Rd"] - ref["SAE"][2]) <= 1e-3 * ref["SAE"][2]
    assert abs(lay["A"] - ref["SAE"][1]) <= 1e-3 * ref["SAE"][1]
    assert dJ <= 1e-3
