"""Layered media (layered.cu).  No reference semantics exist for more than
one layer (MAXLAYERS is declared, definitions.h:24, but unused).  The
engine follows the oracle's CPU restatement of the same model on the same
Philox streams, photon for photon, and the checks the physics fixes hold:
one semi-infinite layer equals the mcsub kernel; a layer split in two equals
the whole; a clear absorbing slab follows Beer-Lambert; a clear
non-absorbing slab follows the Fresnel multiple-reflection sums; weight is
conserved."""
import math

import numpy as np
import pytest

from nmc_gb300 import abi
import nmc_cases as cases

pytestmark = pytest.mark.gpu

SKIN3 = cases.LAYERED_SKIN3
SLABS = [(0.5, 80.0, 0.9, 1.33, 0.05), (2.0, 30.0, 0.0, 1.5, 0.02), (0.2, 120.0, 0.7, 1.37, 0.1)]


@pytest.mark.parametrize("layers,n_below", [(SKIN3, 1.0), (SLABS, 1.2)], ids=["skin3", "finite_slabs"])
def test_layered_follows_the_oracle(gpu, oracle, layers, n_below):
    # same Philox streams: the FP32 engine and the FP64 restatement follow the
    # same photons, so their sums agree far inside the statistical error
    from nmc_gb300 import layered

    n = 200_000
    kw = dict(n_above=1.0, n_below=n_below, nr=40, dr=0.02, nz=40, dz=0.01, seed=5, first=1000)
    g = layered.run(layers, n, **kw)
    o = oracle.layered(layers, n, **kw)
    print(f"Rd {g['rd']:.6f} / {o['rd']:.6f}, Tt {g['tt']:.6f} / {o['tt']:.6f}, A {g['A'] / n:.6f} / "
          f"{o['A'] / n:.6f}, interactions {g['interactions']:.0f} / {o['interactions']:.0f}")
    assert g["photons"] == o["photons"] == n
    assert abs(g["specular"] - o["specular"]) <= 1e-9 * n
    for k in ("rd", "tt"):
        assert abs(g[k] - o[k]) <= 0.05 * g[k + "_se"] + 1e-9
    assert abs(g["A"] - o["A"]) <= 1e-3 * o["A"]
    assert abs(g["interactions"] - o["interactions"]) <= 1e-3 * o["interactions"]
    np.testing.assert_allclose(g["a_layer"], o["a_layer"], rtol=2e-3, atol=1e-6 * n)
    for t in ("rd_r", "tt_r", "a_z"):
        assert np.abs(g[t] - o[t]).sum() <= 5e-3 * max(o[t].sum(), 1e-9) + 1e-6 * n, t
    # bin by bin: within 3 sigma of the oracle, each bin's error from the
    # spread of the oracle's 8 batches, for bins photons reach in most batches
    B = 8
    ob = [oracle.layered(layers, n // B, **{**kw, "first": kw["first"] + b * (n // B)}) for b in range(B)]
    for t in ("rd_r", "tt_r", "a_z"):
        orc = np.stack([r[t] for r in ob])
        se = np.sqrt(B) * orc.std(0, ddof=1)
        live = ((orc != 0).sum(0) >= 5) & (se > 0)
        if live.any():
            z = np.abs(g[t][live] - orc.sum(0)[live]) / se[live]
            print(f"{t}: {int(live.sum())} bins, max |z| {z.max():.2f}")
            assert z.max() <= 3.0, t


def test_one_layer_on_reference_streams_follows_the_pinned_oracle(gpu, oracle):
    # One semi-infinite layer on the reference's generator in MCSubKernel's
    # draw order, with its isotropic scattering: the oracle's restatement of
    # this run is, photon for photon, MCSubKernel compiled from the reference
    # (tests/test_cpu_layered_oracle.py); the GPU follows the same photons.
    # Totals within 1e-3, Rd(r) within 1e-3 of its total (L1).
    from nmc_gb300 import layered

    rp, tp, _ = cases.mcsub_case(phase=abi.PHASE_ISOTROPIC_REF, rng=abi.RNG_TAUS_REF, dr=0.002, dz=0.002)
    batch, n = 10_000, 100_000
    lay = [(tp.muav[1], tp.musv[1], 0.9, rp.n1, math.inf)]
    kw = dict(n_above=rp.n2, nr=100, dr=0.002, seed=batch, first=batch,
              flags=abi.FLAG_LAYERED_REF_STREAMS | abi.FLAG_LAYERED_ISOTROPIC)
    g = layered.run(lay, n, **kw)
    o = oracle.layered(lay, n, **kw)
    dJ = np.abs(g["rd_r"] - o["rd_r"]).sum() / o["rd_r"].sum()
    print(f"Rd {g['rd']:.6f} / {o['rd']:.6f}, A {g['A'] / n:.6f} / {o['A'] / n:.6f}, Rd(r) L1 {dJ:.2e}")
    assert abs(g["Rd"] - o["Rd"]) <= 1e-3 * o["Rd"]
    assert abs(g["A"] - o["A"]) <= 1e-3 * o["A"]
    assert abs(g["interactions"] - o["interactions"]) <= 1e-3 * o["interactions"]
    assert dJ <= 1e-3


def test_single_layer_equals_mcsub(gpu):
    from nmc_gb300 import layered

    n = 400_000
    r = layered.run([(1.0, 100.0, 0.9, 1.37, math.inf)], n, n_above=1.0, seed=4)
    rp, tp, ext = cases.mcsub_case(g=0.9, seed=8)
    with gpu.Engine(abi.SIM_MCSUB, 0, ext) as e:
        e.prepare_data(rp, tp)
        e.run(0, n)
        sm = e.summary()
    rd_m = sm["E"] / n
    se_m = math.sqrt(max(sm["rd_sumsq"] / n - rd_m ** 2, 0) / n)
    z = (r["rd"] - rd_m) / math.hypot(r["rd_se"], se_m)
    print(f"Rd layered {r['rd']:.5f} +- {r['rd_se']:.5f}, mcsub {rd_m:.5f} +- {se_m:.5f}, z={z:.2f}")
    assert abs(z) <= 3.0
    assert r["specular"] / n == pytest.approx(sm["S"] / n, rel=1e-5)


def test_split_layer_equals_whole(gpu):
    from nmc_gb300 import layered

    n = 400_000
    whole = layered.run([(0.5, 80.0, 0.8, 1.4, 0.1), (2.0, 50.0, 0.7, 1.4, math.inf)], n, seed=1)
    split = layered.run([(0.5, 80.0, 0.8, 1.4, 0.04), (0.5, 80.0, 0.8, 1.4, 0.06), (2.0, 50.0, 0.7, 1.4, math.inf)],
                        n, seed=2)
    z = (whole["rd"] - split["rd"]) / math.hypot(whole["rd_se"], split["rd_se"])
    print(f"Rd whole {whole['rd']:.5f} split {split['rd']:.5f} z={z:.2f}")
    assert abs(z) <= 3.0
    a_top = split["a_layer"][0] + split["a_layer"][1]
    assert a_top == pytest.approx(whole["a_layer"][0], rel=0.03)


def test_beer_lambert_slab(gpu):
    from nmc_gb300 import layered

    n, mua, d = 200_000, 2.0, 0.3
    r = layered.run([(mua, 0.0, 0.0, 1.0, d)], n, n_above=1.0, n_below=1.0, seed=3)
    p = math.exp(-mua * d)
    se = math.sqrt(p * (1 - p) / n)
    print(f"Tt {r['tt']:.5f} vs {p:.5f}")
    assert abs(r["tt"] - p) <= 4 * se
    assert r["rd"] == 0.0


def test_fresnel_slab(gpu):
    from nmc_gb300 import layered

    n, ns = 200_000, 1.5
    r = layered.run([(0.0, 0.0, 0.0, ns, 1.0)], n, seed=5)
    R = ((ns - 1) / (ns + 1)) ** 2
    tt, rd = (1 - R) / (1 + R), (1 - R) * R / (1 + R)  # escape after an even / odd number of internal reflections
    print(f"Tt {r['tt']:.5f} vs {tt:.5f}, Rd {r['rd']:.5f} vs {rd:.5f}")
    assert abs(r["tt"] - tt) <= 4 * math.sqrt(tt * (1 - tt) / n)
    assert abs(r["rd"] - rd) <= 4 * math.sqrt(rd * (1 - rd) / n) + 1e-4


def test_weight_conservation_and_tallies(gpu):
    from nmc_gb300 import layered

    n = 200_000
    lay = [(0.3, 120.0, 0.9, 1.4, 0.02), (5.0, 200.0, 0.85, 1.37, 0.05), (0.5, 90.0, 0.8, 1.45, 0.3)]
    r = layered.run(lay, n, n_above=1.0, n_below=1.33, a_rz=True, seed=6)
    total = (r["specular"] + r["Rd"] + r["Tt"] + r["A"]) / n
    print(f"S+Rd+Tt+A = {total:.5f}")
    assert total == pytest.approx(1.0, abs=2e-3)  # roulette keeps weight in expectation
    assert r["a_layer"].sum() == pytest.approx(r["A"], rel=1e-9)
    assert r["a_z"].sum() == pytest.approx(r["A"], rel=1e-6)
    assert r["a_rz"].sum() == pytest.approx(r["A"], rel=1e-6)
    assert r["rd_r"].sum() == pytest.approx(r["Rd"], rel=1e-6)
    assert r["tt_r"].sum() == pytest.approx(r["Tt"], rel=1e-6)


def test_layer_adjoint_matches_crn_finite_differences(gpu):
    # per-layer pMC gradients of a loss on Rd(r) and Tt(r) against central
    # differences with common random numbers, 16 batches of 40k photons
    from nmc_gb300 import layered

    lay = [[0.5, 120.0, 0.9, 1.4, 0.02], [3.0, 150.0, 0.85, 1.4, 0.05], [1.0, 80.0, 0.8, 1.4, 0.2]]
    nr, B, nb = 60, 16, 40_000
    rng = np.random.default_rng(9)
    G_rd = rng.uniform(0.5, 1.5, nr + 1).astype(np.float32)
    G_tt = rng.uniform(0.0, 1.0, nr + 1).astype(np.float32)
    loss = lambda r: float(G_rd.astype(np.float64) @ r["rd_r"] + G_tt.astype(np.float64) @ r["tt_r"])  # noqa: E731
    pm = np.zeros((B, 3, 3))
    fd = np.zeros((B, 3, 3))
    for b in range(B):
        a = layered.adjoint(lay, nb, G_rd, G_tt, nr=nr, dr=0.005, first=b * nb, seed=2)
        pm[b] = np.stack([a["grad_mua"], a["grad_mus"], a["grad_g"]])
    for p, idx, rel in ((0, 0, 0.02), (1, 1, 0.02), (2, 2, None)):
        for l in range(3):
            base = lay[l][idx]
            h = 0.01 if rel is None else rel * base
            sides = []
            for sgn in (1, -1):
                l2 = [list(q) for q in lay]
                l2[l][idx] = base + sgn * h
                sides.append(np.array([loss(layered.run(l2, nb, nr=nr, dr=0.005, first=b * nb, seed=2))
                                       for b in range(B)]))
            fd[:, p, l] = (sides[0] - sides[1]) / (2 * h)
    for p, name in enumerate(("mua", "mus", "g")):
        d = pm[:, p] - fd[:, p]
        t = d.mean(0) / (d.std(0, ddof=1) / np.sqrt(B))
        print(f"{name}: pmc {pm[:, p].mean(0)} fd {fd[:, p].mean(0)} t {t}")
        if name == "mua":
            P, F = pm[:, p].mean(0), fd[:, p].mean(0)
            assert np.all(np.abs(P - F) <= np.maximum(4.5 * d.std(0, ddof=1) / np.sqrt(B), 1e-3 * np.abs(F)))
        else:
            assert np.all(np.abs(t) <= 4.5)


def test_layer_adjoint_satisfies_the_scaling_identity(gpu):
    # one semi-infinite layer has no length scale: total Rd is unchanged when
    # mua and mus are scaled alike, so mua dRd/dmua + mus dRd/dmus = 0 (the
    # pathwise and likelihood-ratio parts cancel, within their statistics)
    from nmc_gb300 import layered

    lay = [(1.0, 100.0, 0.9, 1.4, math.inf)]
    nr, B, nb = 40, 8, 200_000
    G = np.ones(nr + 1, np.float32)
    a, s = [], []
    for b in range(B):
        r = layered.adjoint(lay, nb, G, None, nr=nr, dr=0.05, first=b * nb, seed=4)
        a.append(1.0 * r["grad_mua"][0] / nb)
        s.append(100.0 * r["grad_mus"][0] / nb)
    a, s = np.array(a), np.array(s)
    tot = a + s
    se = tot.std(ddof=1) / np.sqrt(B)
    print(f"mua . dRd/dmua {a.mean():.5f}, mus . dRd/dmus {s.mean():.5f}, sum {tot.mean():.2e} +- {se:.1e}")
    assert abs(tot.mean()) <= 3.5 * se + 1e-5
    assert abs(a.mean()) >= 20 * se
