"""GPU parity: the CUDA kernels against the FP64 oracle on the same photon
streams (per photon and per tally), through the C ABI.

Tolerances:
 * per-photon match = same fate and SPIN count, detected and absorbed weight
   within 1e-3 relative (+1e-6 absolute); FP32 stepping against FP64
   arithmetic flips a boundary decision now and then, so a stated fraction
   of photons must match, not all;
 * tallies agree within 3 combined standard errors (batch means).
"""
import numpy as np
import pytest

from nmc_gb300 import abi
import nmc_cases as cases

pytestmark = pytest.mark.gpu


def _engine(gpu, sim, rp, tp, v, ext):
    e = gpu.Engine(sim, 0, ext)
    e.prepare_data(rp, tp, v)
    return e


def test_mcsub_reference_rng_per_photon(gpu, oracle):
    """Reference generator and isotropic sampling (kernels.metal:252): the GPU
    replays the reference's own photon streams."""
    rp, tp, ext = cases.mcsub_case(phase=abi.PHASE_ISOTROPIC_REF, rng=abi.RNG_TAUS_REF, dr=0.002, dz=0.002)
    n = 20000
    e = _engine(gpu, abi.SIM_MCSUB, rp, tp, None, ext)
    recs, _ = e.run_traced(0, n)
    o = oracle.run(abi.SIM_MCSUB, rp, tp, ext=ext, n=n, trace=True)
    frac, _ = cases.match_fraction(recs, o["recs"], fields=("detected", "absorbed"))
    print(f"mcsub taus per-photon match {frac:.5f}")
    assert frac >= 0.99
    s = e.summary()
    assert s["photons"] == n
    assert abs(s["S"] + s["A"] + s["E"] - n) / n < 1e-4  # weight conservation (roulette: in expectation)


def test_mcsub_hg_philox_per_photon_and_tallies(gpu, oracle):
    rp, tp, ext = cases.mcsub_case()
    n = 20000
    e = _engine(gpu, abi.SIM_MCSUB, rp, tp, None, ext)
    recs, ev = e.run_traced(0, n, k_events=8)
    o = oracle.run(abi.SIM_MCSUB, rp, tp, ext=ext, n=n, trace=True, k_events=8)
    frac, _ = cases.match_fraction(recs, o["recs"])
    d = np.abs(ev - o["events"])
    ev_ok = np.nanmax(d[..., :3], axis=(1, 2)) <= 1e-4
    print(f"mcsub HG philox per-photon match {frac:.5f}; first-8-events match {np.mean(ev_ok):.5f}")
    assert frac >= 0.98
    assert np.mean(ev_ok) >= 0.99
    J = e.tally(abi.TALLY_J)
    F = e.tally(abi.TALLY_F)
    assert abs(J.sum() - o["J"].sum()) <= 1e-3 * o["J"].sum()
    assert abs(F.sum() - o["F"].sum()) <= 1e-3 * o["F"].sum()


def test_mcsub_tallies_within_3_sigma(gpu, oracle):
    rp, tp, ext = cases.mcsub_case()
    n_gpu, n_cpu = 1_000_000, 200_000
    e = _engine(gpu, abi.SIM_MCSUB, rp, tp, None, ext)
    e.run(10_000_000, n_gpu)
    s = e.summary()
    o = oracle.run(abi.SIM_MCSUB, rp, tp, ext=ext, first=0, n=n_cpu)
    for key, g, c, gs, cs in (("Rd", s["rd_sum"], o["rd_sum"], s["rd_sumsq"], o["rd_sumsq"]),):
        mg, mc = g / n_gpu, c / n_cpu
        se = np.sqrt((gs / n_gpu - mg ** 2) / n_gpu + (cs / n_cpu - mc ** 2) / n_cpu)
        print(f"{key}: gpu {mg:.6f} oracle {mc:.6f} z={(mg - mc) / se:.2f}")
        assert abs(mg - mc) <= 3 * se
    assert abs(s["S"] + s["A"] + s["E"] - n_gpu) / n_gpu < 1e-4


@pytest.mark.parametrize("precise", [False, True], ids=["fast-math", "precise-math"])
def test_mcxyz_skin_vessel_per_photon(gpu, oracle, precise):
    rp, tp, v, ext = cases.skin_vessel_case(N=48)
    if precise:
        ext.flags |= abi.FLAG_PRECISE_MATH
    n = 4000
    e = _engine(gpu, abi.SIM_MCXYZ, rp, tp, v, ext)
    recs, ev = e.run_traced(0, n, k_events=16)
    o = oracle.run(abi.SIM_MCXYZ, rp, tp, v, ext=ext, n=n, trace=True, k_events=16)
    frac, _ = cases.match_fraction(recs, o["recs"])
    d = np.abs(ev - o["events"])[..., :3]
    prefix_ok = np.all(np.where(np.isnan(d), True, d <= 1e-4), axis=2)
    first16 = np.mean(np.all(prefix_ok, axis=1))
    print(f"mcxyz skin-vessel ({'precise' if precise else 'fast'}) per-photon match {frac:.4f}; first-16-events match {first16:.4f}; "
          f"substeps/photon gpu {recs['n_sub'].mean():.1f} oracle {o['recs']['n_sub'].mean():.1f}")
    assert frac >= (0.95 if precise else 0.90)
    assert first16 >= 0.98


def test_mcxyz_skin_vessel_tallies_3_sigma(gpu, oracle):
    rp, tp, v, ext = cases.skin_vessel_case(N=64)
    n_gpu, n_cpu = 200_000, 40_000
    e = _engine(gpu, abi.SIM_MCXYZ, rp, tp, v, ext)
    e.run(1_000_000, n_gpu)
    s = e.summary()
    o = oracle.run(abi.SIM_MCXYZ, rp, tp, v, ext=ext, first=0, n=n_cpu)
    mg, mc = s["rd_sum"] / n_gpu, o["rd_sum"] / n_cpu
    se = np.sqrt((s["rd_sumsq"] / n_gpu - mg ** 2) / n_gpu + (o["rd_sumsq"] / n_cpu - mc ** 2) / n_cpu)
    print(f"Rd gpu {mg:.6f} oracle {mc:.6f} z={(mg - mc) / se:.2f}; substeps/photon gpu "
          f"{s['substeps'] / n_gpu:.1f} oracle {o['substeps'] / n_cpu:.1f}")
    assert abs(mg - mc) <= 3 * se
    F = e.tally(abi.TALLY_F3D)
    ag, ac = F.sum() / n_gpu, o["F3D"].sum() / n_cpu
    assert abs(ag - ac) <= 0.02 * ac
    assert abs(s["A"] / n_gpu - o["A"] / n_cpu) <= 0.02 * (o["A"] / n_cpu)


def test_mcxyz_two_term_per_photon(gpu, oracle):
    rp, tp, v, ext = cases.skin_vessel_case(N=40)
    rp.mckernelflag = abi.SIM_MCXYZ_TT
    rp.boundaryflag = 1
    for t in range(1, 5):
        tp.gf[t], tp.af[t], tp.gb[t], tp.ab[t], tp.CC[t] = 0.9, 0.5, 0.3, 0.5, 0.9
    n = 3000
    e = _engine(gpu, abi.SIM_MCXYZ_TT, rp, tp, v, ext)
    recs, _ = e.run_traced(0, n)
    o = oracle.run(abi.SIM_MCXYZ_TT, rp, tp, v, ext=ext, n=n, trace=True)
    frac, _ = cases.match_fraction(recs, o["recs"])
    print(f"mcxyz two-term per-photon match {frac:.4f}")
    assert frac >= 0.75


@pytest.mark.parametrize("case", ["C1 mcsub mua 1 mus 100 g 0.9", "C2 skin-vessel 200^3 x 0.005 cm"])
def test_step_counts_match_the_fp64_oracle(gpu, oracle, case):
    # the unit of the roofline is the photon step (mcsub) or voxel sub-step
    # (mcxyz), counted in the kernel: on the same photons the mean count
    # equals the FP64 oracle's to within 1 %.  Per photon, mcsub counts are
    # equal; a voxel walk in FP32 cell offsets can land a few steps exactly on
    # a face where FP64 lands beside it, so its counts agree within 1 %.
    if case.startswith("C1"):
        sim, (rp, tp, ext), v, n = abi.SIM_MCSUB, cases.mcsub_case(), None, 20_000
    else:
        rp, tp, v, ext = cases.skin_vessel_case(N=200, d=0.005)
        sim, n = abi.SIM_MCXYZ, 3_000
    e = _engine(gpu, sim, rp, tp, v, ext)
    recs, _ = e.run_traced(0, n)
    o = oracle.run(sim, rp, tp, v, ext=ext, n=n, trace=True)
    g_sub, o_sub = recs["n_sub"].astype(np.float64), o["recs"]["n_sub"].astype(np.float64)
    same = np.mean(g_sub == o_sub)
    close = np.mean(np.abs(g_sub - o_sub) <= np.maximum(2.0, 0.01 * o_sub))
    print(f"{case}: steps/photon gpu {g_sub.mean():.2f} oracle {o_sub.mean():.2f}; per photon equal {same:.4f}, "
          f"within 1 % {close:.4f}")
    assert abs(g_sub.mean() - o_sub.mean()) <= 0.01 * o_sub.mean()
    assert (same if sim == abi.SIM_MCSUB else close) >= 0.95
    assert e.summary()["substeps"] == int(g_sub.sum())


@pytest.mark.parametrize("kind", ["mcsub", "mcxyz", "mcxyz_tt"])
def test_every_tally_within_3_sigma_of_the_fp64_oracle(gpu, oracle, kind):
    # every bin of every tally of the engine against the FP64 oracle over the
    # same photons; each bin's standard error comes from the spread of the
    # oracle's 10 batches.  The relative error of each tally's total against
    # the oracle is printed.
    B = 10
    if kind == "mcsub":
        rp, tp, ext = cases.mcsub_case()
        sim, v, per = abi.SIM_MCSUB, None, 20_000
        which = {"J": abi.TALLY_J, "F": abi.TALLY_F}
    else:
        rp, tp, v, ext = cases.skin_vessel_case(N=48)
        sim, per = abi.SIM_MCXYZ, 4_000
        which = {"F3D": abi.TALLY_F3D, "Rd2D": abi.TALLY_RD2D, "DetPhot2D": abi.TALLY_DETPHOT2D,
                 "rd_slots": abi.TALLY_RD_SLOTS}
        if kind == "mcxyz_tt":  # two-term phase function; its Rd2D rule keeps no DetPhot2D
            sim = rp.mckernelflag = abi.SIM_MCXYZ_TT
            rp.boundaryflag = 1
            for t in range(1, 5):
                tp.gf[t], tp.af[t], tp.gb[t], tp.ab[t], tp.CC[t] = 0.9, 0.5, 0.3, 0.5, 0.9
            del which["DetPhot2D"]
    batches = [oracle.run(sim, rp, tp, v, ext=ext, first=b * per, n=per) for b in range(B)]
    e = _engine(gpu, sim, rp, tp, v, ext)
    e.run(0, B * per)
    for name, t in which.items():
        orc = np.stack([r[name] for r in batches])
        tot = orc.sum(0)
        se = np.sqrt(B) * orc.std(0, ddof=1)
        g = e.tally(t)
        assert g.shape == tot.shape, name
        # the batch spread estimates a bin's error once photons reach it in
        # most batches; a bin reached by a photon or two (where one of the
        # ~0.2-2 % of photons whose FP32 walk parts from FP64 can land) is
        # checked in aggregate below
        live = ((orc != 0).sum(0) >= 5) & (se > 0)
        z = (g[live] - tot[live]) / se[live]
        zmax = float(np.abs(z).max()) if live.any() else 0.0
        if live.any():
            k = np.flatnonzero(live)[np.argmax(np.abs(z))]
            print(f"  worst bin {k}: engine {g[k]:.9g} oracle {tot[k]:.9g} se {se[k]:.3g} "
                  f"batches {np.array2string(orc[:, k], precision=6)}")
        rel = abs(g.sum() - tot.sum()) / max(tot.sum(), 1e-30)
        print(f"{kind} {name}: {live.sum()} well-populated bins, max |z| {zmax:.2f}; "
              f"total {g.sum():.6g} vs oracle {tot.sum():.6g} (rel error {rel:.2e})")
        sparse = np.abs(g[~live] - tot[~live]).sum() / max(np.abs(tot).sum(), 1e-30)
        print(f"  sparse bins {int((~live).sum())}: summed |difference| {sparse:.2e} of the tally")
        assert (live.any() or name == "rd_slots") and zmax <= 3.0, name  # a slot holds 4 photons here
        assert rel <= 1e-3, name
        assert sparse <= 1e-3, name


def test_tallies_bit_reproducible(gpu):
    rp, tp, v, ext = cases.skin_vessel_case(N=48)
    out = []
    for _ in range(2):
        e = _engine(gpu, abi.SIM_MCXYZ, rp, tp, v, ext)
        e.run(0, 50_000)
        out.append((e.tally(abi.TALLY_F3D), e.tally(abi.TALLY_RD2D), e.summary()["rd_sum"]))
        e.close()
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2]
