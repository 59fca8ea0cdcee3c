"""Batched sweep: many parameter sets in one persistent launch.

Set s of a sweep draws its photons from Philox key (seed lo, seed hi + s),
so it must reproduce exactly (same integer tallies) a plain single-set run
with seed + (s << 32); and its Rd must agree with the FP64 oracle within 3
combined standard errors.
"""
import numpy as np
import pytest

from nmc_gb300 import abi
import nmc_cases as cases

pytestmark = pytest.mark.gpu


def _sweep_ext():
    return abi.ext_defaults(phase=abi.PHASE_TWO_TERM, sub_bins=101, sub_dr=0.01, sub_dz=0.01, seed=11)


def test_sweep_sets_equal_plain_runs(gpu):
    lam, sets = cases.spectral_sweep_sets(n_wavelengths=12, budget_lo=2e3, budget_hi=5e4)
    ext = _sweep_ext()
    rp, tp, _ = cases.mcsub_case(tt=(0.9, 0.5, 0.3, 0.5, 0.9))
    with gpu.Engine(abi.SIM_MCSUB, 0, ext) as e:
        e.prepare_data(rp, tp)
        sw = e.run_sweep(sets, with_J=True)
    for s in (0, 5, 11):
        q = sets[s]
        ext_s = _sweep_ext()
        ext_s.seed = ext.seed + (s << 32)
        tps = abi.tissue_params(mua=[q.mua], mus=[q.mus], g=[q.g], gf=[q.gf], af=[q.af], gb=[q.gb], ab=[q.ab],
                                cc=[q.cc])
        with gpu.Engine(abi.SIM_MCSUB, 0, ext_s) as e:
            e.prepare_data(rp, tps)
            e.run(0, q.photons)
            sm = e.summary()
            J = e.tally(abi.TALLY_J)
        # same photon streams: identical counts; weights equal up to the FP32
        # rounding the two separately compiled kernels may contract differently
        # (a wrong key or set would differ at the 1e-2 level)
        assert sw["photons"][s] == q.photons == sm["photons"]
        assert sw["hops"][s] == sm["substeps"]
        for k in ("S", "A", "E"):
            assert sw[k][s] == pytest.approx(sm[k], rel=1e-6), (s, k)
        np.testing.assert_allclose(sw["J"][s], J, rtol=1e-5, atol=1e-6)


def test_sweep_rd_against_oracle(gpu, oracle):
    lam, sets = cases.spectral_sweep_sets(n_wavelengths=6, budget_lo=2e5, budget_hi=2e5)
    ext = _sweep_ext()
    rp, tp, _ = cases.mcsub_case(tt=(0.9, 0.5, 0.3, 0.5, 0.9))
    with gpu.Engine(abi.SIM_MCSUB, 0, ext) as e:
        e.prepare_data(rp, tp)
        sw = e.run_sweep(sets)
    for s, q in enumerate(sets):
        tps = abi.tissue_params(mua=[q.mua], mus=[q.mus], g=[q.g], gf=[q.gf], af=[q.af], gb=[q.gb], ab=[q.ab],
                                cc=[q.cc])
        ext_o = _sweep_ext()
        ext_o.seed = 999 + s  # independent streams
        n_o = 40_000
        o = oracle.run(abi.SIM_MCSUB, rp, tps, ext=ext_o, n=n_o, tallies=False)
        rd_o = (o["S"] + o["E"]) / n_o
        se_o = np.sqrt(max(o["rd_sumsq"] / n_o - (o["E"] / n_o) ** 2, 0) / n_o)
        z = (sw["Rd"][s] - rd_o) / np.hypot(sw["Rd_se"][s], se_o)
        print(f"set {s}: mua {q.mua:.3f} mus {q.mus:.1f} Rd gpu {sw['Rd'][s]:.5f} oracle {rd_o:.5f} z={z:.2f}")
        assert abs(z) <= 3.0


# ---- voxel sweeps: many tissue tables on one skin-vessel map


def _sv_engine(gpu, N=64, seed=11):
    rp, tp, v, ext = cases.skin_vessel_case(N=N, d=0.005, seed=seed)
    e = gpu.Engine(abi.SIM_MCXYZ_TT, 0, ext)
    e.prepare_data(rp, tp, v)
    return e, rp, v, ext


def test_tissue_sweep_sets_equal_plain_runs(gpu):
    lam, tables, budgets = cases.skin_vessel_spectral_tables(n_wavelengths=12, budget_lo=2e3, budget_hi=3e4)
    e, rp, v, ext = _sv_engine(gpu)
    with e:
        sw = e.run_sweep_tissues(tables, budgets)
    for s in (0, 5, 11):
        ext_s = cases.skin_vessel_case(N=64, d=0.005, seed=11)[3]
        ext_s.seed = ext.seed + (s << 32)
        with gpu.Engine(abi.SIM_MCXYZ_TT, 0, ext_s) as p:
            p.prepare_data(rp, tables[s], v)
            p.run(0, int(budgets[s]))
            sm = p.summary()
        assert sw["photons"][s] == budgets[s] == sm["photons"]
        assert sw["hops"][s] == sm["substeps"], s
        assert sw["A"][s] == pytest.approx(sm["A"], rel=1e-6)
        assert sw["E"][s] == pytest.approx(sm["rd_sum"], rel=1e-6)


def test_tissue_sweep_rd_against_oracle(gpu, oracle):
    lam, tables, budgets = cases.skin_vessel_spectral_tables(n_wavelengths=351)
    pick = [0, 200]
    e, rp, v, ext = _sv_engine(gpu)
    with e:
        sw = e.run_sweep_tissues([tables[i] for i in pick], [200_000] * len(pick))
    for j, i in enumerate(pick):
        ext_o = cases.skin_vessel_case(N=64, d=0.005)[3]
        ext_o.seed = 777 + j  # independent streams
        n_o = 30_000
        o = oracle.run(abi.SIM_MCXYZ_TT, rp, tables[i], v, ext=ext_o, n=n_o, tallies=False)
        rd_o = o["rd_sum"] / n_o
        se_o = np.sqrt(max(o["rd_sumsq"] / n_o - rd_o ** 2, 0) / n_o)
        z = (sw["Rd"][j] - rd_o) / np.hypot(sw["Rd_se"][j], se_o)
        print(f"{lam[i]:.0f} nm: Rd gpu {sw['Rd'][j]:.5f} +- {sw['Rd_se'][j]:.5f} oracle {rd_o:.5f} +- {se_o:.5f} z={z:.2f}")
        assert abs(z) <= 3.0


def test_tissue_sweep_to_target_continues_each_stream(gpu):
    from nmc_gb300.sweep import TissueSet, sweep

    lam, tables, budgets = cases.skin_vessel_spectral_tables(n_wavelengths=24, budget_lo=1e4, budget_hi=4e5)
    sets = [TissueSet(t, b) for t, b in zip(tables, budgets)]
    e, rp, v, ext = _sv_engine(gpu)
    with e:
        r = sweep(e, sets, target_rel_se=0.01, pilot=5000)
        # the pilot and the top-up are one stream per set: a single launch of
        # the same counts gives the same photons
        one = e.run_sweep_tissues(tables, r["photons"].astype(np.int64))
    assert r["launches"] == 2
    np.testing.assert_array_equal(one["photons"], r["photons"])
    np.testing.assert_array_equal(one["hops"], r["hops"])
    np.testing.assert_allclose(one["E"], r["E"], rtol=1e-9)
    rel = r["Rd_se"] / r["Rd"]
    capped = r["photons"] >= budgets
    assert np.all((rel <= 0.0105) | capped), rel
