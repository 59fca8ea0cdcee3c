"""The adaptive sweep driver (nmc_gb300.sweep.sweep) on the CPU: an engine
stand-in runs each mcsub set through the oracle on the photon range the
driver asks for, so the driver's pilot, budget and stream continuation are
checked without a GPU:
  * with a target, every set that its budget does not cap reaches the target
    relative standard error of Rd, and a capped set runs its whole budget;
  * the pilot and the top-up together equal one run of the same photons
    (each set continues its stream where the pilot stopped);
  * without a target every set runs its budget in one launch.
"""
import math

import numpy as np
import pytest

from nmc_gb300 import abi, sweep
import nmc_cases as cases


class OracleSweepEngine:
    """Runs abi.SweepSet lists like Engine.run_sweep, through the oracle's
    mcsub restatement (set k draws from seed k)."""

    sim_type = abi.SIM_MCSUB

    def __init__(self, oracle):
        self.oracle = oracle
        self.calls = []

    def run_sweep(self, sets):
        self.calls.append([(int(s.photons), int(s.first_photon)) for s in sets])
        out = {k: np.zeros(len(sets)) for k in abi.SWEEP_FIELDS}
        for k, s in enumerate(sets):
            if s.photons == 0:
                continue
            rp, tp, ext = cases.mcsub_case(g=s.g, mua=s.mua, mus=s.mus, n1=s.n1, n2=s.n2, seed=k)
            r = self.oracle.run(abi.SIM_MCSUB, rp, tp, ext=ext, first=int(s.first_photon), n=int(s.photons),
                                nthreads=1, tallies=False)
            n = r["photons"]
            out["photons"][k] = n
            out["hops"][k] = r["substeps"]
            out["S"][k], out["A"][k], out["E"][k], out["E2"][k] = r["S"], r["A"], r["E"], r["rd_sumsq"]
            out["Rd"][k] = (r["S"] + r["E"]) / n
            me = r["E"] / n
            out["Rd_se"][k] = math.sqrt(max(r["rd_sumsq"] / n - me * me, 0.0) / n)
        return out


def _sets():
    # three media of different Rd and variance; the last one (albedo 0.5,
    # isotropic, relative SE of Rd 3% at 3000 photons) has too small a
    # budget for the target
    media = [(1.0, 100.0, 0.9), (5.0, 50.0, 0.8), (20.0, 20.0, 0.0)]
    budgets = [200_000, 200_000, 3_000]
    return [abi.SweepSet(mua=a, mus=s, g=g, gf=0, af=0, gb=0, ab=0, cc=0, n1=1.37, n2=1.0, photons=b,
                         first_photon=0) for (a, s, g), b in zip(media, budgets)]


def test_target_reached_or_budget_spent(oracle):
    e = OracleSweepEngine(oracle)
    sets = _sets()
    r = sweep.sweep(e, sets, target_rel_se=0.02, pilot=2_000)
    assert r["launches"] == 2 and len(e.calls) == 2
    # the pilot runs min(pilot, budget) photons of every set from photon 0
    assert e.calls[0] == [(2_000, 0), (2_000, 0), (2_000, 0)]
    # the top-up continues each stream where the pilot stopped
    assert all(first == 2_000 for _, first in e.calls[1])
    rel = r["Rd_se"] / r["Rd"]
    for k, s in enumerate(sets):
        if r["photons"][k] < s.photons:
            assert rel[k] <= 0.02 * 1.05, (k, rel[k])
        else:
            assert r["photons"][k] == s.photons
    assert r["photons"][2] == 3_000  # capped by its budget
    assert np.all(r["photons"][:2] > 2_000)  # topped up to the target


def test_pilot_and_top_up_equal_one_run(oracle):
    e = OracleSweepEngine(oracle)
    sets = _sets()[:2]
    r = sweep.sweep(e, sets, target_rel_se=0.02, pilot=2_000)
    n = r["photons"].astype(int)
    one = OracleSweepEngine(oracle).run_sweep(
        [sweep._copy(s, photons=int(n[k]), first_photon=0) for k, s in enumerate(sets)])
    for f in ("photons", "hops", "S", "A", "E", "E2", "Rd", "Rd_se"):
        np.testing.assert_allclose(r[f], one[f], rtol=1e-9, err_msg=f)


def test_no_target_runs_budgets_in_one_launch(oracle):
    e = OracleSweepEngine(oracle)
    sets = [sweep._copy(s, photons=1_000) for s in _sets()]
    r = sweep.sweep(e, sets)
    assert r["launches"] == 1 and e.calls == [[(1_000, 0)] * 3]
    assert list(r["photons"]) == [1_000] * 3


@pytest.mark.parametrize("pilot", [500, 5_000])
def test_pilot_never_exceeds_budget(oracle, pilot):
    e = OracleSweepEngine(oracle)
    sets = [sweep._copy(s, photons=1_000) for s in _sets()]
    sweep.sweep(e, sets, target_rel_se=0.5, pilot=pilot)
    assert all(n == min(pilot, 1_000) for n, _ in e.calls[0])
