"""Checkpoint and resume (nmc_gb300.checkpoint) on the CPU: an engine
stand-in accumulates the oracle's mcsub tallies for the photon ranges it is
asked to run, so snapshot, save, load and resume are checked without a GPU.
A run stopped after photon k, saved to a file and resumed on a fresh engine
gives the sums and tallies of one uninterrupted run."""
import numpy as np
import pytest

from nmc_gb300 import abi, checkpoint
import nmc_cases as cases


class OracleMcsubEngine:
    """The Engine calls checkpoint uses, over the oracle's mcsub restatement."""

    sim_type = abi.SIM_MCSUB

    def __init__(self, oracle):
        self.oracle = oracle
        self.rp, self.tp, self.ext = cases.mcsub_case(seed=4, bins=21, dr=0.05, dz=0.05)
        self.reset()

    def reset(self):
        self.acc = {k: 0.0 for k in ("photons", "substeps", "scatters", "S", "A", "E", "rd_sum", "rd_sumsq")}
        nb = self.ext.sub_bins + 1
        self.J, self.F = np.zeros(nb), np.zeros(nb * nb)

    def run(self, first, n):
        r = self.oracle.run(abi.SIM_MCSUB, self.rp, self.tp, ext=self.ext, first=first, n=n, nthreads=1)
        for k in self.acc:
            self.acc[k] += r[k]
        self.J += r["J"]
        self.F += r["F"]

    def summary(self):
        return dict(self.acc)

    def tally(self, which):
        return {abi.TALLY_J: self.J, abi.TALLY_F: self.F}[which].copy()


def test_resume_equals_uninterrupted(oracle, tmp_path):
    total, k = 6_000, 2_500
    a = OracleMcsubEngine(oracle)
    a.run(0, k)
    path = str(tmp_path / "ck.npz")
    checkpoint.save(path, checkpoint.snapshot(a, k))
    b = OracleMcsubEngine(oracle)
    done = checkpoint.resume(b, checkpoint.load(path), total=total, chunk=1_500)
    one = OracleMcsubEngine(oracle)
    one.run(0, total)
    ref = checkpoint.snapshot(one, total)
    assert done["next_photon"] == total
    np.testing.assert_allclose(done["sums"], ref["sums"], rtol=1e-12)
    for t in (abi.TALLY_J, abi.TALLY_F):
        np.testing.assert_allclose(done[f"tally_{t}"], ref[f"tally_{t}"], rtol=1e-12, atol=1e-12)
    assert checkpoint.sums(done)["photons"] == total


def test_resume_refuses_another_kind(oracle):
    a = OracleMcsubEngine(oracle)
    a.run(0, 100)
    snap = checkpoint.snapshot(a, 100)
    snap["sim_type"] = abi.SIM_MCXYZ
    with pytest.raises(ValueError):
        checkpoint.resume(OracleMcsubEngine(oracle), snap, total=200)
