"""Batched parameter sweeps (one persistent launch for many wavelengths or
tissue sets), with an optional target standard error.

Two geometries: the mcsub semi-infinite medium (sets are abi.SweepSet) and a
voxel tissue map (sets are TissueSet: one 19-entry tissue table per set on
the handle's map).  The reference sweeps wavelengths by rewriting its input
files and running one `nmc` process per wavelength on the skin-vessel map
(NMC-samples/example3.ipynb cell 5); here a whole sweep is one call.
"""
from __future__ import annotations

import copy

import numpy as np

from . import abi


class TissueSet:
    """One set of a voxel sweep: a tissue table and its photon budget."""

    def __init__(self, tp: abi.TissueParams, photons: int, first_photon: int = 0):
        self.tp = tp
        self.photons = int(photons)
        self.first_photon = int(first_photon)


def _copy(s, **kw):
    c = copy.copy(s)
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def _run(engine, sets) -> dict:
    if engine.sim_type == abi.SIM_MCSUB:
        return engine.run_sweep(list(sets))
    return engine.run_sweep_tissues([s.tp for s in sets], [s.photons for s in sets],
                                    [s.first_photon for s in sets])


def _combine(parts: list[dict]) -> dict:
    keys = ("photons", "hops", "S", "A", "E", "E2")
    tot = {k: sum(p[k] for p in parts) for k in keys}
    n = np.maximum(tot["photons"], 1)
    me = tot["E"] / n
    tot["Rd"] = (tot["S"] + tot["E"]) / n
    tot["Rd_se"] = np.sqrt(np.maximum(tot["E2"] / n - me * me, 0) / n)
    return tot


def sweep(engine, sets, target_rel_se: float | None = None, pilot: int = 20_000,
          safety: float = 1.15) -> dict:
    """Runs `sets` (abi.SweepSet on an mcsub Engine, TissueSet on an mcxyz
    Engine).

    Without a target every set runs its full budget in one launch.  With
    `target_rel_se`, a pilot launch of min(pilot, budget) photons per set
    estimates each set's per-photon variance of Rd, and one more launch adds
    the photons each set still needs (capped by its budget), continuing each
    set's photon stream where the pilot stopped.  Returns per-set arrays
    (abi.SWEEP_FIELDS) and "launches".
    """
    if target_rel_se is None:
        r = _run(engine, sets)
        r["launches"] = 1
        return r
    pil = [_copy(s, photons=min(int(pilot), int(s.photons)), first_photon=0) for s in sets]
    r1 = _run(engine, pil)
    n1 = r1["photons"]
    me = r1["E"] / np.maximum(n1, 1)
    var = np.maximum(r1["E2"] / np.maximum(n1, 1) - me * me, 1e-30)
    need = np.ceil(safety * var / (target_rel_se * np.maximum(r1["Rd"], 1e-30)) ** 2)
    budget = np.array([s.photons for s in sets], dtype=np.float64)
    extra = np.clip(np.minimum(need, budget) - n1, 0, None).astype(np.int64)
    parts = [r1]
    launches = 1
    if np.any(extra > 0):
        # every set keeps its index (its key) and continues its stream; sets
        # already precise enough get an empty budget
        top = [_copy(s, photons=int(extra[i]), first_photon=int(n1[i])) for i, s in enumerate(sets)]
        parts.append(_run(engine, top))
        launches = 2
    out = _combine(parts)
    out["launches"] = launches
    return out
