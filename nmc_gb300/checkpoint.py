"""Checkpoint and resume of a long run.

Tallies are additive and every photon's random stream is a function of its
id, so a run of photons [0, N) can stop after photon k, save its FP64 tallies
with k, and continue later (another process, another GPU) with photons
[k, N): the sum equals the uninterrupted run (the reference pulls results
once at the end, main.m:191, and offers no resume)."""
from __future__ import annotations

import numpy as np

from . import abi

_SUMS = ("photons", "substeps", "scatters", "S", "A", "E", "rd_sum", "rd_sumsq")


def _tally_ids(engine) -> list[int]:
    if engine.sim_type == abi.SIM_MCSUB:
        return [abi.TALLY_J, abi.TALLY_F]
    ids = [abi.TALLY_F3D, abi.TALLY_RD2D, abi.TALLY_DETPHOT2D, abi.TALLY_RD_SLOTS]
    if engine._L.nmc_tally_size(engine._h, abi.TALLY_RD_R):
        ids.append(abi.TALLY_RD_R)
    return ids


def snapshot(engine, next_photon: int, previous: dict | None = None) -> dict:
    """The engine's tallies and sums (plus `previous`, a snapshot the run
    resumed from) and the id of the next photon to run."""
    s = engine.summary()
    out = {"next_photon": int(next_photon), "sim_type": engine.sim_type,
           "sums": np.array([s[k] for k in _SUMS], np.float64)}
    for t in _tally_ids(engine):
        out[f"tally_{t}"] = engine.tally(t)
    if previous is not None:
        for k, v in previous.items():
            if k == "sums" or k.startswith("tally_"):
                out[k] = out[k] + np.asarray(v) if k in out else np.asarray(v)
    return out


def save(path: str, snap: dict) -> None:
    np.savez(path, **{k: np.asarray(v) for k, v in snap.items()})


def load(path: str) -> dict:
    with np.load(path) as z:
        d = {k: z[k] for k in z.files}
    d["next_photon"] = int(d["next_photon"])
    d["sim_type"] = int(d["sim_type"])
    return d


def resume(engine, snap: dict, total: int, chunk: int | None = None) -> dict:
    """Runs photons [snap.next_photon, total) on a prepared engine (its
    tallies cleared first) and returns the combined snapshot."""
    if snap["sim_type"] != engine.sim_type:
        raise ValueError("checkpoint of another simulation kind")
    engine.reset()
    first = snap["next_photon"]
    chunk = chunk or max(total - first, 1)
    while first < total:
        n = min(chunk, total - first)
        engine.run(first, n)
        first += n
    return snapshot(engine, total, previous=snap)


def sums(snap: dict) -> dict:
    return dict(zip(_SUMS, snap["sums"].tolist()))
