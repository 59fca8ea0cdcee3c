"""Wavelength-dependent tissue optical properties, feeding batched sweeps.

Restates the tissue model the reference's sample notebooks use to build a
tissue table per wavelength (NMC-samples/example3.ipynb cell 2,
`tissue_parameters`; the mcxyz `makeTissueList` model of S. Jacques):
  mua(lambda) = B S muaoxy + B (1 - S) muadeoxy + W muawater + M muamel
  mus'(lambda) = mus'500 (fray (lambda/500)^-4 + (1 - fray) (lambda/500)^-bmie),
  mus = mus' / (1 - g),
with the chromophore spectra interpolated linearly in a spectral library
(the notebooks' spectralLIB.mat: nmLIB, muaoxy, muadeoxy, muawater, muamel,
cm^-1).  The per-tissue parameters below are the notebooks' table, kept
identical because results are compared against runs made with it.
"""
from __future__ import annotations

import numpy as np

from . import abi

# id: (name, B blood fraction, S oxygen saturation, W water, M melanin,
#      mus'500 [1/cm], fray, bmie, g); None = fixed optical properties
TISSUES = {
    1: ("air", None, (1e-4, 1.0, 1.0)),
    2: ("water", "water", (10.0, 1.0)),
    3: ("blood", (1.00, 0.75, 0.95, 0.0, 10.0, 0.0, 1.0, 0.90), None),
    4: ("dermis", (0.002, 0.67, 0.65, 0.0, 43.6, 0.41, 0.562, 0.90), None),
    5: ("epidermis", (0.0, 0.75, 0.75, 0.03, 66.7, 0.29, 0.689, 0.90), None),
    6: ("skull", (0.0005, 0.75, 0.35, 0.0, 30.0, 0.0, 1.0, 0.90), None),
    7: ("gray matter", (0.01, 0.75, 0.75, 0.0, 20.0, 0.2, 1.0, 0.90), None),
    8: ("white matter", (0.01, 0.75, 0.75, 0.0, 20.0, 0.2, 1.0, 0.90), None),
    9: ("standard tissue", None, (1.0, 100.0, 0.90)),
}


def load_library(path: str) -> dict:
    """The spectral library (.mat) as numpy arrays: nmLIB, muaoxy, muadeoxy,
    muawater, muamel."""
    from scipy.io import loadmat

    d = loadmat(path)
    return {k: np.asarray(d[k], dtype=np.float64).ravel() for k in ("nmLIB", "muaoxy", "muadeoxy", "muawater",
                                                                   "muamel")}


def chromophores(nm: float, lib: dict) -> np.ndarray:
    """Absorption of oxy-Hb, deoxy-Hb, water and melanin at nm (linear
    interpolation in the library)."""
    x = lib["nmLIB"]
    return np.array([np.interp(nm, x, lib[k]) for k in ("muaoxy", "muadeoxy", "muawater", "muamel")])


def tissue_list(nm: float, lib: dict | None = None, mu: np.ndarray | None = None) -> dict:
    """{id: {name, mua, mus, g, musp}} at wavelength nm, from the library or
    from the four chromophore absorptions `mu` at nm."""
    MU = chromophores(nm, lib) if mu is None else np.asarray(mu, np.float64)
    x = nm / 500.0
    out = {}
    for tid, (name, mix, fixed) in TISSUES.items():
        if mix is None:
            mua, mus, g = fixed
        elif mix == "water":
            mua, (mus, g) = float(MU[2]), fixed
        else:
            B, S, W, M, musp500, fray, bmie, g = mix
            mua = float(MU @ np.array([B * S, B * (1 - S), W, M]))
            musp = musp500 * (fray * x ** -4 + (1 - fray) * x ** -bmie)
            mus = musp / (1 - g)
        out[tid] = {"name": name, "mua": mua, "mus": mus, "g": g, "musp": mus * (1 - g)}
    return out


def tissue_params(nm: float, lib: dict | None = None, mu=None, two_term: dict | None = None) -> abi.TissueParams:
    """The tissue table at nm as abi.TissueParams (ids 1..9); with
    `two_term` (gf, af, gb, ab, cc) the same two-term phase parameters for
    every tissue."""
    t = tissue_list(nm, lib, mu)
    ids = sorted(t)
    kw = {}
    if two_term:
        kw = {k: [two_term[k]] * len(ids) for k in ("gf", "af", "gb", "ab", "cc")}
    return abi.tissue_params(mua=[t[i]["mua"] for i in ids], mus=[t[i]["mus"] for i in ids],
                             g=[t[i]["g"] for i in ids], **kw)


def spectral_sets(nm_values, lib: dict, photons, two_term: dict | None = None):
    """TissueSets (nmc_gb300.sweep) for a wavelength sweep on one map: the
    replacement for one `nmc` run per wavelength (example3.ipynb cell 5)."""
    from .sweep import TissueSet

    ph = np.broadcast_to(np.asarray(photons), np.shape(nm_values))
    return [TissueSet(tissue_params(float(nm), lib, two_term=two_term), int(n)) for nm, n in zip(nm_values, ph)]
