"""Polarised E-field transport with the coherent-backscattering cone and Raman
conversion (a semi-infinite slab of spheres): Python face of nmc_mie and
nmc_efield_run (include/nmc_abi.h).

The reference's polarisation and Raman kernels are empty stubs
(kernels.metal:1122-1202); this is the engine's own method, described in
nmc_gb300/csrc/efield.cu.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import abi
from .engine import NMCError, _ptr, lib

_P = C.c_void_p


def _bind():
    L = lib()
    if not getattr(L, "_ef_bound", False):
        L.nmc_mie.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int32, _P, _P, _P, _P]
        L.nmc_mie.restype = C.c_int
        L.nmc_efield_run.argtypes = [C.c_int32, C.POINTER(abi.EfieldConfig), _P, _P, C.POINTER(abi.EfieldSetting),
                                     C.c_int32, _P, _P, _P, _P, _P, _P, _P]
        L.nmc_efield_run.restype = C.c_int
        L.nmc_speckle_mutual.argtypes = [C.c_int32, C.c_int32, C.c_int32, _P, _P, _P, C.c_int32, C.c_float,
                                         C.c_float, _P]
        L.nmc_speckle_mutual.restype = C.c_int
        L._ef_bound = True
    return L


def mie(x: float, m: complex, n_angles: int = 1801) -> dict:
    """Mie amplitudes of a sphere: size parameter x = 2 pi n_medium a / lambda,
    relative index m.  Returns S1, S2 (complex, n_angles, theta_j = j pi /
    (n_angles - 1)), the table as float32 rows (Re S1, Im S1, Re S2, Im S2),
    q_ext, q_sca and g."""
    L = _bind()
    S = np.zeros((n_angles, 4), np.float32)
    qe, qs, g = C.c_double(), C.c_double(), C.c_double()
    st = L.nmc_mie(float(x), float(m.real), float(m.imag), int(n_angles), _ptr(S), C.byref(qe), C.byref(qs),
                   C.byref(g))
    if st != 0:
        raise NMCError(st, "nmc_mie")
    return {"S1": S[:, 0] + 1j * S[:, 1], "S2": S[:, 2] + 1j * S[:, 3], "table": S, "q_ext": qe.value,
            "q_sca": qs.value, "g": g.value,
            "theta": np.linspace(0.0, math.pi, n_angles)}


def sphere_suspension(radius_um: float, n_sphere: float, n_medium: float, wavelength_nm: float, mus: float,
                      n_angles: int = 1801) -> dict:
    """Mie table of monodisperse spheres and the number density (per cm^3)
    that gives scattering coefficient `mus` (1/cm)."""
    x = 2 * math.pi * n_medium * radius_um / (wavelength_nm * 1e-3)
    r = mie(x, complex(n_sphere / n_medium, 0.0), n_angles)
    sigma = r["q_sca"] * math.pi * (radius_um * 1e-4) ** 2  # cm^2
    r["x"] = x
    r["number_density"] = mus / sigma
    return r


def run(config: abi.EfieldConfig, S_primary, settings, S_raman=None, device: int = 0, cone: bool = True,
        pol_vs_scatt: bool = True, maps: bool = True, raman_depth: bool = True) -> dict:
    """One persistent launch over `settings` (abi.EfieldSetting).  Returns
    per-setting scalars (abi.EF_FIELDS), and when asked: the complex
    interference cone [setting, channel (co, cross), theta_x, theta_y], the
    XX/XY/YX/YY intensity by scattering order, the exit maps (abi.EF_MAPS)
    and the Raman conversion depth histogram."""
    L = _bind()
    n = len(settings)
    arr = (abi.EfieldSetting * n)(*settings)
    S0 = np.ascontiguousarray(S_primary, np.float32)
    S1 = None if S_raman is None else np.ascontiguousarray(S_raman, np.float32)
    out = np.zeros((n, len(abi.EF_FIELDS)), np.float64)
    cn, mn = config.cone_n, config.map_n
    cbuf = np.zeros((n, 2, cn, cn, 2), np.float32) if cone else None
    pbuf = np.zeros((n, 4, abi.EF_MAX_ORDER + 1), np.float64) if pol_vs_scatt else None
    mbuf = np.zeros((n, len(abi.EF_MAPS), mn, mn), np.float32) if maps else None
    dbuf = np.zeros((n, config.depth_bins), np.float64) if raman_depth else None
    spk = maps and config.speckle_max > 0
    sbuf = np.zeros((n, config.speckle_max, mn, mn), abi.SPECKLE_DTYPE) if spk else None
    scnt = np.zeros((n, mn, mn), np.int32) if spk else None
    st = L.nmc_efield_run(int(device), C.byref(config), _ptr(S0), _ptr(S1), arr, n, _ptr(out), _ptr(cbuf),
                          _ptr(pbuf), _ptr(mbuf), _ptr(dbuf), _ptr(sbuf), _ptr(scnt))
    if st != 0:
        raise NMCError(st, "nmc_efield_run")
    res = {k: out[:, i] for i, k in enumerate(abi.EF_FIELDS)}
    if cone:
        res["cone"] = cbuf[..., 0] + 1j * cbuf[..., 1]
    if pol_vs_scatt:
        res["pol_vs_scatt"] = pbuf
    if maps:
        res["maps"] = {k: mbuf[:, i] for i, k in enumerate(abi.EF_MAPS)}
    if raman_depth:
        res["raman_depth"] = dbuf
    if spk:
        res["speckles"], res["speckle_counts"] = sbuf, scnt
    return res


def speckle_mutual(maps: np.ndarray, records: np.ndarray, counts: np.ndarray, wavelength: float,
                   coherence_length: float, out: np.ndarray | None = None, device: int = 0) -> np.ndarray:
    """The reference's speckle mutual-interference post-processing
    (MetalMC.m:628-742) on the GPU.  maps: (NMC_EF_MAPS, nx, ny) float32 of
    one setting; records: (kmax, nx, ny) abi.SPECKLE_DTYPE; counts (nx, ny).
    Returns `out` (zeros if None) with the mutual maps added."""
    L = _bind()
    m = np.ascontiguousarray(maps, np.float32)
    _, nx, ny = m.shape
    r = np.ascontiguousarray(records, abi.SPECKLE_DTYPE)
    c = np.ascontiguousarray(counts, np.int32)
    o = np.zeros_like(m) if out is None else out
    st = L.nmc_speckle_mutual(int(device), nx, ny, _ptr(m), _ptr(r), _ptr(c), r.shape[0], float(wavelength),
                              float(coherence_length), _ptr(o))
    if st != 0:
        raise NMCError(st, "nmc_speckle_mutual")
    return o
