"""Layered media (nmc_layered_run): the mcsub physics in a stack of plane
layers with Fresnel boundaries, Rd(r), Tt(r), A(z), A(r, z) and absorption per
layer.  The reference declares MAXLAYERS (definitions.h:24) but simulates a
single semi-infinite layer; see nmc_gb300/csrc/layered.cu."""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import abi
from .engine import NMCError, _ptr, lib

_P = C.c_void_p


def _bind():
    L = lib()
    if not getattr(L, "_lay_bound", False):
        L.nmc_layered_run.argtypes = [C.c_int32, C.POINTER(abi.LayeredConfig), C.POINTER(abi.Layer), C.c_uint64,
                                      C.c_uint64, _P, _P, _P, _P, _P, _P]
        L.nmc_layered_run.restype = C.c_int
        L.nmc_layered_adjoint.argtypes = [C.c_int32, C.POINTER(abi.LayeredConfig), C.POINTER(abi.Layer),
                                          C.c_uint64, C.c_uint64, _P, _P, _P, _P, _P, _P, _P, _P]
        L.nmc_layered_adjoint.restype = C.c_int
        L._lay_bound = True
    return L


def run(layers, photons: int, n_above: float = 1.0, n_below: float = 1.0, nr: int = 100, dr: float = 0.01,
        nz: int = 100, dz: float = 0.01, seed: int = 0, first: int = 0, a_rz: bool = False, device: int = 0,
        precise: bool = False, flags: int = 0) -> dict:
    """`layers`: sequence of (mua, mus, g, n, thickness) (cm^-1, cm; the last
    thickness may be math.inf).  Returns the sums (abi.LAY_FIELDS), Rd and Tt
    per launched photon with their standard errors, and the tallies
    (un-normalised weights: rd_r, tt_r with nr+1 bins, a_z with nz+1, a_layer,
    a_rz if asked).  `flags` may add abi.FLAG_LAYERED_REF_STREAMS (the
    reference's generator and draw order; `seed` is then the dispatch batch)
    and abi.FLAG_LAYERED_ISOTROPIC (the reference's isotropic scattering)."""
    L = _bind()
    arr = (abi.Layer * len(layers))(*[abi.Layer(*map(float, q)) for q in layers])
    cfg = abi.LayeredConfig(n_layers=len(layers), n_above=n_above, n_below=n_below, nr=nr, dr=dr, nz=nz, dz=dz,
                            flags=(abi.FLAG_PRECISE_MATH if precise else 0) | flags, seed=seed)
    out = np.zeros(len(abi.LAY_FIELDS), np.float64)
    rd, tt, az = np.zeros(nr + 1), np.zeros(nr + 1), np.zeros(nz + 1)
    al = np.zeros(len(layers))
    arz = np.zeros((nr + 1, nz + 1)) if a_rz else None
    st = L.nmc_layered_run(int(device), C.byref(cfg), arr, int(first), int(photons), _ptr(out), _ptr(rd), _ptr(tt),
                           _ptr(az), _ptr(arz), _ptr(al))
    if st != 0:
        raise NMCError(st, "nmc_layered_run")
    res = {k: out[i] for i, k in enumerate(abi.LAY_FIELDS)}
    n = max(res["photons"], 1.0)
    for k in ("Rd", "Tt"):
        m = res[k] / n
        res[k.lower()] = m
        res[k.lower() + "_se"] = math.sqrt(max(res[k + "2"] / n - m * m, 0.0) / n)
    res.update(rd_r=rd, tt_r=tt, a_z=az, a_layer=al)
    if a_rz:
        res["a_rz"] = arz
    return res


def adjoint(layers, photons: int, grad_rd_r=None, grad_tt_r=None, n_above: float = 1.0, n_below: float = 1.0,
            nr: int = 100, dr: float = 0.01, seed: int = 0, first: int = 0, device: int = 0) -> dict:
    """Per-layer gradients of L = grad_rd_r . rd_r + grad_tt_r . tt_r (the
    un-normalised radial tallies of photons [first, first + photons)) with
    respect to each layer's mua, mus and g (perturbation Monte Carlo), with
    the run's tallies.  At most 16 layers."""
    L = _bind()
    nl = len(layers)
    arr = (abi.Layer * nl)(*[abi.Layer(*map(float, q)) for q in layers])
    cfg = abi.LayeredConfig(n_layers=nl, n_above=n_above, n_below=n_below, nr=nr, dr=dr, nz=1, dz=1.0, flags=0,
                            seed=seed)
    grd = None if grad_rd_r is None else np.ascontiguousarray(grad_rd_r, np.float32)
    gtt = None if grad_tt_r is None else np.ascontiguousarray(grad_tt_r, np.float32)
    for g in (grd, gtt):
        if g is not None and g.size != nr + 1:
            raise ValueError(f"upstream gradients need nr + 1 = {nr + 1} values")
    out = np.zeros(len(abi.LAY_FIELDS), np.float64)
    rd, tt = np.zeros(nr + 1), np.zeros(nr + 1)
    ga, gs, gg = np.zeros(nl), np.zeros(nl), np.zeros(nl)
    st = L.nmc_layered_adjoint(int(device), C.byref(cfg), arr, int(first), int(photons), _ptr(grd), _ptr(gtt),
                               _ptr(out), _ptr(rd), _ptr(tt), _ptr(ga), _ptr(gs), _ptr(gg))
    if st != 0:
        raise NMCError(st, "nmc_layered_adjoint")
    res = {k: out[i] for i, k in enumerate(abi.LAY_FIELDS)}
    res.update(rd_r=rd, tt_r=tt, grad_mua=ga, grad_mus=gs, grad_g=gg)
    return res
