"""ctypes bindings of the CPU oracle (oracle/_build/liboracle.so) and of the
reference harness (oracle/_ref/libnmcref.so).

Test infrastructure only: used by tests/, __graft_entry__.smoke() and
bench.py's CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess

import numpy as np

from nmc_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libnmcref.so")
REF_SRC = "/root/reference/NMC/NMCCode"

_P = C.c_void_p
_dp = C.POINTER(C.c_double)


class OrcOut(C.Structure):
    _fields_ = [
        ("J", _dp),
        ("F", _dp),
        ("F3D", _dp),
        ("Rd2D", _dp),
        ("DetPhot2D", _dp),
        ("rd_slots", _dp),
        ("S", C.c_double),
        ("A", C.c_double),
        ("E", C.c_double),
        ("rd_sum", C.c_double),
        ("rd_sumsq", C.c_double),
        ("photons", C.c_double),
        ("substeps", C.c_double),
        ("scatters", C.c_double),
    ]


def build(ref: bool = True) -> None:
    """Compile the oracle (and, when the reference sources exist, the harness)."""
    targets = ["oracle"] + (["ref"] if ref else [])
    subprocess.run(["make", "-s", "-C", HERE, *targets], check=True)


def ref_available() -> bool:
    return os.path.exists(REF_SO)


_oracle = None
_ref = None


def oracle_lib():
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_SO):
            build(ref=False)
        lib = C.CDLL(ORACLE_SO)
        lib.orc_run.restype = C.c_int
        lib.orc_run.argtypes = [C.c_int, C.c_int, _P, _P, _P, _P, C.c_uint64, C.c_uint64, C.c_int,
                                C.POINTER(OrcOut), _P, _P, C.c_uint32]
        lib.orc_philox4x32_10.argtypes = [_P, _P, _P]
        lib.orc_uniforms.argtypes = [_P, C.c_int, C.c_uint64, C.c_int, _P]
        lib.orc_rfresnel.restype = C.c_double
        lib.orc_rfresnel.argtypes = [C.c_double, C.c_double, C.c_double, _dp]
        lib.orc_tt_costheta.restype = C.c_double
        lib.orc_tt_costheta.argtypes = [C.c_double] * 7
        lib.orc_hg_costheta.restype = C.c_double
        lib.orc_hg_costheta.argtypes = [C.c_double, C.c_double]
        lib.orc_speckle_mutual.argtypes = [C.c_int, C.c_int, _P, _P, _P, C.c_int, C.c_float, C.c_float, _P]
        lib.orc_speckle_mutual.restype = None
        lib.orc_layered_run.restype = C.c_int
        lib.orc_layered_run.argtypes = [C.c_int, _P, _P, C.c_uint64, C.c_uint64, C.c_int, _P, _P, _P, _P, _P, _P]
        lib.orc_efield_run.restype = C.c_int
        lib.orc_efield_run.argtypes = [C.c_int, _P, _P, _P, _P, C.c_int, C.c_int, C.c_int, _P]
        _oracle = lib
    return _oracle


def ref_lib():
    global _ref
    if _ref is None:
        if not os.path.exists(REF_SO):
            raise FileNotFoundError("reference harness not built (needs the reference sources)")
        lib = C.CDLL(REF_SO)
        for name in ("ref_mcsub", "ref_mcxyz", "ref_mcxyz_tt"):
            getattr(lib, name).restype = C.c_int
        lib.ref_rfresnel.restype = C.c_float
        lib.ref_rfresnel.argtypes = [C.c_float, C.c_float, C.c_float, C.POINTER(C.c_float)]
        lib.ref_taus_draws.argtypes = [C.c_uint, C.c_uint, C.c_uint, C.c_int, _P]
        _ref = lib
    return _ref


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_P)


def _dptr(a):
    return C.cast(None, _dp) if a is None else a.ctypes.data_as(_dp)


def run(sim: int, rp: abi.RunParams, tp: abi.TissueParams, v=None, ext: abi.Ext | None = None,
        first: int = 0, n: int = 1000, nthreads: int | None = None, real_bits: int = 64,
        tallies: bool = True, trace: bool = False, k_events: int = 0) -> dict:
    """Run photons [first, first+n) through the oracle; returns tallies and sums."""
    lib = oracle_lib()
    ext = ext or abi.ext_defaults()
    nthreads = nthreads or os.cpu_count() or 1
    out = OrcOut()
    res: dict = {}
    if tallies:
        if sim == abi.SIM_MCSUB:
            nb = ext.sub_bins + 1
            res["J"] = np.zeros(nb)
            res["F"] = np.zeros(nb * nb)
            out.J, out.F = _dptr(res["J"]), _dptr(res["F"])
        else:
            nvox = rp.Nx * rp.Ny * rp.Nz
            n2d = rp.Nx * rp.Ny
            res["F3D"] = np.zeros(nvox)
            res["Rd2D"] = np.zeros(n2d)
            res["DetPhot2D"] = np.zeros(n2d)
            res["rd_slots"] = np.zeros(ext.photons_per_dispatch)
            out.F3D, out.Rd2D = _dptr(res["F3D"]), _dptr(res["Rd2D"])
            out.DetPhot2D, out.rd_slots = _dptr(res["DetPhot2D"]), _dptr(res["rd_slots"])
    recs = np.zeros(n, abi.PHOTON_RECORD_DTYPE) if trace else None
    events = np.zeros((n, max(k_events, 0), 4), np.float32) if (trace and k_events) else None
    vv = None if v is None else np.ascontiguousarray(v, dtype=np.uint8)
    st = lib.orc_run(sim, real_bits, C.byref(rp), C.byref(tp), _ptr(vv), C.byref(ext), first, n,
                     nthreads, C.byref(out), _ptr(recs), _ptr(events), k_events if events is not None else 0)
    if st != 0:
        raise RuntimeError(f"orc_run failed: {abi.STATUS.get(st, st)}")
    for k in ("S", "A", "E", "rd_sum", "rd_sumsq", "photons", "substeps", "scatters"):
        res[k] = getattr(out, k)
    if recs is not None:
        res["recs"] = recs
    if events is not None:
        res["events"] = events
    return res


def philox(ctr, key):
    c = np.asarray(ctr, np.uint32)
    k = np.asarray(key, np.uint32)
    o = np.zeros(4, np.uint32)
    oracle_lib().orc_philox4x32_10(_ptr(c), _ptr(k), _ptr(o))
    return o


def uniforms(ext: abi.Ext, sim: int, photon: int, n: int) -> np.ndarray:
    o = np.zeros(n)
    oracle_lib().orc_uniforms(C.byref(ext), sim, photon, n, _ptr(o))
    return o


def rfresnel(n1, n2, ca1):
    ca2 = C.c_double(0)
    r = oracle_lib().orc_rfresnel(n1, n2, ca1, C.byref(ca2))
    return r, ca2.value


def tt_costheta(gf, af, gb, ab, cc, u_choice, u_sample):
    return oracle_lib().orc_tt_costheta(gf, af, gb, ab, cc, u_choice, u_sample)


def hg_costheta(g, u):
    return oracle_lib().orc_hg_costheta(g, u)


# ------------------------------------------------------------ reference harness
def ref_mcsub(rp, tp, run_lo=1, run_hi=10, batch=10000, nthreads=None, per_photon=False) -> dict:
    lib = ref_lib()
    nthreads = nthreads or os.cpu_count() or 1
    bins = lib.ref_bins()
    J = np.zeros(bins + 1)
    F = np.zeros((bins + 1) ** 2)
    SAE = np.zeros(3)
    n = (run_hi - run_lo + 1) * batch
    pp = np.zeros((n, 3), np.float32) if per_photon else None
    lib.ref_mcsub(C.byref(rp), C.byref(tp), run_lo, run_hi, batch, nthreads, _ptr(J), _ptr(F),
                  _ptr(SAE), _ptr(pp))
    return {"J": J, "F": F, "SAE": SAE, "per_photon": pp, "bins": bins}


def ref_mcxyz(rp, tp, v, run_lo=1, run_hi=10, batch=10000, nthreads=None, per_photon=False) -> dict:
    lib = ref_lib()
    nthreads = nthreads or os.cpu_count() or 1
    nvox = rp.Nx * rp.Ny * rp.Nz
    n2d = rp.Nx * rp.Ny
    F3D = np.zeros(nvox)
    Rd2D = np.zeros(n2d)
    Det = np.zeros(n2d)
    slots = np.zeros(batch)
    n = (run_hi - run_lo + 1) * batch
    pp = np.zeros(n, np.float32) if per_photon else None
    vv = np.ascontiguousarray(v, dtype=np.uint8)
    lib.ref_mcxyz(C.byref(rp), C.byref(tp), _ptr(vv), run_lo, run_hi, batch, nthreads, _ptr(F3D),
                  _ptr(Rd2D), _ptr(Det), _ptr(slots), _ptr(pp))
    return {"F3D": F3D, "Rd2D": Rd2D, "DetPhot2D": Det, "rd_slots": slots, "per_photon": pp}


def ref_mcxyz_tt(rp, tp, v, run_lo=1, run_hi=10, batch=10000, nthreads=None, replay_run1=True,
                 per_photon=False) -> dict:
    lib = ref_lib()
    nthreads = nthreads or os.cpu_count() or 1
    nvox = rp.Nx * rp.Ny * rp.Nz
    n2d = rp.Nx * rp.Ny
    F3D = np.zeros(nvox)
    Rd2D = np.zeros(n2d)
    slots = np.zeros(batch)
    n = (run_hi - run_lo + 1) * batch
    pp = np.zeros(n, np.float32) if per_photon else None
    vv = np.ascontiguousarray(v, dtype=np.uint8)
    lib.ref_mcxyz_tt(C.byref(rp), C.byref(tp), _ptr(vv), run_lo, run_hi, batch, nthreads,
                     -1 if replay_run1 else 0, _ptr(F3D), _ptr(Rd2D), _ptr(slots), _ptr(pp))
    return {"F3D": F3D, "Rd2D": Rd2D, "rd_slots": slots, "per_photon": pp}


def ref_taus(s1, s2, s3, n):
    o = np.zeros(n, np.float32)
    ref_lib().ref_taus_draws(s1, s2, s3, n, _ptr(o))
    return o


def speckle_mutual(maps, records, counts, lam, lc, out):
    """MetalMC.m:628-742 restated: adds the mutual maps into `out` (float32,
    NMC_EF_MAPS x ny*nx)."""
    lib = oracle_lib()
    nmaps, nx, ny = maps.shape
    kmax = records.shape[0]
    lib.orc_speckle_mutual(nx, ny, _ptr(np.ascontiguousarray(maps, np.float32)),
                           _ptr(np.ascontiguousarray(records)), _ptr(np.ascontiguousarray(counts, np.int32)),
                           kmax, float(lam), float(lc), _ptr(out))
    return out


def layered(layers, photons: int, n_above: float = 1.0, n_below: float = 1.0, nr: int = 100, dr: float = 0.01,
            nz: int = 100, dz: float = 0.01, seed: int = 0, first: int = 0, real_bits: int = 64,
            nthreads: int | None = None, flags: int = 0, per_photon: bool = False) -> dict:
    """The engine's layered model on the CPU (orc_layered_run), with the
    arguments and the result keys of nmc_gb300.layered.run; per_photon adds
    `per_photon` (photons x 3: escaped up, escaped down, absorbed)."""
    lib = oracle_lib()
    arr = (abi.Layer * len(layers))(*[abi.Layer(*map(float, q)) for q in layers])
    cfg = abi.LayeredConfig(n_layers=len(layers), n_above=n_above, n_below=n_below, nr=nr, dr=dr, nz=nz, dz=dz,
                            flags=flags, seed=seed)
    out = np.zeros(len(abi.LAY_FIELDS), np.float64)
    rd, tt, az, al = np.zeros(nr + 1), np.zeros(nr + 1), np.zeros(nz + 1), np.zeros(len(layers))
    pp = np.zeros((photons, 3)) if per_photon else None
    st = lib.orc_layered_run(int(real_bits), C.addressof(cfg), C.addressof(arr), int(first), int(photons),
                             int(nthreads or os.cpu_count() or 1), _ptr(out), _ptr(rd), _ptr(tt), _ptr(az), _ptr(al),
                             _ptr(pp))
    if st != 0:
        raise RuntimeError(f"orc_layered_run failed with status {st}")
    res = {k: out[i] for i, k in enumerate(abi.LAY_FIELDS)}
    n = max(res["photons"], 1.0)
    for k in ("Rd", "Tt"):
        m = res[k] / n
        res[k.lower()] = m
        res[k.lower() + "_se"] = math.sqrt(max(res[k + "2"] / n - m * m, 0.0) / n)
    res.update(rd_r=rd, tt_r=tt, a_z=az, a_layer=al)
    if pp is not None:
        res["per_photon"] = pp
    return res


def efield(cfg: abi.EfieldConfig, S_primary, settings, S_raman=None, cone: bool = False, real_bits: int = 64,
           nthreads: int | None = None) -> dict:
    """The engine's polarised E-field model on the CPU (orc_efield_run): the
    per-setting sums of nmc_gb300.efield.run (keys abi.EF_FIELDS), each an
    array over `settings`."""
    lib = oracle_lib()
    n = len(settings)
    arr = (abi.EfieldSetting * n)(*settings)
    S0 = np.ascontiguousarray(S_primary, np.float32)
    S1 = None if S_raman is None else np.ascontiguousarray(S_raman, np.float32)
    out = np.zeros((n, len(abi.EF_FIELDS)), np.float64)
    st = lib.orc_efield_run(int(real_bits), C.addressof(cfg), _ptr(S0), _ptr(S1), C.addressof(arr), n, int(cone),
                            int(nthreads or os.cpu_count() or 1), _ptr(out))
    if st != 0:
        raise RuntimeError(f"orc_efield_run failed with status {st}")
    return {k: out[:, i] for i, k in enumerate(abi.EF_FIELDS)}
