"""Python face of the engine: a ctypes wrapper over include/nmc_abi.h.

``Engine`` mirrors the reference's host class (NMC/NMCCode/MetalMC.h:25-31):

    MetalMC initWithDevice:kernel_type  -> Engine(sim_type, device)
    prepareData: run_params tiss v      -> Engine.prepare_data(rp, tp, v)
    setNumRunsSeed:                     -> Engine.set_num_runs_seed(run, seed)
    sendComputeCommand                  -> Engine.send_compute_command()
    getComputeResults: (16 arrays)      -> Engine.get_compute_results(...)

plus whole-job calls (``run``, ``summary``, ``tally``).  There is no CPU
fallback: constructing an Engine without the built library raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi

_BUILD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "_build")
# NMC_CHECKED=1 selects the checked build (every tally index tested)
LIB_PATH = os.path.join(_BUILD, "checked" if os.environ.get("NMC_CHECKED") == "1" else "", "libnmc_gb300.so")

_lib = None
_P = C.c_void_p


class NMCError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{abi.STATUS.get(status, status)}: {msg}")
        self.status = status


def lib() -> C.CDLL:
    """The loaded engine library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FileNotFoundError(
                f"engine library {LIB_PATH} is missing; build it with `python -m nmc_gb300.build`")
        L = C.CDLL(LIB_PATH)
        H = C.c_void_p
        L.nmc_ext_defaults.argtypes = [C.POINTER(abi.Ext)]
        L.nmc_abi_version.restype = C.c_int32
        L.nmc_create.argtypes = [C.c_int32, C.c_int32, C.POINTER(H)]
        L.nmc_prepare.argtypes = [H, C.POINTER(abi.RunParams), C.POINTER(abi.TissueParams), _P]
        L.nmc_set_ext.argtypes = [H, C.POINTER(abi.Ext)]
        L.nmc_set_tissue_params.argtypes = [H, C.POINTER(abi.TissueParams)]
        L.nmc_set_num_runs_seed.argtypes = [H, C.c_int32, C.c_float]
        L.nmc_send_compute_command.argtypes = [H]
        L.nmc_run.argtypes = [H, C.c_uint64, C.c_uint64]
        L.nmc_run_async.argtypes = [H, C.c_uint64, C.c_uint64]
        L.nmc_synchronize.argtypes = [H]
        L.nmc_run_traced.argtypes = [H, C.c_uint64, C.c_uint64, _P, _P, C.c_uint32]
        L.nmc_get_compute_results.argtypes = [H] + [_P] * 16
        L.nmc_get_summary.argtypes = [H, C.POINTER(abi.Summary)]
        L.nmc_get_tally_f64.argtypes = [H, C.c_int32, _P, C.c_size_t]
        L.nmc_set_fold_interval.argtypes = [H, C.c_uint64]
        L.nmc_tally_size.argtypes = [H, C.c_int32]
        L.nmc_tally_size.restype = C.c_size_t
        L.nmc_reset.argtypes = [H]
        L.nmc_stream.argtypes = [H]
        L.nmc_stream.restype = C.c_void_p
        L.nmc_last_error.argtypes = [H]
        L.nmc_last_error.restype = C.c_char_p
        L.nmc_destroy.argtypes = [H]
        L.nmc_probe_issue_peaks.argtypes = [C.c_int32, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.nmc_run_sweep.argtypes = [H, C.POINTER(abi.SweepSet), C.c_int32, _P, _P]
        L.nmc_run_sweep.restype = C.c_int
        L.nmc_autotune.argtypes = [H, C.c_uint64, C.POINTER(abi.TuneResult)]
        L.nmc_autotune.restype = C.c_int
        L.nmc_run_sweep_tissues.argtypes = [H, C.POINTER(abi.TissueParams), _P, _P, C.c_int32, _P]
        L.nmc_run_sweep_tissues.restype = C.c_int
        L.nmc_set_voxel_props.argtypes = [H, _P, _P, _P]
        L.nmc_set_radial_tally.argtypes = [H, C.c_int32, C.c_float]
        L.nmc_adjoint_forward.argtypes = [H, C.c_uint64, C.c_uint64, C.c_uint64]
        L.nmc_adjoint_forward_ex.argtypes = [H, C.c_uint64, C.c_uint64, C.c_uint64, C.c_uint64]
        L.nmc_adjoint_deposit_list_complete.argtypes = [H]
        L.nmc_adjoint_deposit_list_complete.restype = C.c_int32
        L.nmc_adjoint_backward.argtypes = [H, _P, _P, _P, _P]
        L.nmc_adjoint_backward_ex.argtypes = [H, _P, _P, _P, _P, _P]
        for name in ("nmc_create", "nmc_prepare", "nmc_set_ext", "nmc_set_tissue_params", "nmc_set_num_runs_seed",
                     "nmc_send_compute_command", "nmc_run", "nmc_run_async", "nmc_synchronize",
                     "nmc_run_traced", "nmc_get_compute_results", "nmc_get_summary",
                     "nmc_get_tally_f64", "nmc_reset", "nmc_set_voxel_props", "nmc_set_radial_tally",
                     "nmc_adjoint_forward", "nmc_adjoint_forward_ex", "nmc_adjoint_backward",
                     "nmc_adjoint_backward_ex"):
            getattr(L, name).restype = C.c_int
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(_P)


def probe_issue_peaks(device: int = 0) -> tuple[float, float]:
    """Measured FP32 FMA lanes/s and MUFU lanes/s of `device`."""
    f, m = C.c_double(), C.c_double()
    st = lib().nmc_probe_issue_peaks(int(device), C.byref(f), C.byref(m))
    if st != 0:
        raise NMCError(st, "nmc_probe_issue_peaks")
    return f.value, m.value


class Engine:
    """One simulation handle on one GPU (not thread-safe; one per host thread)."""

    def __init__(self, sim_type: int, device: int = 0, ext: abi.Ext | None = None):
        self._L = lib()
        self._h = C.c_void_p()
        st = self._L.nmc_create(int(sim_type), int(device), C.byref(self._h))
        if st != 0:
            raise NMCError(st, f"nmc_create(sim_type={sim_type}, device={device})")
        self.sim_type = int(sim_type)
        self.ext = ext or abi.ext_defaults()
        self._check(self._L.nmc_set_ext(self._h, C.byref(self.ext)), "nmc_set_ext")
        self.rp: abi.RunParams | None = None

    # -- plumbing
    def _check(self, st: int, what: str):
        if st != 0:
            msg = self._L.nmc_last_error(self._h) if self._h else b""
            raise NMCError(st, f"{what}: {msg.decode(errors='replace') if msg else ''}")

    def close(self):
        if getattr(self, "_h", None):
            self._L.nmc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- reference lifecycle
    def set_ext(self, ext: abi.Ext):
        self.ext = ext
        self._check(self._L.nmc_set_ext(self._h, C.byref(ext)), "nmc_set_ext")

    def prepare_data(self, rp: abi.RunParams, tp: abi.TissueParams, v=None):
        self.rp = rp
        vv = None if v is None else np.ascontiguousarray(v, dtype=np.uint8).ravel()
        self._check(self._L.nmc_prepare(self._h, C.byref(rp), C.byref(tp), _ptr(vv)), "nmc_prepare")

    def set_tissue_params(self, tp: abi.TissueParams):
        """Swap the tissue table (e.g. the next wavelength) keeping the map."""
        self._check(self._L.nmc_set_tissue_params(self._h, C.byref(tp)), "nmc_set_tissue_params")

    def set_num_runs_seed(self, run: int, time_seed: float = 0.0):
        self._check(self._L.nmc_set_num_runs_seed(self._h, int(run), float(time_seed)), "nmc_set_num_runs_seed")

    def send_compute_command(self):
        self._check(self._L.nmc_send_compute_command(self._h), "nmc_send_compute_command")

    def get_compute_results(self) -> dict:
        """Reference-layout float arrays (getComputeResults, MetalMC.m:508-824)."""
        out: dict = {}
        J = F = F3D = SAE = Rd = Rd2D = Det = None
        if self.sim_type == abi.SIM_MCSUB:
            b = self.ext.sub_bins
            J = out["J"] = np.zeros(b + 1, np.float32)
            F = out["F"] = np.zeros((b + 1) * (b + 1), np.float32)
            SAE = out["SAE"] = np.zeros(3, np.float32)
        else:
            rp = self.rp
            F3D = out["F3D"] = np.zeros(rp.Nx * rp.Ny * rp.Nz, np.float32)
            Rd = out["Rd"] = np.zeros(self.ext.photons_per_dispatch, np.float32)
            Rd2D = out["Rd2D"] = np.zeros(rp.Nx * rp.Ny, np.float32)
            Det = out["DetPhot2D"] = np.zeros(rp.Nx * rp.Ny, np.int32)
        args = [J, F, F3D, SAE, Rd, Rd2D, Det] + [None] * 9
        self._check(self._L.nmc_get_compute_results(self._h, *[_ptr(a) for a in args]),
                    "nmc_get_compute_results")
        return out

    # -- whole-job calls
    def run(self, first: int, n: int):
        self._check(self._L.nmc_run(self._h, int(first), int(n)), "nmc_run")

    def run_async(self, first: int, n: int):
        self._check(self._L.nmc_run_async(self._h, int(first), int(n)), "nmc_run_async")

    def synchronize(self):
        self._check(self._L.nmc_synchronize(self._h), "nmc_synchronize")

    def run_traced(self, first: int, n: int, k_events: int = 0):
        recs = np.zeros(n, abi.PHOTON_RECORD_DTYPE)
        ev = np.zeros((n, k_events, 4), np.float32) if k_events else None
        self._check(self._L.nmc_run_traced(self._h, int(first), int(n), _ptr(recs), _ptr(ev), int(k_events)),
                    "nmc_run_traced")
        return recs, ev

    def summary(self) -> dict:
        s = abi.Summary()
        self._check(self._L.nmc_get_summary(self._h, C.byref(s)), "nmc_get_summary")
        return {k: getattr(s, k) for k, _ in abi.Summary._fields_}

    def tally(self, which: int) -> np.ndarray:
        n = self._L.nmc_tally_size(self._h, int(which))
        out = np.zeros(n, np.float64)
        self._check(self._L.nmc_get_tally_f64(self._h, int(which), _ptr(out), n), "nmc_get_tally_f64")
        return out

    def reset(self):
        self._check(self._L.nmc_reset(self._h), "nmc_reset")

    def set_fold_interval(self, photons: int):
        """Photons between folds of the fixed-point tallies into FP64 (default 2^31)."""
        self._check(self._L.nmc_set_fold_interval(self._h, int(photons)), "nmc_set_fold_interval")

    def run_sweep(self, sets, with_J: bool = False) -> dict:
        """Batched sweep (mcsub handle): `sets` is a sequence of abi.SweepSet.
        Returns per-set arrays named as abi.SWEEP_FIELDS (and J if asked)."""
        n = len(sets)
        arr = (abi.SweepSet * n)(*sets)
        out = np.zeros((n, len(abi.SWEEP_FIELDS)), np.float64)
        J = np.zeros((n, self.ext.sub_bins + 1), np.float64) if with_J else None
        self._check(self._L.nmc_run_sweep(self._h, arr, n, _ptr(out), _ptr(J)), "nmc_run_sweep")
        res = {k: out[:, i] for i, k in enumerate(abi.SWEEP_FIELDS)}
        if with_J:
            res["J"] = J
        return res

    def autotune(self, photons: int = 200_000) -> dict:
        """Times the kernel under candidate launch shapes on photons
        [0, photons), keeps the fastest in the handle and clears the tallies."""
        r = abi.TuneResult()
        self._check(self._L.nmc_autotune(self._h, int(photons), C.byref(r)), "nmc_autotune")

        def d(t):
            return {"block_size": t.block_size, "blocks_per_sm": t.blocks_per_sm, "flags": t.flags,
                    "photons_per_fetch": t.photons_per_fetch, "ms": t.ms}

        self.ext.block_size = r.best.block_size
        self.ext.blocks_per_sm = r.best.blocks_per_sm
        self.ext.photons_per_fetch = r.best.photons_per_fetch
        self.ext.flags = (self.ext.flags & ~abi.FLAG_GLOBAL_TALLIES) | r.best.flags
        return {"best": d(r.best), "default": d(r.fallback), "tried": [d(r.tried[i]) for i in range(r.n_tried)]}

    def run_sweep_tissues(self, tables, photons, first_photon=None) -> dict:
        """Batched sweep on a voxel tissue map (mcxyz handle): set s runs
        photons[s] photons with tissue table tables[s] (abi.TissueParams).
        Returns per-set arrays named as abi.SWEEP_FIELDS."""
        n = len(tables)
        arr = (abi.TissueParams * n)(*tables)
        ph = np.ascontiguousarray(photons, dtype=np.uint64)
        fp = None if first_photon is None else np.ascontiguousarray(first_photon, dtype=np.uint64)
        if ph.size != n or (fp is not None and fp.size != n):
            raise ValueError("one photon budget (and first photon) per table")
        out = np.zeros((n, len(abi.SWEEP_FIELDS)), np.float64)
        self._check(self._L.nmc_run_sweep_tissues(self._h, arr, _ptr(ph), _ptr(fp), n, _ptr(out)),
                    "nmc_run_sweep_tissues")
        return {k: out[:, i] for i, k in enumerate(abi.SWEEP_FIELDS)}

    # -- per-voxel media and the perturbation Monte Carlo adjoint
    def set_voxel_props(self, mua, mus, g=None):
        """Per-voxel mua, mus (1/cm) and HG g, arrays of Nz x Nx x Ny (the
        engine's voxel order iz*Ny*Nx + ix*Ny + iy) or flat."""
        a = np.ascontiguousarray(mua, dtype=np.float32).ravel()
        s = np.ascontiguousarray(mus, dtype=np.float32).ravel()
        gg = None if g is None else np.ascontiguousarray(g, dtype=np.float32).ravel()
        n = self.rp.Nx * self.rp.Ny * self.rp.Nz
        if a.size != n or s.size != n or (gg is not None and gg.size != n):
            raise ValueError(f"per-voxel arrays need {n} values")
        self._check(self._L.nmc_set_voxel_props(self._h, _ptr(a), _ptr(s), _ptr(gg)), "nmc_set_voxel_props")

    def set_radial_tally(self, bins: int, dr: float):
        self._check(self._L.nmc_set_radial_tally(self._h, int(bins), float(dr)), "nmc_set_radial_tally")

    def adjoint_forward(self, first: int, n: int, event_capacity: int | None = None, deposit_capacity: int = 0):
        """The record pass of the adjoint; deposit_capacity > 0 also keeps the
        deposit list (8 bytes a record) that spares a fluence-loss backward
        its score replay."""
        cap = int(event_capacity) if event_capacity else max(1 << 20, 4 * int(n))
        self._check(self._L.nmc_adjoint_forward_ex(self._h, int(first), int(n), cap, int(deposit_capacity)),
                    "nmc_adjoint_forward_ex")

    @property
    def deposit_list_complete(self) -> bool:
        return bool(self._L.nmc_adjoint_deposit_list_complete(self._h))

    def adjoint_backward(self, grad_rd_r=None, grad_absorbed=None):
        """(grad_mua, grad_mus, grad_g) per voxel for the upstream gradients of
        the un-normalised radial tally (bins + 1 values) and of the absorbed
        weight per voxel (NMC_TALLY_F3D); either may be None, not both."""
        n = self.rp.Nx * self.rp.Ny * self.rp.Nz
        G = GF = None
        if grad_rd_r is not None:
            G = np.ascontiguousarray(grad_rd_r, dtype=np.float32).ravel()
            nb = self._L.nmc_tally_size(self._h, abi.TALLY_RD_R)
            if G.size != nb:
                raise ValueError(f"grad_rd_r needs {nb} values")
        if grad_absorbed is not None:
            GF = np.ascontiguousarray(grad_absorbed, dtype=np.float32).ravel()
            if GF.size != n:
                raise ValueError(f"grad_absorbed needs {n} values")
        ga, gs, gg = (np.zeros(n, np.float64) for _ in range(3))
        self._check(self._L.nmc_adjoint_backward_ex(self._h, _ptr(G), _ptr(GF), _ptr(ga), _ptr(gs), _ptr(gg)),
                    "nmc_adjoint_backward_ex")
        return ga, gs, gg

    @property
    def stream(self) -> int:
        return self._L.nmc_stream(self._h) or 0
