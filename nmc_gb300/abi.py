"""ctypes mirror of include/nmc_abi.h.

The two configuration structs are byte-identical to the reference's
``struct RunParams`` (172 bytes) and ``struct TissueParams`` (608 bytes),
NMC/NMCCode/definitions.h:186-218.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

NTISS = 19  # definitions.h:57 Ntiss
STRLEN = 32  # definitions.h:58

PHOTON_TOTAL_DEFAULT = 100000  # definitions.h:16
PHOTON_BATCH_DEFAULT = 10000  # definitions.h:17
MCSUB_BINS_DEFAULT = 101  # definitions.h:31
MCSUB_DR_DEFAULT = 0.0020  # definitions.h:52
MCSUB_DZ_DEFAULT = 0.0020  # definitions.h:53

# enum MC_SIM_TYPE, definitions.h:151-164
SIM_MCSUB = 0
SIM_MCXYZ = 1
SIM_MCXYZ_TT = 2
SIM_POLARIZATION_CBS_ELECTRIC_FIELDS = 3
SIM_POLARIZATION_MUELLER_STOKES = 4
SIM_RAMAN = 5

DET_REFLECTANCE = 0
DET_TRANSMITTANCE = 1

RNG_PHILOX = 0
RNG_TAUS_REF = 1

PHASE_HG = 0
PHASE_ISOTROPIC_REF = 1
PHASE_TWO_TERM = 2

FLAG_TT_REPLAY_RUN1 = 1 << 0
FLAG_NO_HARD_KILL = 1 << 1
FLAG_PRECISE_MATH = 1 << 2
FLAG_SKIP_FLUENCE = 1 << 3
FLAG_GLOBAL_TALLIES = 1 << 4
FLAG_LAYERED_REF_STREAMS = 1 << 5
FLAG_LAYERED_ISOTROPIC = 1 << 6
FLAG_NO_L2_PERSIST = 1 << 7

FATE_ALIVE, FATE_ESCAPED, FATE_ROULETTE, FATE_MINWEIGHT, FATE_MAXSCATT, FATE_BOUNDARY, FATE_STEPCAP = range(7)

TALLY_J, TALLY_F, TALLY_F3D, TALLY_RD2D, TALLY_DETPHOT2D, TALLY_RD_SLOTS, TALLY_RD_R = range(7)

STATUS = {
    0: "NMC_OK",
    1: "NMC_EINVAL",
    2: "NMC_EIO",
    3: "NMC_EDEVICE",
    4: "NMC_ETIMEOUT",
    5: "NMC_ESTEPCAP",
    6: "NMC_ENOMEM",
    7: "NMC_EUNSUPPORTED",
    8: "NMC_ESTATE",
}


class RunParams(C.Structure):
    """struct RunParams (definitions.h:186-209)."""

    _fields_ = [
        ("myname", C.c_char * STRLEN),
        ("mcflag", C.c_int32),
        ("launchflag", C.c_int32),
        ("boundaryflag", C.c_int32),
        ("speckleflag", C.c_int32),
        ("semiflag", C.c_int32),
        ("xfocus", C.c_float),
        ("yfocus", C.c_float),
        ("zfocus", C.c_float),
        ("ux0", C.c_float),
        ("uy0", C.c_float),
        ("uz0", C.c_float),
        ("radius", C.c_float),
        ("det_radius", C.c_float),
        ("xd", C.c_float),
        ("waist", C.c_float),
        ("zsurf", C.c_float),
        ("n1", C.c_float),
        ("n2", C.c_float),
        ("na", C.c_float),
        ("lambda_", C.c_float),
        ("lc", C.c_float),
        ("det_state", C.c_int32),
        ("ph_quant", C.c_int32),
        ("dx", C.c_float),
        ("dy", C.c_float),
        ("dz", C.c_float),
        ("Nx", C.c_int32),
        ("Ny", C.c_int32),
        ("Nz", C.c_int32),
        ("Nt", C.c_int32),
        ("xs", C.c_float),
        ("ys", C.c_float),
        ("zs", C.c_float),
        ("time_min", C.c_float),
        ("mckernelflag", C.c_int32),
    ]


class TissueParams(C.Structure):
    """struct TissueParams (definitions.h:211-218)."""

    _fields_ = [
        ("muav", C.c_float * NTISS),
        ("musv", C.c_float * NTISS),
        ("gv", C.c_float * NTISS),
        ("gf", C.c_float * NTISS),
        ("af", C.c_float * NTISS),
        ("gb", C.c_float * NTISS),
        ("ab", C.c_float * NTISS),
        ("CC", C.c_float * NTISS),
    ]


class Ext(C.Structure):
    """nmc_ext: the knobs that are compile-time #defines in the reference."""

    _fields_ = [
        ("size", C.c_uint32),
        ("rng", C.c_uint32),
        ("seed", C.c_uint64),
        ("phase", C.c_uint32),
        ("flags", C.c_uint32),
        ("photons_per_dispatch", C.c_uint64),
        ("photons_total", C.c_uint64),
        ("sub_bins", C.c_int32),
        ("sub_dr", C.c_float),
        ("sub_dz", C.c_float),
        ("sub_mcflag", C.c_int32),
        ("sub_boundaryflag", C.c_int32),
        ("sub_radius", C.c_float),
        ("sub_waist", C.c_float),
        ("sub_zfocus", C.c_float),
        ("sub_xs", C.c_float),
        ("sub_ys", C.c_float),
        ("sub_zs", C.c_float),
        ("block_size", C.c_int32),
        ("blocks_per_sm", C.c_int32),
        ("timeout_s", C.c_double),
        ("photons_per_fetch", C.c_uint32),
        ("reserved", C.c_uint32 * 7),
    ]


class EfieldConfig(C.Structure):
    """nmc_efield_config."""

    _fields_ = [("mua", C.c_float), ("mus", C.c_float), ("wavelength_cm", C.c_float),
                ("raman_mua", C.c_float), ("raman_mus", C.c_float), ("raman_wavelength_cm", C.c_float),
                ("mu_raman", C.c_float), ("n_medium", C.c_float), ("n_outside", C.c_float),
                ("n_angles", C.c_int32), ("cone_n", C.c_int32), ("cone_half_angle", C.c_float),
                ("sep_n", C.c_int32), ("sep_half_width", C.c_float), ("map_n", C.c_int32), ("map_dx", C.c_float),
                ("depth_bins", C.c_int32), ("depth_dz", C.c_float), ("seed", C.c_uint64), ("flags", C.c_uint32),
                ("speckle_max", C.c_uint32)]


class EfieldSetting(C.Structure):
    """nmc_efield_setting."""

    _fields_ = [("pol_angle", C.c_float), ("theta_in", C.c_float), ("phi_in", C.c_float), ("pad", C.c_uint32),
                ("photons", C.c_uint64)]


EF_FIELDS = ("photons", "specular", "Rd", "Rd2", "co", "cross", "multi_co", "multi_cross", "interf_co",
             "interf_cross", "sep_outside", "raman_n", "raman_Rd", "raman_co", "raman_cross", "scatters")
EF_MAPS = ("XX", "XY", "YX", "YY", "Rd", "Det", "Phase0", "Phase1", "Phase2", "Phase3")
EF_MAX_ORDER = 150
# struct SPECKLE (definitions.h:220-229) / nmc_speckle
SPECKLE_DTYPE = np.dtype([("Phase", "<f4"), ("Path", "<f4"), ("Scatt", "<f4"), ("Total", "<f4"), ("XX", "<f4"),
                          ("XY", "<f4"), ("Ryx", "<f4")])


class Layer(C.Structure):
    """nmc_layer."""

    _fields_ = [("mua", C.c_float), ("mus", C.c_float), ("g", C.c_float), ("n", C.c_float), ("thickness", C.c_float)]


class LayeredConfig(C.Structure):
    """nmc_layered_config."""

    _fields_ = [("n_layers", C.c_int32), ("n_above", C.c_float), ("n_below", C.c_float), ("nr", C.c_int32),
                ("dr", C.c_float), ("nz", C.c_int32), ("dz", C.c_float), ("flags", C.c_uint32), ("seed", C.c_uint64)]


LAY_FIELDS = ("photons", "specular", "Rd", "Rd2", "Tt", "Tt2", "A", "interactions")


class TuneEntry(C.Structure):
    """nmc_tune_entry."""

    _fields_ = [("block_size", C.c_int32), ("blocks_per_sm", C.c_int32), ("flags", C.c_uint32),
                ("photons_per_fetch", C.c_uint32), ("ms", C.c_float)]


class TuneResult(C.Structure):
    """nmc_tune_result."""

    _fields_ = [("best", TuneEntry), ("fallback", TuneEntry), ("n_tried", C.c_int32), ("tried", TuneEntry * 48)]


class Summary(C.Structure):
    """nmc_summary."""

    _fields_ = [
        ("photons", C.c_uint64),
        ("substeps", C.c_uint64),
        ("scatters", C.c_uint64),
        ("S", C.c_double),
        ("A", C.c_double),
        ("E", C.c_double),
        ("rd_sum", C.c_double),
        ("rd_sumsq", C.c_double),
        ("kernel_ms", C.c_double),
        ("launches", C.c_uint32),
        ("device_flags", C.c_uint32),
    ]


class PhotonRecord(C.Structure):
    """nmc_photon_record (per-photon trace)."""

    _fields_ = [
        ("n_scatt", C.c_uint32),
        ("n_sub", C.c_uint32),
        ("fate", C.c_uint32),
        ("n_detect", C.c_uint32),
        ("w_final", C.c_float),
        ("absorbed", C.c_float),
        ("detected", C.c_float),
        ("x", C.c_float),
        ("y", C.c_float),
        ("z", C.c_float),
    ]


class SweepSet(C.Structure):
    """nmc_sweep_set: one parameter set of a batched sweep."""

    _fields_ = [
        ("mua", C.c_float),
        ("mus", C.c_float),
        ("g", C.c_float),
        ("gf", C.c_float),
        ("af", C.c_float),
        ("gb", C.c_float),
        ("ab", C.c_float),
        ("cc", C.c_float),
        ("n1", C.c_float),
        ("n2", C.c_float),
        ("pad", C.c_uint32),
        ("photons", C.c_uint64),
        ("first_photon", C.c_uint64),
    ]


SWEEP_FIELDS = ("photons", "hops", "S", "A", "E", "E2", "Rd", "Rd_se")

PHOTON_RECORD_DTYPE = np.dtype(
    [
        ("n_scatt", np.uint32),
        ("n_sub", np.uint32),
        ("fate", np.uint32),
        ("n_detect", np.uint32),
        ("w_final", np.float32),
        ("absorbed", np.float32),
        ("detected", np.float32),
        ("x", np.float32),
        ("y", np.float32),
        ("z", np.float32),
    ]
)

assert C.sizeof(RunParams) == 172
assert RunParams.n1.offset == 96 and RunParams.det_state.offset == 116
assert RunParams.dx.offset == 124 and RunParams.Nx.offset == 136
assert RunParams.xs.offset == 152 and RunParams.mckernelflag.offset == 168
assert C.sizeof(TissueParams) == 608
assert C.sizeof(PhotonRecord) == PHOTON_RECORD_DTYPE.itemsize == 40


def ext_defaults(**kw) -> Ext:
    """nmc_ext with the reference's compile-time constants (definitions.h:16-54)."""
    e = Ext()
    e.size = C.sizeof(Ext)
    e.rng = RNG_PHILOX
    e.seed = 0
    e.phase = PHASE_HG
    e.flags = 0
    e.photons_per_dispatch = PHOTON_BATCH_DEFAULT
    e.photons_total = PHOTON_TOTAL_DEFAULT
    e.sub_bins = MCSUB_BINS_DEFAULT
    e.sub_dr = MCSUB_DR_DEFAULT
    e.sub_dz = MCSUB_DZ_DEFAULT
    e.sub_mcflag = 0  # mcflag_mcsub
    e.sub_boundaryflag = 1  # boundaryflag_mcsub
    e.sub_radius = 0.0  # radius_mcsub
    e.sub_waist = 0.10  # waist_mcsub
    e.sub_zfocus = 1.0  # zfocus_mcsub
    e.sub_xs = 0.0
    e.sub_ys = 0.0
    e.sub_zs = 0.0
    e.block_size = 0
    e.blocks_per_sm = 0
    e.timeout_s = 600.0
    for k, v in kw.items():
        if not hasattr(e, k):
            raise AttributeError(f"nmc_ext has no field {k!r}")
        setattr(e, k, v)
    return e


def run_params(**kw) -> RunParams:
    """RunParams with the given fields (others zero)."""
    rp = RunParams()
    for k, v in kw.items():
        if k == "lambda":
            k = "lambda_"
        if k == "myname":
            v = v.encode() if isinstance(v, str) else v
        if not hasattr(rp, k):
            raise AttributeError(f"RunParams has no field {k!r}")
        setattr(rp, k, v)
    return rp


def tissue_params(mua=(), mus=(), g=(), gf=None, af=None, gb=None, ab=None, cc=None) -> TissueParams:
    """TissueParams from per-tissue lists for tissue ids 1..len(mua) (index 0 unused, mcio.h:128)."""
    tp = TissueParams()

    def put(arr, vals):
        if vals is None:
            return
        vals = list(vals)
        if len(vals) > NTISS - 1:
            raise ValueError(f"at most {NTISS - 1} tissues")
        for i, v in enumerate(vals, start=1):
            arr[i] = float(v)

    put(tp.muav, mua)
    put(tp.musv, mus)
    put(tp.gv, g)
    put(tp.gf, gf)
    put(tp.af, af)
    put(tp.gb, gb)
    put(tp.ab, ab)
    put(tp.CC, cc)
    return tp
