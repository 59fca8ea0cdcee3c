"""nmc_mcxyz_run_noalloc: the voxel transport for callers that cannot let a
library allocate device memory (they own a memory pool or a fixed budget).
The test plays such a caller: it owns the device buffers and passes them in,
then checks two calls in a row against the regular entry point (nmc_prepare
+ nmc_run on a fresh handle) for the same photons, for both voxel kernels
and both random streams, and with the optional outputs left out.

This file is collected last on purpose (test_zz_*).
"""
import ctypes as C
import math

import numpy as np
import pytest

from nmc_gb300 import abi
import nmc_cases as cases

pytestmark = pytest.mark.gpu

EINVAL = {v: k for k, v in abi.STATUS.items()}["NMC_EINVAL"]


def _bind(lib):
    f = lib.nmc_mcxyz_run_noalloc
    f.restype = C.c_int
    f.argtypes = [C.POINTER(abi.RunParams), C.POINTER(abi.TissueParams), C.POINTER(abi.Ext), C.c_void_p,
                  C.c_uint64, C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    return f


def _case(kind, rng):
    rp, tp, v, ext = cases.skin_vessel_case(N=48, rng=rng)
    if kind == "two-term":
        rp.mckernelflag = abi.SIM_MCXYZ_TT
        rp.boundaryflag = 1
        for t in range(1, 5):
            tp.gf[t], tp.af[t], tp.gb[t], tp.ab[t], tp.CC[t] = 0.9, 0.5, 0.3, 0.5, 0.9
    if rng == abi.RNG_TAUS_REF:
        ext.photons_per_dispatch = 20_000  # the reference's streams depend on the batch size
    return rp, tp, v, ext


@pytest.mark.parametrize("kind,rng", [("one-term", abi.RNG_PHILOX), ("two-term", abi.RNG_PHILOX),
                                      ("one-term", abi.RNG_TAUS_REF)])
def test_noalloc_matches_regular_entry_point_twice(gpu, kind, rng):
    import torch

    run_noalloc = _bind(gpu.lib())
    rp, tp, v, ext = _case(kind, rng)
    sim = rp.mckernelflag
    nvox, n2d = rp.Nx * rp.Ny * rp.Nz, rp.Nx * rp.Ny
    dev = torch.device("cuda:0")
    torch.cuda.set_device(0)
    d_v = torch.from_numpy(v).to(dev)
    d_F3D = torch.full((nvox,), -1.0, dtype=torch.float32, device=dev)
    d_Rd2D = torch.full((n2d,), -1.0, dtype=torch.float32, device=dev)
    d_Det = torch.full((n2d,), -1, dtype=torch.int32, device=dev)
    d_tot = torch.zeros(8, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)

    for first, n in ((0, 40_000), (40_000, 25_000)):
        st = run_noalloc(C.byref(rp), C.byref(tp), C.byref(ext), d_v.data_ptr(), first, n, d_F3D.data_ptr(),
                         d_Rd2D.data_ptr(), d_Det.data_ptr(), d_tot.data_ptr(), stream.cuda_stream)
        assert st == 0, abi.STATUS.get(st, st)
        torch.cuda.synchronize()
        with gpu.Engine(sim, 0, ext) as e:
            e.prepare_data(rp, tp, v)
            e.run(first, n)
            F = e.tally(abi.TALLY_F3D)
            R = e.tally(abi.TALLY_RD2D)
            D = e.tally(abi.TALLY_DETPHOT2D)
            s = e.summary()
        # same photon streams, same integer tallies: equal up to float rounding
        np.testing.assert_allclose(d_F3D.cpu().numpy(), F, rtol=1e-6, atol=1e-12)
        np.testing.assert_allclose(d_Rd2D.cpu().numpy(), R, rtol=1e-6, atol=1e-12)
        assert np.array_equal(d_Det.cpu().numpy().astype(np.float64), D)
        tot = d_tot.cpu().numpy()
        assert tot[0] == n == s["photons"]
        assert tot[1] == s["substeps"]
        assert tot[4] == pytest.approx(s["rd_sum"], rel=1e-12)
        assert tot[3] == pytest.approx(s["A"], rel=1e-12)
        assert tot[6] == 0.0  # no device flag raised


def test_noalloc_optional_outputs_may_be_null(gpu):
    import torch

    run_noalloc = _bind(gpu.lib())
    rp, tp, v, ext = _case("one-term", abi.RNG_PHILOX)
    nvox = rp.Nx * rp.Ny * rp.Nz
    d_v = torch.from_numpy(v).to("cuda:0")
    d_F3D = torch.full((nvox,), -1.0, dtype=torch.float32, device="cuda:0")
    stream = torch.cuda.current_stream()
    st = run_noalloc(C.byref(rp), C.byref(tp), C.byref(ext), d_v.data_ptr(), 0, 20_000, d_F3D.data_ptr(),
                     None, None, None, stream.cuda_stream)
    assert st == 0, abi.STATUS.get(st, st)
    torch.cuda.synchronize()
    with gpu.Engine(abi.SIM_MCXYZ, 0, ext) as e:
        e.prepare_data(rp, tp, v)
        e.run(0, 20_000)
        F = e.tally(abi.TALLY_F3D)
    np.testing.assert_allclose(d_F3D.cpu().numpy(), F, rtol=1e-6, atol=1e-12)


def test_noalloc_rejects_grids_beyond_its_limit(gpu):
    import torch

    run_noalloc = _bind(gpu.lib())
    rp, tp, v, ext = cases.skin_vessel_case(N=8)
    rp.Nx = rp.Ny = 256
    rp.Nz = 64  # 256*256*64 = 4,194,304 voxels > NMC_NOALLOC_MAX_VOXELS
    d = torch.zeros(16, dtype=torch.float32, device="cuda:0")
    st = run_noalloc(C.byref(rp), C.byref(tp), C.byref(ext), d.data_ptr(), 0, 10, d.data_ptr(), None, None,
                     None, torch.cuda.current_stream().cuda_stream)
    assert st == EINVAL  # before any device work


def test_noalloc_rejects_what_the_regular_entry_point_rejects(gpu):
    # a NaN two-term phase term and a tissue id past the 19-entry table are
    # refused with NMC_EINVAL, as nmc_prepare refuses them; the map check runs
    # on the GPU over the caller's own buffer
    import torch

    run_noalloc = _bind(gpu.lib())
    rp, tp, v, ext = _case("two-term", abi.RNG_PHILOX)
    nvox = rp.Nx * rp.Ny * rp.Nz
    d_F3D = torch.zeros(nvox, dtype=torch.float32, device="cuda:0")
    stream = torch.cuda.current_stream().cuda_stream

    bad_tp = abi.TissueParams.from_buffer_copy(tp)
    bad_tp.gf[2] = math.nan
    d_v = torch.from_numpy(v).to("cuda:0")
    st = run_noalloc(C.byref(rp), C.byref(bad_tp), C.byref(ext), d_v.data_ptr(), 0, 100, d_F3D.data_ptr(),
                     None, None, None, stream)
    assert st == EINVAL

    bad_v = v.copy()
    bad_v[nvox // 2] = 19
    d_bad = torch.from_numpy(bad_v).to("cuda:0")
    st = run_noalloc(C.byref(rp), C.byref(tp), C.byref(ext), d_bad.data_ptr(), 0, 100, d_F3D.data_ptr(),
                     None, None, None, stream)
    assert st == EINVAL

    # the entry point stays usable after the refusals
    st = run_noalloc(C.byref(rp), C.byref(tp), C.byref(ext), d_v.data_ptr(), 0, 100, d_F3D.data_ptr(),
                     None, None, None, stream)
    assert st == 0
    torch.cuda.synchronize()
    assert float(d_F3D.sum()) > 0.0
