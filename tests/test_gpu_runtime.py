"""Runtime pieces around the kernels: the autotuner and the graph-captured
result reduction.

Every photon's random stream is a function of its id only, so a launch
shape chosen by the autotuner must leave every integer tally unchanged; and
the reduction graph must return exactly the device tallies, accumulated
(+=) into the caller's arrays as the reference's getComputeResults does
(MetalMC.m:508-538).
"""
import numpy as np
import pytest

from nmc_gb300 import abi
import nmc_cases as cases

pytestmark = pytest.mark.gpu


def _tallies(e, which):
    return {w: e.tally(w) for w in which}


@pytest.mark.parametrize("per", [2, 8])
def test_photons_per_fetch_keeps_results(gpu, per):
    # a thread taking runs of consecutive photons from the queue runs the same
    # photons: every integer tally is equal
    rp, tp, v, ext = cases.skin_vessel_case(N=48)
    out = []
    for p in (1, per):
        ext.photons_per_fetch = p
        with gpu.Engine(abi.SIM_MCXYZ, 0, ext) as e:
            e.prepare_data(rp, tp, v)
            e.run(7, 30_001)
            out.append((_tallies(e, (abi.TALLY_F3D, abi.TALLY_RD2D)), e.summary()))
    for w in (abi.TALLY_F3D, abi.TALLY_RD2D):
        np.testing.assert_array_equal(out[0][0][w], out[1][0][w])
    for k in ("photons", "substeps", "scatters", "rd_sum"):
        assert out[0][1][k] == out[1][1][k], k


@pytest.mark.parametrize("kind", ["mcsub", "mcxyz"])
def test_autotune_keeps_results(gpu, kind):
    if kind == "mcsub":
        rp, tp, ext = cases.mcsub_case()
        sim, v, which, n = abi.SIM_MCSUB, None, (abi.TALLY_J, abi.TALLY_F), 100_000
    else:
        rp, tp, v, ext = cases.skin_vessel_case(N=64)
        sim, which, n = abi.SIM_MCXYZ, (abi.TALLY_F3D, abi.TALLY_RD2D, abi.TALLY_DETPHOT2D), 50_000
    with gpu.Engine(sim, 0, ext) as e:
        e.prepare_data(rp, tp, v)
        e.run(0, n)
        before = _tallies(e, which)
        s0 = e.summary()
        r = e.autotune(50_000)
        print(kind, "default", r["default"], "best", r["best"], "tried", len(r["tried"]))
        assert len(r["tried"]) >= 3
        # runs of several photons per queue fetch are among the shapes tried
        assert {t["photons_per_fetch"] for t in r["tried"]} >= {1, 2, 4, 8}
        assert r["best"]["ms"] <= r["default"]["ms"]
        assert e.summary()["photons"] == 0  # tallies cleared
        e.run(0, n)
        after = _tallies(e, which)
        s1 = e.summary()
    for w in which:
        np.testing.assert_array_equal(before[w], after[w])
    for k in ("photons", "substeps", "scatters", "S", "A", "E", "rd_sum"):
        assert s0[k] == s1[k], k


@pytest.mark.parametrize("kind", ["mcsub", "mcxyz"])
def test_reduction_graph_returns_the_tallies(gpu, kind):
    if kind == "mcsub":
        rp, tp, ext = cases.mcsub_case()
        sim, v, n = abi.SIM_MCSUB, None, 50_000
    else:
        rp, tp, v, ext = cases.skin_vessel_case(N=64)
        sim, n = abi.SIM_MCXYZ, 20_000
    with gpu.Engine(sim, 0, ext) as e:
        e.prepare_data(rp, tp, v)
        e.run(0, n)
        r1 = e.get_compute_results()
        r2 = e.get_compute_results()  # the graph replayed
        if kind == "mcsub":
            ref = {"J": e.tally(abi.TALLY_J), "F": e.tally(abi.TALLY_F)}
            sm = e.summary()
            np.testing.assert_allclose(r1["SAE"], np.float32([sm["S"], sm["A"], sm["E"]]), rtol=1e-6)
        else:
            ref = {"F3D": e.tally(abi.TALLY_F3D), "Rd2D": e.tally(abi.TALLY_RD2D),
                   "DetPhot2D": e.tally(abi.TALLY_DETPHOT2D)}
        for k, want in ref.items():
            np.testing.assert_array_equal(r1[k], want.astype(np.float32).astype(r1[k].dtype))
            np.testing.assert_array_equal(r2[k], r1[k])
        # accumulation into the caller's arrays: a second call adds again
        acc = {k: np.array(r1[k]) for k in r1}
        L = e._L
        if kind == "mcxyz":
            args = [None, None, acc["F3D"], None, acc["Rd"], acc["Rd2D"], acc["DetPhot2D"]] + [None] * 9
        else:
            args = [acc["J"], acc["F"], None, acc["SAE"], None, None, None] + [None] * 9
        from nmc_gb300.engine import _ptr
        e._check(L.nmc_get_compute_results(e._h, *[_ptr(a) for a in args]), "nmc_get_compute_results")
        for k in acc:
            np.testing.assert_allclose(acc[k], 2 * r1[k], rtol=1e-6)


@pytest.mark.parametrize("kind", ["mcsub", "mcxyz"])
def test_folded_tallies_equal_unfolded(gpu, kind):
    # folding the fixed-point tallies into FP64 (here every 7,000 photons,
    # which also splits each run into launches of 7,000) changes no result:
    # every folded part is exact in FP64 at these sizes
    if kind == "mcsub":
        rp, tp, ext = cases.mcsub_case()
        sim, v, which = abi.SIM_MCSUB, None, (abi.TALLY_J, abi.TALLY_F)
    else:
        rp, tp, v, ext = cases.skin_vessel_case(N=48)
        sim, which = abi.SIM_MCXYZ, (abi.TALLY_F3D, abi.TALLY_RD2D, abi.TALLY_DETPHOT2D, abi.TALLY_RD_SLOTS)
    n = 50_000
    out = []
    for interval in (None, 7_000):
        with gpu.Engine(sim, 0, ext) as e:
            e.prepare_data(rp, tp, v)
            if interval:
                e.set_fold_interval(interval)
            e.run(0, n // 2)
            e.run(n // 2, n - n // 2)
            s = e.summary()
            out.append((s, [e.tally(w) for w in which], e.get_compute_results()))
    (s0, t0, r0), (s1, t1, r1) = out
    assert s1["launches"] > s0["launches"]
    for k in ("photons", "substeps", "scatters", "S", "A", "E", "rd_sum"):
        assert s0[k] == s1[k], k
    for a, b in zip(t0, t1):
        np.testing.assert_array_equal(a, b)
    for k in r0:
        np.testing.assert_array_equal(np.asarray(r0[k]), np.asarray(r1[k]), err_msg=k)
    with gpu.Engine(sim, 0, ext) as e:
        with pytest.raises(gpu.NMCError):
            e.set_fold_interval(0)
        with pytest.raises(gpu.NMCError):
            e.set_fold_interval(2 ** 31 + 1)


def test_handles_on_two_host_threads(gpu):
    # one handle per host thread: two handles run concurrently from two
    # threads (each on its own stream) and give the results each gives alone
    import threading

    rp, tp, v, ext = cases.skin_vessel_case(N=48)

    def run(first, out, key):
        with gpu.Engine(abi.SIM_MCXYZ, 0, ext) as e:
            e.prepare_data(rp, tp, v)
            e.run(first, 30_000)
            out[key] = (e.summary(), e.tally(abi.TALLY_F3D))

    alone, together = {}, {}
    run(0, alone, "a")
    run(10_000_000, alone, "b")
    th = [threading.Thread(target=run, args=(f, together, k)) for f, k in ((0, "a"), (10_000_000, "b"))]
    for t in th:
        t.start()
    for t in th:
        t.join()
    for k in ("a", "b"):
        for f in ("photons", "substeps", "S", "A", "E", "rd_sum"):
            assert alone[k][0][f] == together[k][0][f], (k, f)
        np.testing.assert_array_equal(alone[k][1], together[k][1])


def test_current_device_is_kept(gpu):
    # every entry point makes the handle's device current and gives the
    # caller's back; with two GPUs a handle on the second one runs while the
    # first is current and gives the results it gives with its own current
    import torch

    dev = torch.cuda.device_count() - 1
    rp, tp, v, ext = cases.skin_vessel_case(N=32)
    res = {}
    for cur in sorted({0, dev}):
        torch.cuda.set_device(cur)
        with gpu.Engine(abi.SIM_MCXYZ, dev, ext) as e:
            e.prepare_data(rp, tp, v)
            e.run(0, 20_000)
            assert torch.cuda.current_device() == cur
            res[cur] = (e.summary(), e.tally(abi.TALLY_F3D))
        assert torch.cuda.current_device() == cur
    a, b = res[0], res[dev]
    for f in ("photons", "substeps", "S", "A", "E", "rd_sum"):
        assert a[0][f] == b[0][f], f
    np.testing.assert_array_equal(a[1], b[1])


def test_l2_persisting_window_keeps_results(gpu):
    # the fluence tally kept in L2 (the default) or left to the normal policy
    # (NMC_FLAG_NO_L2_PERSIST) is a cache hint only: every tally is equal
    rp, tp, v, ext = cases.skin_vessel_case(N=64)
    out = []
    for flags in (ext.flags, ext.flags | abi.FLAG_NO_L2_PERSIST):
        ext.flags = flags
        with gpu.Engine(abi.SIM_MCXYZ, 0, ext) as e:
            e.prepare_data(rp, tp, v)
            e.run(3, 40_000)
            out.append((_tallies(e, (abi.TALLY_F3D, abi.TALLY_RD2D, abi.TALLY_DETPHOT2D)), e.summary()))
    for w in (abi.TALLY_F3D, abi.TALLY_RD2D, abi.TALLY_DETPHOT2D):
        np.testing.assert_array_equal(out[0][0][w], out[1][0][w])
    for k in ("photons", "substeps", "scatters", "rd_sum"):
        assert out[0][1][k] == out[1][1][k], k


def _cudart():
    """The CUDA runtime library, through ctypes, to read the context's limits
    from outside the engine (the engine links its own copy; both use the
    device's primary context)."""
    import ctypes
    import glob
    import os

    home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    for path in sorted(glob.glob(os.path.join(home, "lib64", "libcudart.so*"))) + ["libcudart.so"]:
        try:
            return ctypes.CDLL(path)
        except OSError:
            continue
    return None


def test_l2_set_aside_restored_on_destroy(gpu):
    # the handle raises the context's persisting-L2 set-aside while it lives
    # and puts back the value it found when it is destroyed
    import ctypes

    rt = _cudart()
    if rt is None:
        pytest.skip("no CUDA runtime library to read the limit with")
    persisting_l2 = 0x06  # cudaLimitPersistingL2CacheSize

    def limit():
        v = ctypes.c_size_t(0)
        assert rt.cudaDeviceGetLimit(ctypes.byref(v), persisting_l2) == 0
        return v.value

    # a 160^3 grid: its 33 MB tally is above the set-aside a context starts
    # with on GB300 (24 MB), so the handle has to raise it
    rp, tp, v, ext = cases.skin_vessel_case(N=160)
    before = limit()
    with gpu.Engine(abi.SIM_MCXYZ, 0, ext) as e:
        e.prepare_data(rp, tp, v)
        during = limit()
        e.run(0, 10_000)
    after = limit()
    maxp = ctypes.c_int(0)
    assert rt.cudaDeviceGetAttribute(ctypes.byref(maxp), 108, 0) == 0  # cudaDevAttrMaxPersistingL2CacheSize
    needed = min(160 ** 3 * 8, maxp.value)  # the u64 fluence tally of the grid, capped by the device
    print("persisting L2 set-aside before / during / after:", before, during, after, "needed", needed)
    assert during >= max(before, needed)  # the CUDA driver may round the set-aside up
    assert after == before


def test_prepare_again_for_a_same_size_grid_equals_a_fresh_handle(gpu):
    # a voxel handle prepared again for a grid of the same size keeps its
    # buffers; its results are a fresh handle's, and what the first
    # preparation grew (per-voxel properties, a radial tally) is gone
    rp, tp, v, ext = cases.skin_vessel_case(N=48)
    v2 = np.ascontiguousarray(v.reshape(48, 48, 48)[::-1, :, :].reshape(-1))  # the map upside down
    which = (abi.TALLY_F3D, abi.TALLY_RD2D, abi.TALLY_DETPHOT2D, abi.TALLY_RD_SLOTS)
    with gpu.Engine(abi.SIM_MCXYZ, 0, ext) as e:
        e.prepare_data(rp, tp, v)
        e.set_radial_tally(32, 0.01)
        e.set_voxel_props(np.full(v.size, 1.0, np.float32), np.full(v.size, 90.0, np.float32),
                          np.full(v.size, 0.9, np.float32))
        e.run(0, 20_000)
        e.prepare_data(rp, tp, v2)
        e.run(5, 30_000)
        again = (_tallies(e, which), e.summary())
        with pytest.raises(Exception):
            e.tally(abi.TALLY_RD_R)  # the radial tally went with the first preparation
    with gpu.Engine(abi.SIM_MCXYZ, 0, ext) as e:
        e.prepare_data(rp, tp, v2)
        e.run(5, 30_000)
        fresh = (_tallies(e, which), e.summary())
    for w in which:
        np.testing.assert_array_equal(again[0][w], fresh[0][w])
    for k in ("photons", "substeps", "scatters", "rd_sum"):
        assert again[1][k] == fresh[1][k], k
