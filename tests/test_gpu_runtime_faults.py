"""Failure handling and resume without faulting the GPU: invalid inputs are
rejected on the host with NMC_EINVAL before any device work and leave the
handle usable; a host wait that runs out returns NMC_ETIMEOUT and leaves the
handle usable; a run checkpointed and resumed in another engine equals the
uninterrupted run."""
import math

import numpy as np
import pytest

from nmc_gb300 import abi, checkpoint
import nmc_cases as cases

pytestmark = pytest.mark.gpu


def _bad_inputs():
    """(label, mutate(rp, tp, v) -> v) pairs, each an input nmc_prepare rejects."""
    def tissue_id(rp, tp, v):
        v = v.copy()
        v[len(v) // 2] = abi.NTISS  # ids run 0 .. 18
        return v

    def nan_mua(rp, tp, v):
        tp.muav[2] = math.nan
        return v

    def zero_mus(rp, tp, v):
        tp.musv[3] = 0.0
        return v

    def inf_g(rp, tp, v):
        tp.gv[2] = math.inf
        return v

    def empty_grid(rp, tp, v):
        rp.Nz = 0
        return v

    def bad_voxel(rp, tp, v):
        rp.dx = -rp.dx
        return v

    def boundary(rp, tp, v):
        rp.boundaryflag = 3
        return v

    def index(rp, tp, v):
        rp.n2 = 0.0
        return v

    return [("tissue id > 18", tissue_id), ("NaN mua", nan_mua), ("mus = 0", zero_mus), ("inf g", inf_g),
            ("Nz = 0", empty_grid), ("dx < 0", bad_voxel), ("boundaryflag 3", boundary), ("n2 = 0", index)]


@pytest.mark.parametrize("label,mutate", _bad_inputs(), ids=[b[0] for b in _bad_inputs()])
def test_prepare_rejects_invalid_inputs_and_stays_usable(gpu, label, mutate):
    rp, tp, v, ext = cases.skin_vessel_case(N=32)
    with gpu.Engine(abi.SIM_MCXYZ, 0, ext) as e:
        bad_rp, bad_tp, _, _ = cases.skin_vessel_case(N=32)
        bad_v = mutate(bad_rp, bad_tp, v)
        with pytest.raises(gpu.NMCError) as err:
            e.prepare_data(bad_rp, bad_tp, bad_v)
        assert err.value.status == 1, label  # NMC_EINVAL
        e.prepare_data(rp, tp, v)  # the same handle still works
        e.run(0, 20_000)
        assert e.summary()["photons"] == 20_000


def test_unused_tissue_entries_are_not_checked(gpu):
    # the reference reads tissue tables of up to 18 entries and uses only the
    # ids present in the map: an unused entry may hold anything
    rp, tp, v, ext = cases.skin_vessel_case(N=32)
    tp.muav[10] = math.nan
    tp.musv[11] = 0.0
    with gpu.Engine(abi.SIM_MCXYZ, 0, ext) as e:
        e.prepare_data(rp, tp, v)
        e.run(0, 10_000)
        assert e.summary()["photons"] == 10_000


def test_mcsub_rejects_a_medium_without_interaction(gpu):
    rp, tp, ext = cases.mcsub_case()
    tp.muav[1] = 0.0
    tp.musv[1] = 0.0
    with gpu.Engine(abi.SIM_MCSUB, 0, ext) as e:
        with pytest.raises(gpu.NMCError) as err:
            e.prepare_data(rp, tp, None)
        assert err.value.status == 1


def test_timeout_then_recover(gpu):
    rp, tp, v, ext = cases.skin_vessel_case(N=64)
    ext.timeout_s = 1e-4
    with gpu.Engine(abi.SIM_MCXYZ, 0, ext) as e:
        e.prepare_data(rp, tp, v)
        e.run_async(0, 5_000_000)
        with pytest.raises(gpu.NMCError) as err:
            e.synchronize()
        assert err.value.status == 4  # NMC_ETIMEOUT
        ext2 = cases.skin_vessel_case(N=64)[3]
        ext2.timeout_s = 0.0  # no limit
        e.set_ext(ext2)
        e.synchronize()
        assert e.summary()["photons"] == 5_000_000


@pytest.mark.parametrize("kind", ["mcsub", "mcxyz"])
def test_checkpoint_resume_equals_one_run(gpu, kind, tmp_path):
    if kind == "mcsub":
        rp, tp, ext = cases.mcsub_case()
        sim, v = abi.SIM_MCSUB, None
    else:
        rp, tp, v, ext = cases.skin_vessel_case(N=48)
        sim = abi.SIM_MCXYZ
    N, k = 60_000, 25_000
    with gpu.Engine(sim, 0, ext) as e:
        e.prepare_data(rp, tp, v)
        e.run(0, N)
        whole = checkpoint.snapshot(e, N)
    with gpu.Engine(sim, 0, ext) as e:
        e.prepare_data(rp, tp, v)
        e.run(0, k)
        checkpoint.save(str(tmp_path / "ck.npz"), checkpoint.snapshot(e, k))
    with gpu.Engine(sim, 0, ext) as e:  # a fresh process would do the same
        e.prepare_data(rp, tp, v)
        done = checkpoint.resume(e, checkpoint.load(str(tmp_path / "ck.npz")), N, chunk=10_000)
    assert done["next_photon"] == N
    for key in whole:
        if key.startswith("tally_"):
            np.testing.assert_array_equal(done[key], whole[key])
    s0, s1 = checkpoint.sums(whole), checkpoint.sums(done)
    for key in ("photons", "substeps", "scatters", "S", "A", "E", "rd_sum"):
        assert s1[key] == pytest.approx(s0[key], rel=1e-12, abs=1e-9), key
