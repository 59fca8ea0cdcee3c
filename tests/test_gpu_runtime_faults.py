"""Failure handling and resume without faulting the GPU: a host wait that
runs out returns NMC_ETIMEOUT and leaves the handle usable; a run
checkpointed and resumed in another engine equals the uninterrupted run."""
import numpy as np
import pytest

from nmc_gb300 import abi, checkpoint
import nmc_cases as cases

pytestmark = pytest.mark.gpu


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
