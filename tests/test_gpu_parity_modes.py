"""Per-photon parity with the oracle over the reference's launch, boundary
and detection modes (kernels.metal:366-463 launch, :556-637 detection,
:646-672 boundaries) and over grid shapes the skin-vessel case does not
exercise: odd and non-cubic grids, non-square voxels.  Same Philox streams
on both sides; a photon matches when its fate, SPIN count, detected and
absorbed weight agree (rel 1e-3)."""
import pytest

from nmc_gb300 import abi
import nmc_cases as cases

pytestmark = pytest.mark.gpu


_medium = cases.modes_medium
MODES = cases.PARITY_MODES


@pytest.mark.parametrize("mode", list(MODES))
def test_mode_per_photon(gpu, oracle, mode):
    kw = dict(MODES[mode])
    grid = {k: kw.pop(k) for k in ("Nx", "Ny", "Nz", "dx", "dy", "dz") if k in kw}
    rp, tp, v = _medium(**grid, **kw)
    ext = abi.ext_defaults(rng=abi.RNG_PHILOX, seed=21)
    n = 3000
    with gpu.Engine(abi.SIM_MCXYZ, 0, ext) as e:
        e.prepare_data(rp, tp, v)
        recs, _ = e.run_traced(0, n)
        s = e.summary()
    o = oracle.run(abi.SIM_MCXYZ, rp, tp, v, ext=ext, n=n, trace=True)
    frac, _ = cases.match_fraction(recs, o["recs"])
    print(f"{mode}: per-photon match {frac:.4f}, Rd gpu {s['rd_sum'] / n:.5f} oracle {o['rd_sum'] / n:.5f}, "
          f"sub-steps/photon {recs['n_sub'].mean():.1f} / {o['recs']['n_sub'].mean():.1f}")
    assert frac >= 0.9
    assert s["photons"] == n


@pytest.mark.parametrize("mode", [m for m in MODES if m != "gaussian-beam"])
def test_two_term_mode_per_photon(gpu, oracle, mode):
    # the two-term kernel (kernels.metal:757-1118; its launch has no Gaussian
    # branch) over the same launch, boundary and detection modes
    kw = dict(MODES[mode])
    grid = {k: kw.pop(k) for k in ("Nx", "Ny", "Nz", "dx", "dy", "dz") if k in kw}
    rp, tp, v = _medium(**grid, **kw)
    rp.mckernelflag = abi.SIM_MCXYZ_TT
    for t in range(1, 4):
        tp.gf[t], tp.af[t], tp.gb[t], tp.ab[t], tp.CC[t] = 0.9, 0.5, 0.3, 0.5, 0.9
    ext = abi.ext_defaults(rng=abi.RNG_PHILOX, seed=23)
    n = 3000
    with gpu.Engine(abi.SIM_MCXYZ_TT, 0, ext) as e:
        e.prepare_data(rp, tp, v)
        recs, _ = e.run_traced(0, n)
        s = e.summary()
    o = oracle.run(abi.SIM_MCXYZ_TT, rp, tp, v, ext=ext, n=n, trace=True)
    frac, _ = cases.match_fraction(recs, o["recs"])
    print(f"two-term {mode}: per-photon match {frac:.4f}, Rd gpu {s['rd_sum'] / n:.5f} oracle "
          f"{o['rd_sum'] / n:.5f}")
    assert frac >= 0.9
    assert s["photons"] == n


@pytest.mark.parametrize("mcflag", [1, 2], ids=["gaussian-focus", "isotropic-point"])
def test_mcsub_launch_modes_per_photon(gpu, oracle, mcflag):
    rp, tp, ext = cases.mcsub_case(g=0.9, seed=4)
    ext.sub_mcflag = mcflag
    ext.sub_radius, ext.sub_waist, ext.sub_zfocus = 0.05, 0.02, 0.1
    ext.sub_zs = 0.1 if mcflag == 2 else 0.0
    n = 4000
    with gpu.Engine(abi.SIM_MCSUB, 0, ext) as e:
        e.prepare_data(rp, tp)
        recs, _ = e.run_traced(0, n)
    o = oracle.run(abi.SIM_MCSUB, rp, tp, ext=ext, n=n, trace=True)
    frac, _ = cases.match_fraction(recs, o["recs"])
    print(f"mcsub mcflag {mcflag}: per-photon match {frac:.4f}")
    assert frac >= 0.98


def test_edge_photon_counts(gpu):
    rp, tp, v = _medium()
    ext = abi.ext_defaults(rng=abi.RNG_PHILOX, seed=1)
    with gpu.Engine(abi.SIM_MCXYZ, 0, ext) as e:
        e.prepare_data(rp, tp, v)
        e.run(0, 0)  # nothing to do
        assert e.summary()["photons"] == 0
        e.run(5, 1)  # a single photon, anywhere in the id space
        assert e.summary()["photons"] == 1
        e.run(2 ** 40, 1000)
        assert e.summary()["photons"] == 1001
