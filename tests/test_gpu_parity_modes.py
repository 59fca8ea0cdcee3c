"""Per-photon parity with the oracle over the reference's launch, boundary
and detection modes (kernels.metal:366-463 launch, :556-637 detection,
:646-672 boundaries) and over grid shapes the skin-vessel case does not
exercise: odd and non-cubic grids, non-square voxels.  Same Philox streams
on both sides; a photon matches when its fate, SPIN count, detected and
absorbed weight agree (rel 1e-3)."""
import math

import numpy as np
import pytest

from nmc_gb300 import abi
import nmc_cases as cases

pytestmark = pytest.mark.gpu


def _medium(Nx=40, Ny=40, Nz=40, dx=0.01, dy=0.01, dz=0.01, **run):
    """Air above zsurf = 2 dz, tissue (mua 1, mus 80, g 0.85) below, a
    spherical inclusion (mua 5, mus 120, g 0.9) of radius 0.06 cm at depth 0.1."""
    zsurf = 2 * dz
    base = dict(myname="modes", Nx=Nx, Ny=Ny, Nz=Nz, dx=dx, dy=dy, dz=dz, mcflag=0, launchflag=0,
                boundaryflag=2, xs=0.0, ys=0.0, zs=zsurf + 1e-4, xfocus=0.0, yfocus=0.0, zfocus=float("inf"),
                ux0=0.0, uy0=0.0, uz0=1.0, radius=0.03, waist=0.03, zsurf=zsurf, det_radius=15.0, xd=0.0,
                n1=1.37, n2=1.0, na=90.0, det_state=0, mckernelflag=abi.SIM_MCXYZ, Nt=3)
    base.update(run)
    rp = abi.run_params(**base)
    tp = abi.tissue_params(mua=[0.0001, 1.0, 5.0], mus=[1.0, 80.0, 120.0], g=[1.0, 0.85, 0.9])
    T = np.full((Nz, Nx, Ny), 2, np.uint8)
    T[:2] = 1
    x = (np.arange(Nx) + 0.5 - Nx / 2) * dx
    y = (np.arange(Ny) + 0.5 - Ny / 2) * dy
    z = (np.arange(Nz) + 0.5) * dz
    inc = (x[None, :, None] ** 2 + y[None, None, :] ** 2 + (z[:, None, None] - 0.1) ** 2) <= 0.06 ** 2
    T[inc] = 3
    return rp, tp, T.reshape(-1)


MODES = {
    "gaussian-beam": dict(mcflag=1, radius=0.02, waist=0.02, zfocus=0.1),
    "isotropic-point": dict(mcflag=2, xs=0.0, ys=0.0, zs=0.1),
    "rectangle": dict(mcflag=3, radius=0.05),
    "point-collimated": dict(mcflag=4),
    "manual-direction": dict(launchflag=1, xs=0.01, ys=-0.02, zs=0.0201, ux0=0.3, uy0=0.2,
                             uz0=math.sqrt(1 - 0.13)),
    "boundary-0": dict(boundaryflag=0),
    "boundary-1": dict(boundaryflag=1),
    "transmittance": dict(det_state=1, Nz=16, zsurf=0.16, boundaryflag=1),
    "ring-detector": dict(xd=0.05, det_radius=0.02, na=30.0),
    "odd-noncubic-grid": dict(Nx=41, Ny=37, Nz=29, dx=0.011, dy=0.009, dz=0.0125),
}


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
