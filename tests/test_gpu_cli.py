"""`nmc <name>` end to end on the GPU: the files it writes hold what the
engine computes for the same photons (the reference's streams and dispatch
loop), normalised as main.m does."""
import numpy as np
import pytest

from nmc_gb300 import abi, mci
import nmc_cases as cases

pytestmark = pytest.mark.gpu


def _engine_results(gpu, sim, rp, tp, v, photons=100_000, batch=10_000):
    ext = abi.ext_defaults(rng=abi.RNG_TAUS_REF, photons_per_dispatch=batch, photons_total=photons)
    with gpu.Engine(sim, 0, ext) as e:
        e.prepare_data(rp, tp, v)
        for run in range(1, photons // batch + 1):
            e.set_num_runs_seed(run)
            e.send_compute_command()
        return e.get_compute_results(), e.ext


def test_cli_mcxyz_files(gpu, tmp_path):
    rp, tp, v, ext = cases.skin_vessel_case(N=40, d=0.005)
    name = str(tmp_path / "sv")
    mci.write_mci(name, rp, tp)
    mci.write_tissue(name, v)
    r = mci.run_nmc(name)
    assert r.returncode == 0, r.stdout + r.stderr
    res, _ = _engine_results(gpu, abi.SIM_MCXYZ, rp, tp, v)
    N = np.float32(100_000)
    temp = np.float32(rp.dx) * np.float32(rp.dy) * np.float32(rp.dz) * N
    mua = np.asarray(tp.muav, np.float32)[v]
    with np.errstate(divide="ignore", invalid="ignore"):
        F = res["F3D"] / (temp * mua)
    F[~np.isfinite(F)] = 0
    np.testing.assert_allclose(mci.read_fluence(name, rp), F, rtol=2e-6, atol=0)
    rd = np.float32(res["Rd"][np.isfinite(res["Rd"])].sum(dtype=np.float32)) / N
    assert f"{mci.read_rd(name):.4f}" == f"{rd:.4f}"
    assert f"Total Rd = {rd:.8f}" in r.stdout
    ryx = mci.read_table(name + "_Ryx.dat")
    det = mci.read_table(name + "_DetPhot2D.dat", int)
    assert ryx.shape == (rp.Nx, rp.Ny)
    idx = np.arange(rp.Ny)[None, :] + np.arange(rp.Nx)[:, None] * rp.Nx
    np.testing.assert_allclose(ryx, res["Rd2D"][idx], rtol=1e-6, atol=1e-12)
    np.testing.assert_array_equal(det, res["DetPhot2D"][idx])
    import json

    rep = json.load(open(name + "_report.json"))
    assert rep["photons"] == 100_000 and rep["rng"] == "reference"
    assert rep["Rd"] == pytest.approx(float(rd), rel=1e-5) and 0 < rep["Rd_se"] < rep["Rd"]


def test_cli_mcsub_files(gpu, tmp_path):
    rp, tp, ext = cases.mcsub_case(g=0.9)
    rp.Nx = rp.Ny = rp.Nz = 1
    name = str(tmp_path / "sub")
    mci.write_mci(name, rp, tp)
    r = mci.run_nmc(name, cwd=str(tmp_path))
    assert r.returncode == 0, r.stdout + r.stderr
    res, ex = _engine_results(gpu, abi.SIM_MCSUB, rp, tp, None)
    out = mci.read_mcout(str(tmp_path / "mcOUT0.dat"))
    B, dr = ex.sub_bins, 0.0020
    ir = np.arange(1, B + 1)
    rr = ((ir - 0.5) * dr).astype(np.float32).astype(np.float64)
    J = (res["J"][1:B + 1].astype(np.float64) / (2.0 * 3.1415926 * rr * dr * 100_000)).astype(np.float32)
    np.testing.assert_allclose(out["J"], J, rtol=1e-6)
    sae = res["SAE"] / np.float32(100_000)
    assert out["S"] == pytest.approx(float(sae[0]), rel=1e-6)
    assert out["E"] == pytest.approx(float(sae[2]), rel=1e-6)
    assert f"{mci.read_rd(name):.4f}" == f"{np.float32(sae[2] + sae[0]):.4f}"
    assert out["F"].shape == (B, B)


def test_persistent_launch_equals_the_dispatch_loop(gpu, tmp_path):
    # the default single launch and the reference's ten blocking dispatches
    # draw the same streams per photon; every file is identical
    rp, tp, v, ext = cases.skin_vessel_case(N=40, d=0.005)
    outs = {}
    for mode in ("default", "--dispatch"):
        name = str(tmp_path / mode.strip("-"))
        mci.write_mci(name, rp, tp)
        mci.write_tissue(name, v)
        r = mci.run_nmc(name, *([] if mode == "default" else [mode]))
        assert r.returncode == 0, r.stdout + r.stderr
        outs[mode] = {ext_: open(name + ext_, "rb").read() for ext_ in ("_F.bin", "_Rd.dat", "_Ryx.dat",
                                                                       "_DetPhot2D.dat")}
    assert outs["default"] == outs["--dispatch"]
