"""The `nmc` program's input side, without a GPU (--dry-run): _H.mci parsed
as the reference reads it (mcio.h:16-171, fgets into 32 bytes per line),
_props.m written in its format (mcio.h:298-325), errors reported with exit
status 1 instead of a crash."""
import os
import subprocess

import numpy as np
import pytest

from nmc_gb300 import abi, mci
import nmc_cases as cases


@pytest.fixture(scope="module")
def cli(engine_lib):
    from nmc_gb300 import build

    build.build()
    assert os.path.exists(mci.NMC)
    return mci.NMC


def test_dry_run_parses_mci_and_writes_props(cli, tmp_path):
    rp, tp, v, ext = cases.skin_vessel_case(N=16)
    name = str(tmp_path / "sv")
    mci.write_mci(name, rp, tp)
    mci.write_tissue(name, v)
    r = mci.run_nmc(name, "--dry-run")
    assert r.returncode == 0, r.stderr
    out = r.stdout
    assert "Nx = 16, dx = 0.0050 [mm]" in out
    assert "# of tissues available, Nt = 4" in out
    assert "muav[4] = 230.0000" in out
    props = open(name + "_props.m").read()
    assert props.startswith("muav(1) = 0.0001;\nmusv(1) = 1.0000;\ngv(1) = 1.0000;\n\n")
    assert "muav(2) = 20.0000;\nmusv(2) = 300.0000;\ngv(2) = 0.9000;\n\n" in props


def test_two_term_mci(cli, tmp_path):
    rp, tp, v, ext = cases.skin_vessel_case(N=8)
    rp.mckernelflag = abi.SIM_MCXYZ_TT
    for i in range(1, 5):
        tp.gf[i], tp.af[i], tp.gb[i], tp.ab[i], tp.CC[i] = 0.9, 0.5, 0.3, 0.5, 0.9
    name = str(tmp_path / "tt")
    mci.write_mci(name, rp, tp)
    mci.write_tissue(name, v)
    r = mci.run_nmc(name, "--dry-run")
    assert r.returncode == 0, r.stderr
    props = open(name + "_props.m").read()
    assert "gf(3) = 0.9000;\n\naf(3) = 0.5000;\n\ngb(3) = 0.3000;\n\nab(3) = 0.5000;\n\nCC(3) = 0.9000;\n\n" in props


def test_long_line_splits_like_fgets(cli, tmp_path):
    # a value line longer than 31 characters is read in two pieces, as the
    # reference's fgets(buf, 32) does: the tail becomes the next field
    rp, tp, v, ext = cases.skin_vessel_case(N=8)
    name = str(tmp_path / "long")
    mci.write_mci(name, rp, tp)
    mci.write_tissue(name, v)
    lines = open(name + "_H.mci").read().splitlines()
    lines[0] = "10.00" + " " * 26 + "7"  # 32 characters: time_min, then "7" read as Nx
    open(name + "_H.mci", "w").write("\n".join(lines) + "\n")
    r = mci.run_nmc(name, "--dry-run")
    assert "Nx = 7" in r.stdout


def test_errors_exit_1(cli, tmp_path):
    rp, tp, v, ext = cases.skin_vessel_case(N=8)
    name = str(tmp_path / "bad")
    mci.write_mci(name, rp, tp)
    r = mci.run_nmc(name, "--dry-run")  # no _T.bin for a voxel kind
    assert r.returncode == 1 and "_T.bin" in r.stderr
    mci.write_tissue(name, v[:10])
    r = mci.run_nmc(name, "--dry-run")
    assert r.returncode == 1
    rp.mckernelflag = abi.SIM_POLARIZATION_CBS_ELECTRIC_FIELDS if hasattr(abi, "SIM_POLARIZATION_CBS_ELECTRIC_FIELDS") else 3
    mci.write_mci(name, rp, tp)
    mci.write_tissue(name, v)
    r = mci.run_nmc(name, "--dry-run")
    assert r.returncode == 1 and "unsupported" in r.stdout
    r = mci.run_nmc(str(tmp_path / "missing"), "--dry-run")
    assert r.returncode == 1
    r = subprocess.run([mci.NMC], capture_output=True, text=True)
    assert r.returncode == 0 and "USAGE" in r.stdout


def test_merge_replicas_is_the_photon_weighted_run(tmp_path):
    # three replica runs of one voxel problem, written in the formats `nmc`
    # writes; the merge equals one run of all their photons
    import json

    rng = np.random.default_rng(5)
    Nx = Ny = 6
    Nz = 4
    names, Ns, Fs, R, D, rds, ses = [], [100, 300, 600], [], [], [], [], []
    for k, n in enumerate(Ns):
        name = str(tmp_path / f"rep{k}")
        F = rng.uniform(0, 5, Nx * Ny * Nz).astype(np.float32)
        ryx = rng.uniform(0, 1, (Nx, Ny))
        det = rng.integers(0, 50, (Nx, Ny))
        F.tofile(name + "_F.bin")
        with open(name + "_Ryx.dat", "w") as f:
            for row in ryx:
                f.write("".join(f"\t {v:1.6e}" for v in row) + "\n")
        with open(name + "_DetPhot2D.dat", "w") as f:
            for row in det:
                f.write("".join(f"\t {int(v)}" for v in row) + "\n")
        rd, se = rng.uniform(0.2, 0.3), rng.uniform(0.001, 0.003)
        json.dump({"photons": n, "Rd": rd, "Rd_se": se, "rng": "philox4x32-10"}, open(name + "_report.json", "w"))
        names.append(name)
        Fs.append(F.astype(np.float64))
        R.append(np.array([[float(f"{v:1.6e}") for v in row] for row in ryx]))
        D.append(det)
        rds.append(rd)
        ses.append(se)
    out = str(tmp_path / "merged")
    m = mci.merge_replicas(names, out, Nx, Ny, Nz)
    w = np.array(Ns, float)
    assert m["photons"] == 1000
    assert m["Rd"] == pytest.approx(float((w * np.array(rds)).sum() / 1000), rel=1e-12)
    assert m["Rd_se"] == pytest.approx(float(np.sqrt(((w * np.array(ses)) ** 2).sum()) / 1000), rel=1e-12)
    F = np.fromfile(out + "_F.bin", np.float32)
    np.testing.assert_allclose(F, (sum(wi * f for wi, f in zip(w, Fs)) / 1000).astype(np.float32), rtol=1e-7)
    np.testing.assert_allclose(mci.read_table(out + "_Ryx.dat"), sum(wi * r for wi, r in zip(w, R)) / 1000,
                               rtol=1e-6)
    np.testing.assert_array_equal(mci.read_table(out + "_DetPhot2D.dat", int), sum(D))
    assert mci.read_rd(out) == pytest.approx(round(m["Rd"], 4))
