"""The reference's file formats for the `nmc` program (nmc_gb300/_build/nmc).

Writers produce what the sample notebooks write before running `nmc <name>`
(NMC-samples/example3.ipynb cell 5: one value per line in the order
mcio.h:16-171 reads them; the tissue map as raw uint8); readers parse what
`nmc` writes (main.m:203-262, 473-561; mcio.h:298-389).
"""
from __future__ import annotations

import json
import os
import subprocess

import numpy as np

from . import abi

HERE = os.path.dirname(os.path.abspath(__file__))
NMC = os.path.join(HERE, "_build", "nmc")

_ORDER = [("time_min", "f2"), ("Nx", "d"), ("Ny", "d"), ("Nz", "d"), ("dx", "f"), ("dy", "f"), ("dz", "f"),
          ("mcflag", "d"), ("launchflag", "d"), ("boundaryflag", "d"), ("xs", "f"), ("ys", "f"), ("zs", "f"),
          ("xfocus", "f"), ("yfocus", "f"), ("zfocus", "f"), ("ux0", "f"), ("uy0", "f"), ("uz0", "f"),
          ("radius", "f"), ("waist", "f"), ("zsurf", "f"), ("det_radius", "f"), ("xd", "f"), ("n1", "f"),
          ("n2", "f"), ("na", "f"), ("lambda_", "f"), ("lc", "f"), ("speckleflag", "d"), ("semiflag", "d"),
          ("det_state", "d"), ("mckernelflag", "d")]


def _fmt(v, kind):
    if kind == "d":
        return f"{int(v)}"
    if kind == "f2":
        return f"{float(v):.2f}"
    v = float(v)
    if np.isinf(v):
        v = 1e12  # the notebooks write zfocus = inf as 1e12
    return f"{v:.4f}" if abs(v) < 1e6 else f"{v:.6g}"


def write_mci(name: str, rp: abi.RunParams, tp: abi.TissueParams) -> str:
    """Writes <name>_H.mci from the run and tissue parameters."""
    lines = []
    for field, kind in _ORDER:
        lines.append(_fmt(getattr(rp, field), kind))
    nt = int(rp.Nt)
    lines.append(str(nt))
    for i in range(1, nt + 1):
        lines += [f"{tp.muav[i]:.4f}", f"{tp.musv[i]:.4f}"]
        if int(rp.mckernelflag) == abi.SIM_MCXYZ_TT:
            lines += [f"{tp.gf[i]:.4f}", f"{tp.af[i]:.4f}", f"{tp.gb[i]:.4f}", f"{tp.ab[i]:.4f}", f"{tp.CC[i]:.4f}"]
        else:
            lines.append(f"{tp.gv[i]:.4f}")
    path = f"{name}_H.mci"
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return path


def write_tissue(name: str, v) -> str:
    """Writes <name>_T.bin: the uint8 map in the engine's voxel order."""
    path = f"{name}_T.bin"
    np.ascontiguousarray(v, dtype=np.uint8).ravel().tofile(path)
    return path


def run_nmc(name: str, *args: str, cwd: str | None = None, timeout: float = 600.0) -> subprocess.CompletedProcess:
    """Runs `nmc <name> args...` as the notebooks do."""
    if not os.path.exists(NMC):
        raise FileNotFoundError(f"{NMC} is missing; build with `python -m nmc_gb300.build`")
    return subprocess.run([NMC, name, *args], cwd=cwd, capture_output=True, text=True, timeout=timeout)


def read_rd(name: str) -> float:
    with open(f"{name}_Rd.dat") as f:
        return float(f.read().strip())


def read_fluence(name: str, rp: abi.RunParams) -> np.ndarray:
    """<name>_F.bin as float32 in the engine's voxel order."""
    return np.fromfile(f"{name}_F.bin", dtype=np.float32, count=rp.Nx * rp.Ny * rp.Nz)


def read_table(path: str, dtype=float) -> np.ndarray:
    """_Ryx.dat / _DetPhot2D.dat: rows of tab-separated values."""
    with open(path) as f:
        return np.array([[dtype(t) for t in line.split()] for line in f if line.strip()])


def read_mcout(path: str = "mcOUT0.dat") -> dict:
    """mcOUT0.dat: header values, S/A/E, r row, J row and F(z, r)."""
    with open(path) as f:
        lines = f.read().splitlines()
    head = [float(line.split("\t")[0]) for line in lines[:19]]
    r = np.array([float(t) for t in lines[19].split("\t")[1:]])
    J = np.array([float(t) for t in lines[20].split("\t")[1:]])
    rows = [[float(t) for t in line.split()] for line in lines[21:] if line.strip()]
    z = np.array([row[0] for row in rows])
    F = np.array([row[1:] for row in rows])
    return {"mua": head[0], "mus": head[1], "g": head[2], "n1": head[3], "n2": head[4], "NR": int(head[11]),
            "dr": head[13], "dz": head[14], "photons": head[15], "S": head[16], "A": head[17], "E": head[18],
            "r": r, "J": J, "z": z, "F": F}


def merge_replicas(names, out: str, Nx: int, Ny: int, Nz: int) -> dict:
    """Combines the outputs of independent `nmc` runs of one voxel problem
    (replicas on other GPUs or boxes, each with its own Philox seed or photon
    range) into one run of all their photons, in FP64: _F.bin and _Ryx.dat
    are photon-weighted means of the per-run normalised values, _DetPhot2D.dat
    is the sum of the counts, Rd the photon-weighted mean with the standard
    errors combined as independent.  Reads each <name>_report.json; writes
    <out>_F.bin, _Rd.dat, _Ryx.dat, _DetPhot2D.dat and _report.json in the
    formats `nmc` writes (main.m:473-561).  Returns the merged report."""
    reps = []
    for n in names:
        with open(f"{n}_report.json") as f:
            reps.append(json.load(f))
    N = np.array([float(r["photons"]) for r in reps])
    tot = float(N.sum())
    nv, n2d = Nx * Ny * Nz, Nx * Ny
    F = np.zeros(nv)
    ryx = np.zeros((Nx, Ny))
    det = np.zeros((Nx, Ny), np.int64)
    for n, w in zip(names, N):
        F += w * np.fromfile(f"{n}_F.bin", dtype=np.float32, count=nv).astype(np.float64)
        ryx += w * read_table(f"{n}_Ryx.dat")
        det += read_table(f"{n}_DetPhot2D.dat", int).astype(np.int64)
    F /= tot
    ryx /= tot
    rd = float(sum(w * r["Rd"] for w, r in zip(N, reps)) / tot)
    se = float(np.sqrt(sum((w * r["Rd_se"]) ** 2 for w, r in zip(N, reps))) / tot)
    F.astype(np.float32).tofile(f"{out}_F.bin")
    with open(f"{out}_Rd.dat", "w") as f:
        f.write(f"{rd:0.4f}\n")
    with open(f"{out}_Ryx.dat", "w") as f:
        for row in ryx:
            f.write("".join(f"\t {v:1.6e}" for v in row) + "\n")
    with open(f"{out}_DetPhot2D.dat", "w") as f:
        for row in det:
            f.write("".join(f"\t {int(v)}" for v in row) + "\n")
    merged = {"name": os.path.basename(out), "photons": int(tot), "Rd": rd, "Rd_se": se,
              "replicas": [{"name": n, "photons": int(w), "rng": r.get("rng")} for n, w, r in zip(names, N, reps)]}
    with open(f"{out}_report.json", "w") as f:
        json.dump(merged, f)
    return merged
