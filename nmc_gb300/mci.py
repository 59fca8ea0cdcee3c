"""The reference's file formats for the `nmc` program (nmc_gb300/_build/nmc).

Writers produce what the sample notebooks write before running `nmc <name>`
(NMC-samples/example3.ipynb cell 5: one value per line in the order
mcio.h:16-171 reads them; the tissue map as raw uint8); readers parse what
`nmc` writes (main.m:203-262, 473-561; mcio.h:298-389).
"""
from __future__ import annotations

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
