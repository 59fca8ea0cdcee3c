"""Builds the engine library nmc_gb300/_build/libnmc_gb300.so with nvcc.

One -gencode (sm_103a), translation units compiled in parallel, then linked
into a shared library that exports the C ABI of include/nmc_abi.h.

    python -m nmc_gb300.build            # build if sources changed
    python -m nmc_gb300.build --force    # rebuild
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libnmc_gb300.so")
CLI_SRC = os.path.join(HERE, "cli", "nmc.cpp")
CLI = os.path.join(OUT, "nmc")
SOURCES = ["mcxyz.cu", "mcxyz_voxel.cu", "mcxyz_sweep.cu", "efield.cu", "mie.cu", "layered.cu", "mcsub.cu", "sweep.cu", "runtime.cu", "params.cu", "probe.cu", "noalloc.cu"]
HEADERS = ["nmc_device.cuh", "engine.h", "mcxyz_kernel.cuh"]
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


CHECKED_OUT = os.path.join(OUT, "checked")
CHECKED_LIB = os.path.join(CHECKED_OUT, "libnmc_gb300.so")


def flags(checked: bool = False) -> list[str]:
    # -ftz=true: FP32 subnormals flush to zero, which drops the subnormal
    # handling around every SFU approximation (rcp, ex2, lg2, rsqrt, sin,
    # cos) of the photon step; no FP32 quantity of the transport comes near
    # 1e-38 (weights stop at 1e-6)
    f = [ARCH, "-O3", "-lineinfo", "-std=c++17", "-ftz=true", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         f"-I{os.path.join(ROOT, 'include')}", f"-I{CSRC}"]
    return f + ["-DNMC_CHECK_BOUNDS"] if checked else f


def _stale(lib: str) -> bool:
    if not os.path.exists(lib):
        return True
    t = os.path.getmtime(lib)
    deps = [os.path.join(CSRC, s) for s in SOURCES + HEADERS] + [os.path.join(ROOT, "include", "nmc_abi.h"),
                                                              __file__, CLI_SRC]
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, checked: bool = False) -> str:
    obj = os.path.join(CHECKED_OUT if checked else OUT, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *flags(checked), "-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    if not force and not _stale(LIB) and os.path.exists(CLI):
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", tmp]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_cli()
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_checked(force: bool = False) -> str:
    """The checked library (every tally index tested, NMC_DEVFLAG_BOUNDS on a
    miss) in _build/checked/; select it with NMC_CHECKED=1 before importing
    nmc_gb300.engine."""
    os.makedirs(CHECKED_OUT, exist_ok=True)
    if not force and not _stale(CHECKED_LIB):
        return CHECKED_LIB
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, True), SOURCES))
    tmp = CHECKED_LIB + ".tmp"
    r = subprocess.run([nvcc(), ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", tmp], capture_output=True,
                       text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, CHECKED_LIB)
    return CHECKED_LIB


def build_cli() -> str:
    """The `nmc` program (host C++ over the C ABI), next to the library."""
    cxx = "g++" if subprocess.run(["which", "g++"], capture_output=True).returncode == 0 else nvcc()
    tmp = CLI + ".tmp"
    cmd = [cxx, "-O2", "-std=c++17", f"-I{os.path.join(ROOT, 'include')}", CLI_SRC, "-o", tmp, f"-L{OUT}",
           "-lnmc_gb300", "-Wl,-rpath,$ORIGIN"]
    if cxx != "g++":
        cmd = [cxx, "-O2", "-std=c++17", f"-I{os.path.join(ROOT, 'include')}", CLI_SRC, "-o", tmp, f"-L{OUT}",
               "-lnmc_gb300", "-Xlinker", "-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nmc CLI build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, CLI)
    return CLI


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    if "--checked" in sys.argv:
        print(f"built {build_checked(force='--force' in sys.argv)}")
