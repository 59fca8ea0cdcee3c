"""The C ABI without a GPU: struct layouts, exported symbols, error paths."""
import ctypes as C
import os
import re

import numpy as np

import pytest

from nmc_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    src = open(os.path.join(ROOT, "include", "nmc_abi.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(nmc_[a-z0-9_]+)\s*\(", src)))


def test_struct_layouts_match_reference_sizes():
    assert C.sizeof(abi.RunParams) == 172
    assert C.sizeof(abi.TissueParams) == 608
    assert abi.RunParams.myname.offset == 0
    assert abi.RunParams.n1.offset == 96
    assert abi.RunParams.det_state.offset == 116
    assert abi.RunParams.Nx.offset == 136
    assert abi.RunParams.mckernelflag.offset == 168


def test_struct_layouts_match_reference_compiler_layout(oracle):
    if not oracle.ref_available():
        pytest.skip("reference sources not present on this machine")
    lib = oracle.ref_lib()
    assert lib.ref_sizeof_runparams() == C.sizeof(abi.RunParams)
    assert lib.ref_sizeof_tissueparams() == C.sizeof(abi.TissueParams)


def test_library_exports_every_declared_symbol(engine_lib):
    L = engine_lib.lib()
    names = _declared_functions()
    assert "nmc_create" in names and "nmc_get_compute_results" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert L.nmc_abi_version() == 1


def test_ext_defaults_match_reference_constants(engine_lib):
    L = engine_lib.lib()
    e = abi.Ext()
    L.nmc_ext_defaults(C.byref(e))
    assert e.size == C.sizeof(abi.Ext)
    assert e.photons_per_dispatch == 10000 and e.photons_total == 100000  # definitions.h:16-17
    assert e.sub_bins == 101 and abs(e.sub_dr - 0.002) < 1e-9  # definitions.h:31,52
    assert e.sub_boundaryflag == 1 and e.sub_mcflag == 0
    py = abi.ext_defaults()
    for name, _ in abi.Ext._fields_:
        if name in ("reserved",):
            continue
        assert getattr(e, name) == pytest.approx(getattr(py, name)), name


def test_create_reports_missing_device_or_unsupported_kind(engine_lib):
    L = engine_lib.lib()
    h = C.c_void_p()
    # empty reference kernels (kernels.metal:1122-1202) are not offered
    assert L.nmc_create(abi.SIM_POLARIZATION_CBS_ELECTRIC_FIELDS, 0, C.byref(h)) == 7
    assert L.nmc_create(abi.SIM_RAMAN, 0, C.byref(h)) == 7
    assert L.nmc_create(42, 0, C.byref(h)) == 1
    st = L.nmc_create(abi.SIM_MCXYZ, 10_000, C.byref(h))
    assert st == 3  # NMC_EDEVICE: no such device
    assert not h.value


def test_null_handle_calls_do_not_crash(engine_lib):
    L = engine_lib.lib()
    assert L.nmc_run(None, 0, 1) == 1
    assert L.nmc_reset(None) == 1
    assert L.nmc_last_error(None) == b"null handle"
    L.nmc_destroy(None)


def test_adjoint_case_and_autograd_module_import():
    import nmc_cases as cases
    from nmc_gb300 import autograd

    rp, tp, v, ext, mua, mus, g, bins, dr = cases.adjoint_case(N=16)
    assert mua.shape == (16, 16, 16) and mua.dtype == np.float32
    assert 0.1 - 1e-6 <= mua.min() and mua.max() <= 5.0 + 1e-5
    assert 50.0 - 1e-4 <= mus.min() and mus.max() <= 300.0 + 1e-3
    assert np.all(g == np.float32(0.85))
    assert callable(autograd.radial_reflectance)


def test_python_mirrors_of_the_new_structs():
    # sizes the header pins with static_assert
    assert C.sizeof(abi.EfieldConfig) == 88
    assert C.sizeof(abi.EfieldSetting) == 24
    assert C.sizeof(abi.Layer) == 20
    assert C.sizeof(abi.LayeredConfig) == 40
    assert C.sizeof(abi.TuneResult) == 1004
    assert abi.SPECKLE_DTYPE.itemsize == 28
    assert C.sizeof(abi.SweepSet) == 64


def test_integration_c_snippet_compiles(tmp_path):
    # the C host binding shown to maintainers compiles against include/nmc_abi.h
    import re
    import shutil
    import subprocess

    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    doc = open(os.path.join(root, "INTEGRATION.md")).read()
    snippets = re.findall(r"```c\n(.*?)```", doc, re.S)
    assert len(snippets) >= 2

    def body(snippet):
        return "\n".join(ln for ln in snippet.splitlines() if not ln.startswith("#include"))

    # the first replaces main.m's calls; later ones run on an existing handle
    src = tmp_path / "host.c"
    src.write_text(
        "#include <stdio.h>\n#include <stdint.h>\n#include <stdlib.h>\n#include \"nmc_abi.h\"\n"
        "void host(nmc_run_params runParams, nmc_tissue_params tissParams, const char* v, int NumGPURuns,\n"
        "          float t_seed, float* ResJ_GPU, float* ResF_GPU, float* ResF3D_GPU, float* ResSAE_GPU,\n"
        "          float* ResRd_GPU, float* ResRd2D_GPU, int32_t* ResDetPhotons2D_GPU) {\n"
        + body(snippets[0]) + "\n}\n"
        + "".join(f"void extra{k}(nmc_handle* h) {{\n{body(b)}\n}}\n" for k, b in enumerate(snippets[1:])))
    r = subprocess.run([cc, "-std=c11", "-Wall", "-Werror", "-fsyntax-only", f"-I{os.path.join(root, 'include')}",
                        str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_integration_python_snippets_parse():
    # every Python example shown to maintainers is valid Python and names
    # functions the package has
    import ast
    import importlib
    import re

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    doc = open(os.path.join(root, "INTEGRATION.md")).read()
    blocks = re.findall(r"```python\n(.*?)```", doc, re.S)
    assert blocks
    for b in blocks:
        tree = ast.parse(b)
        for node in ast.walk(tree):
            if isinstance(node, ast.ImportFrom) and node.module and node.module.startswith("nmc_gb300"):
                for a in node.names:
                    mod = importlib.import_module(node.module)
                    assert hasattr(mod, a.name) or importlib.util.find_spec(f"{node.module}.{a.name}"), a.name


def test_photon_limits_refused_before_any_device_call():
    # the functional entry points check their limits on the host before they
    # touch a device, so the refusals are testable without a GPU
    import math

    import nmc_cases as cases
    from nmc_gb300 import efield, engine, layered

    cfg, s633, s700, st = cases.cbs_case(n_settings=2, photons=2 ** 52 + 1, cone_n=8, sep_n=8)
    with pytest.raises(engine.NMCError) as e:  # 2^53 + 2 photons in all: beyond exact FP64 counts
        efield.run(cfg, s633, st, S_raman=s700)
    assert abi.STATUS[e.value.status] == "NMC_EINVAL"
    with pytest.raises(engine.NMCError) as e:
        layered.run([(0.1, 100.0, 0.9, 1.4, math.inf)], photons=2 ** 31 + 1)
    assert abi.STATUS[e.value.status] == "NMC_EINVAL"


def test_noalloc_photon_limit_refused_before_any_device_call(engine_lib):
    # nmc_mcxyz_run_noalloc never folds its fixed-point sums, so it takes at
    # most 2^31 photons per call; the check comes before any CUDA call, and
    # the device pointers below are never dereferenced
    import nmc_cases as cases

    L = engine_lib.lib()
    f = L.nmc_mcxyz_run_noalloc
    f.restype = C.c_int
    f.argtypes = [C.POINTER(abi.RunParams), C.POINTER(abi.TissueParams), C.POINTER(abi.Ext), C.c_void_p,
                  C.c_uint64, C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    rp, tp, _, ext = cases.skin_vessel_case(N=8)
    fake = C.c_void_p(0x1000)  # not a device address: only the refusals run
    code = {v: k for k, v in abi.STATUS.items()}
    for first, n in ((0, 2 ** 31 + 1), (2 ** 64 - 10, 11), (0, 2 ** 64 - 1)):
        st = f(C.byref(rp), C.byref(tp), C.byref(ext), fake, first, n, fake, None, None, None, None)
        assert st == code["NMC_EINVAL"], (first, n)
    bad = abi.Ext.from_buffer_copy(ext)
    bad.block_size = 2048
    st = f(C.byref(rp), C.byref(tp), C.byref(bad), fake, 0, 10, fake, None, None, None, None)
    assert st == code["NMC_EINVAL"]


def test_refusals_without_a_device():
    # status codes for calls that fail before any device work: kinds the
    # reference leaves empty, unknown kinds, null handles and outputs
    import ctypes as C

    from nmc_gb300 import engine

    L = engine.lib()
    h = C.c_void_p()
    code = {v: k for k, v in abi.STATUS.items()}
    assert L.nmc_create(abi.SIM_MCXYZ, 0, None) == code["NMC_EINVAL"]
    for kind in (3, 4, 5):  # polarisation / Raman / Mueller kernels are empty in the reference
        assert L.nmc_create(kind, 0, C.byref(h)) == code["NMC_EUNSUPPORTED"] and not h.value
    assert L.nmc_create(99, 0, C.byref(h)) == code["NMC_EINVAL"] and not h.value
    assert L.nmc_run(None, C.c_uint64(0), C.c_uint64(1)) == code["NMC_EINVAL"]
    assert L.nmc_prepare(None, None, None, None) == code["NMC_EINVAL"]
    assert L.nmc_set_fold_interval(None, C.c_uint64(1)) == code["NMC_EINVAL"]
    L.nmc_last_error.restype = C.c_char_p
    assert L.nmc_last_error(None) == b"null handle"
    L.nmc_destroy(None)  # a no-op


def test_invalid_configurations_refused_before_any_device_call():
    import math

    import numpy as np

    import nmc_cases as cases
    from nmc_gb300 import efield, engine, layered

    def refused(f, *a, **kw):
        with pytest.raises(engine.NMCError) as e:
            f(*a, **kw)
        assert abi.STATUS[e.value.status] == "NMC_EINVAL"

    cfg, s633, s700, st = cases.cbs_case(n_settings=1, photons=10, cone_n=8, sep_n=8)
    cfg.n_angles = 1  # a table needs two angles at least
    refused(efield.run, cfg, s633[:1], st, S_raman=s700[:1])
    cfg, s633, s700, st = cases.cbs_case(n_settings=1, photons=10, cone_n=8, sep_n=8)
    cfg.mua = float("nan")
    refused(efield.run, cfg, s633, st, S_raman=s700)
    cfg, s633, s700, st = cases.cbs_case(n_settings=1, photons=10, cone_n=8, sep_n=8)
    st[0].theta_in = 2.0  # grazing or beyond: no refracted beam
    refused(efield.run, cfg, s633, st, S_raman=s700)
    refused(layered.run, [], 10)
    refused(layered.run, [(0.1, 100.0, 0.9, 1.4, -0.1), (0.1, 100.0, 0.9, 1.4, math.inf)], 10)
    # the reference's streams need the dispatch batch (seed) to be > 0
    refused(layered.run, [(0.1, 100.0, 0.9, 1.4, math.inf)], 10, seed=0, flags=abi.FLAG_LAYERED_REF_STREAMS)
    maps = np.zeros((len(abi.EF_MAPS), 4, 4), np.float32)
    recs = np.zeros((1, 4, 4), abi.SPECKLE_DTYPE)
    refused(efield.speckle_mutual, maps, recs, np.zeros((4, 4), np.int32), float("inf"), 1.0)
