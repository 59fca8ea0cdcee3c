"""Wavelength-dependent tissue tables (nmc_gb300/spectral.py) against golden
values from the reference notebook's own `tissue_parameters`
(example3.ipynb cell 2) on its spectral library, generated by
tests/golden/make_spectral_fixture.py."""
import json
import os

import numpy as np
import pytest

from nmc_gb300 import spectral

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "spectral_tissues.json")))


@pytest.mark.parametrize("case", GOLD, ids=[str(c["nm"]) for c in GOLD])
def test_tissue_list_matches_notebook(case):
    t = spectral.tissue_list(case["nm"], mu=np.array(case["mu"]))
    for k, want in case["tissues"].items():
        got = t[int(k)]
        for f in ("mua", "mus", "g"):
            assert got[f] == pytest.approx(want[f], rel=1e-12, abs=1e-15), (case["nm"], k, f)


def test_tissue_params_and_sets():
    case = GOLD[2]
    lib = {"nmLIB": np.array([case["nm"] - 1.0, case["nm"] + 1.0])}
    for i, k in enumerate(("muaoxy", "muadeoxy", "muawater", "muamel")):
        lib[k] = np.array([case["mu"][i], case["mu"][i]])
    tp = spectral.tissue_params(case["nm"], lib, two_term=dict(gf=0.9, af=0.5, gb=0.3, ab=0.5, cc=0.9))
    assert tp.muav[3] == pytest.approx(case["tissues"]["3"]["mua"], rel=1e-6)
    assert tp.musv[4] == pytest.approx(case["tissues"]["4"]["mus"], rel=1e-6)
    assert tp.CC[5] == pytest.approx(0.9)
    sets = spectral.spectral_sets([case["nm"], case["nm"]], lib, [1000, 2000])
    assert [s.photons for s in sets] == [1000, 2000]


# the reference checkout, when one is at hand: NMC_REFERENCE=<path>, else the
# checkout the oracle builds the reference kernels from
from oracle import bindings as _orc  # noqa: E402

REF_ROOT = os.environ.get("NMC_REFERENCE") or os.path.dirname(os.path.dirname(_orc.REF_SRC))
LIB_PATH = os.path.join(REF_ROOT, "NMC-samples", "spectralLIB.mat")


@pytest.mark.skipif(not os.path.exists(LIB_PATH), reason="reference spectral library not present")
def test_interpolation_in_the_library():
    lib = spectral.load_library(LIB_PATH)
    for case in GOLD:
        np.testing.assert_allclose(spectral.chromophores(case["nm"], lib), case["mu"], rtol=1e-12)
