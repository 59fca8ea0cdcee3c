"""Generates tests/golden/spectral_tissues.json from the reference's own
`tissue_parameters` (NMC-samples/example3.ipynb cell 2) run on its
spectralLIB.mat.  Needs the reference checkout; run from the repository root:
    python tests/golden/make_spectral_fixture.py /path/to/reference
"""
import json
import os
import sys

import numpy as np


def main(ref_root):
    samples = os.path.join(ref_root, "NMC-samples")
    nb = json.load(open(os.path.join(samples, "example3.ipynb")))
    src = "".join(nb["cells"][2]["source"])
    src = src[src.index("def tissue_parameters"):]
    g = {"os": os, "np": np, "spectralLIB_dir": samples}
    from scipy.io import loadmat

    g["loadmat"] = loadmat
    exec(src, g)
    data = loadmat(os.path.join(samples, "spectralLIB.mat"))
    lib = {k: np.asarray(data[k], float).ravel() for k in ("nmLIB", "muaoxy", "muadeoxy", "muawater", "muamel")}
    cases = []
    for nm in (400, 450, 532, 577, 600, 650, 700, 750):
        mu = [float(np.interp(nm, lib["nmLIB"], lib[k])) for k in ("muaoxy", "muadeoxy", "muawater", "muamel")]
        t = g["tissue_parameters"](nm)
        cases.append({"nm": nm, "mu": mu,
                      "tissues": {str(k): {"mua": float(v["mua"]), "mus": float(v["mus"]), "g": float(v["g"])}
                                  for k, v in t.items()}})
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "spectral_tissues.json")
    with open(out, "w") as f:
        json.dump(cases, f, indent=1)
    print("wrote", out)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
