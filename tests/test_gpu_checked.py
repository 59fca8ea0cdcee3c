"""The checked build (-DNMC_CHECK_BOUNDS): every tally index is tested
against its buffer and a miss raises NMC_DEVFLAG_BOUNDS.  compute-sanitizer
is not available for these kernels, so this is the bounds check: the main
kernels run their parity cases under the checked library (in a child process:
the library is chosen at import) with no flag raised and the same results as
the normal build."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r'''
import json, sys
sys.path[:0] = [ROOT, ROOT + "/tests"]
import numpy as np
from nmc_gb300 import abi, engine, layered
import nmc_cases as cases
out = {}
rp, tp, v, ext = cases.skin_vessel_case(N=48)
for name, sim in (("xyz", abi.SIM_MCXYZ), ("tt", abi.SIM_MCXYZ_TT)):
    with engine.Engine(sim, 0, ext) as e:
        e.prepare_data(rp, tp, v)
        e.set_radial_tally(64, 0.005)
        e.run(0, 20000)
        out[name] = [float(e.summary()["rd_sum"]), float(e.tally(abi.TALLY_F3D).sum()),
                     float(e.tally(abi.TALLY_RD2D).sum()), float(e.tally(abi.TALLY_RD_R).sum())]
rp, tp, ext = cases.mcsub_case()
with engine.Engine(abi.SIM_MCSUB, 0, ext) as e:
    e.prepare_data(rp, tp)
    e.run(0, 20000)
    out["sub"] = [float(e.tally(abi.TALLY_J).sum()), float(e.tally(abi.TALLY_F).sum())]
case = cases.adjoint_case(N=24)
rp, tp, v, ext, mua, mus, g, bins, dr = case
with engine.Engine(abi.SIM_MCXYZ, 0, ext) as e:
    e.prepare_data(rp, tp, v)
    e.set_radial_tally(bins, dr)
    e.set_voxel_props(mua, mus, g)
    e.adjoint_forward(0, 20000)
    ga, gs, gg = e.adjoint_backward(np.ones(bins + 1, np.float32), np.ones(24 ** 3, np.float32))
    out["adj"] = [float(ga.sum()), float(gs.sum()), float(gg.sum())]
r = layered.run([(0.3, 120.0, 0.9, 1.4, 0.02), (5.0, 200.0, 0.85, 1.37, 0.05), (0.5, 90.0, 0.8, 1.45, 0.3)],
                20000, a_rz=True, seed=6)
out["lay"] = [float(r["Rd"]), float(r["Tt"]), float(r["A"])]
print(json.dumps(out))
'''


def _run(checked: bool) -> dict:
    env = dict(os.environ)
    env["NMC_CHECKED"] = "1" if checked else "0"
    code = "ROOT = " + repr(ROOT) + "\n" + SCRIPT
    r = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_checked_build_raises_no_flag_and_agrees():
    from nmc_gb300 import build

    build.build_checked()
    plain, checked = _run(False), _run(True)
    for k in plain:
        np.testing.assert_allclose(checked[k], plain[k], rtol=1e-6, atol=1e-9, err_msg=k)
