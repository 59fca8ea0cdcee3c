"""Cost per photon of the CPU baseline against the reference's own kernel.

TEST INFRASTRUCTURE: times, on one host and the same photons, the reference's
MCXYZKernel compiled from its own sources (oracle/_ref/libnmcref.so, built by
`make -C oracle ref` where the reference checkout exists) and the oracle's
FP32 restatement with the reference's generator (the timed CPU baseline of
bench.py), on the 200^3 skin-vessel workload at 0.005 cm.  Both keep their
fluence tallies.  Prints one JSON line per thread count: photons/s of each,
the restatement's sub-steps per photon, and the ratio of their times.

    python oracle/compare_cost.py [--photons 4000] [--threads 1 8] [--repeats 2]
"""
import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "tests"))

import nmc_cases as cases  # noqa: E402
from nmc_gb300 import abi  # noqa: E402
from oracle import bindings  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--photons", type=int, default=4000)
    ap.add_argument("--threads", type=int, nargs="+", default=[1, os.cpu_count() or 1])
    ap.add_argument("--repeats", type=int, default=2)
    a = ap.parse_args()
    bindings.build(ref=True)
    if not bindings.ref_available():
        print(json.dumps({"unavailable": "reference build not present (make -C oracle ref)"}))
        return
    rp, tp, v, ext = cases.skin_vessel_case(N=200, rng=abi.RNG_TAUS_REF)
    n = a.photons
    ext.photons_per_dispatch = n  # photons (run 1, index 0..n-1) of the reference's dispatch loop
    for th in a.threads:
        t_ref, t_port, sub = [], [], None
        for _ in range(a.repeats):
            t0 = time.perf_counter()
            r = bindings.ref_mcxyz(rp, tp, v, run_lo=1, run_hi=1, batch=n, nthreads=th)
            t_ref.append(time.perf_counter() - t0)
            t0 = time.perf_counter()
            p = bindings.run(abi.SIM_MCXYZ, rp, tp, v, ext=ext, n=n, nthreads=th, real_bits=32, tallies=True)
            t_port.append(time.perf_counter() - t0)
            sub = p["substeps"] / n
        tr, tp_ = min(t_ref), min(t_port)
        print(json.dumps({"threads": th, "photons": n, "reference_photons_per_s": n / tr,
                          "port_photons_per_s": n / tp_, "port_time_over_reference_time": tp_ / tr,
                          "port_substeps_per_photon": sub, "rd_reference": float(r["rd_slots"].sum() / n),
                          "rd_port": p["rd_sum"] / n, "host_cpus": os.cpu_count()}))


if __name__ == "__main__":
    main()
