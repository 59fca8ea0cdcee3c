"""Extracts the results the reference's sample notebooks recorded (their
saved cell outputs) into tests/golden/notebook_pins.json: the Rd of each
run, with the tissue tables example3 printed for every wavelength (the
values it wrote to _H.mci, 4 decimals).  Needs the reference checkout:
    python tests/golden/make_notebook_fixture.py /path/to/reference
"""
import json
import os
import re
import sys


def outputs(nb):
    for c in nb["cells"]:
        for o in c.get("outputs", []):
            yield "".join(o.get("text", ""))


def main(ref_root):
    d = os.path.join(ref_root, "NMC-samples")
    load = lambda n: json.load(open(os.path.join(d, n)))  # noqa: E731
    pins = {}
    t0 = "".join(outputs(load("example0.ipynb")))
    fit = re.findall(r"a = ([0-9.e+-]+), b = ([0-9.]+) 1/mm", t0)[0]
    pins["example0"] = {"Rd": float(re.findall(r"Total Rd = ([0-9.]+)", t0)[0]), "photons": 100000,
                        "a": float(fit[0]), "b": float(fit[1])}
    t1 = "".join(outputs(load("example1.ipynb")))
    pins["example1"] = {"Rd": [float(v) for v in re.findall(r"Total Rd = ([0-9.]+)", t1)]}
    t2 = "".join(outputs(load("example2.ipynb")))
    tot = re.findall(r"total simulated photons: (\d+) out of (\d+)", t2)[-1]
    pins["example2"] = {"nm": 532, "Rd": float(re.findall(r"Total Rd = ([0-9.]+)", t2)[0]), "photons": int(tot[1])}
    t3 = "".join(outputs(load("example3.ipynb")))
    runs = []
    for block in t3.split("=== Optical properties at ")[1:]:
        nm = int(block.split(" nm")[0])
        rows = re.findall(r"^\s*(\d+)\s*\|\s*([0-9.]+)\s*\|\s*([0-9.]+)\s*\|\s*([0-9.]+)", block, re.M)
        rd = re.findall(r"Rd \(MC\) @ %d nm: ([0-9.]+)" % nm, block)
        runs.append({"nm": nm, "tissues": [[float(a), float(b), float(c)] for _, a, b, c in rows],
                     "Rd": float(rd[0]) if rd else None})
    pins["example3"] = runs
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "notebook_pins.json")
    with open(out, "w") as f:
        json.dump(pins, f, indent=1)
    print("wrote", out, len(runs), "example3 runs")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
