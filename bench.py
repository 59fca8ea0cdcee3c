"""Benchmark: photons/s of the voxel photon-transport path on the 200^3
skin-vessel workload (mcxyz kernel, 1e8 photons per step).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one pass of the transport over the workload's photon budget
(1e8 photons per GPU) with inputs resident in HBM.  Prints one JSON line.

  value     photons/s over all ranks, device time (CUDA events) of K steps
  e2e       photons/s through the C ABI with host buffers: nmc_prepare (H2D of
            the tissue map), nmc_run, nmc_get_compute_results (D2H of F3D,
            Rd slots, Rd2D, DetPhot2D) inside the timed region
  roofline  the transport kernel against the measured FP32-issue ceiling
  cpu_baseline  the reference algorithm restated on the host cores (FP32,
            the reference's own generator, fluence tally kept), a bounded
            sample of the workload, with its sub-steps per photon and the
            ratio at equal work (sub-steps/s)

Extras in the same line (each with its own rate, its unit-of-work rate
against the FP32-issue ceiling and a CPU baseline): the 351-wavelength sweep
to 1 % Rd SE against plain runs, the pMC adjoint against a forward (1e7
photons, Rd(r) and Rd(r) + fluence losses), C1 (mcsub, 1e6 photons), the
three-layer stack (1e8 photons) and C5 (E-field / CBS / Raman, 1e8 photons).

--impl reference times that CPU restatement alone on the same workload (the
reference runs only on Apple Metal; its kernels cannot execute on this machine).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

METRIC = "photons/s at 1% Rd std-err, batched+adjoint vs plain kernel, 1×GB300"
PHOTONS_PER_STEP = 100_000_000
WORKLOAD = "mcxyz skin-vessel 200^3 @0.005 cm, 1e8 photons per GPU per step"

# Algorithmic work of one voxel sub-step (the kernel's loop trip), counted
# from the source of the transport loop: FP32/INT lane operations issued on
# the FMA/ALU pipes for the sub-step proper (position update, same-voxel
# test, face distances, absorption, voxel index and tissue lookup) and the
# per-hop SPIN/roulette share.  Fixed once, not re-counted per build.
OPS_PER_SUBSTEP = 64.0
MUFU_PER_SUBSTEP = 3.0
# The same count for the other transport kernels' units, fixed once from
# their loop bodies: one Philox4x32-10 block (~109 integer lane operations:
# 10 rounds of 4 multiply halves, 4 xors and 2 key adds, plus 3 uniform
# conversions) per step or scattering, plus the FP32 work of the step.
OPS_PER_MCSUB_STEP = 164.0     # HOP 5, DROP + F(r,z) index 21, HG + SPIN 24, roulette/loop 5, Philox 109
MUFU_PER_MCSUB_STEP = 9.0
OPS_PER_LAYERED_STEP = 170.0   # an mcsub step plus the distance to the layer boundary
OPS_PER_EF_SCATTER = 320.0     # step 17, theta search 26, S1/S2 12, phi density + Newton 54, frame 43,
                               # Jones update 51, loop 8, Philox 109
MUFU_PER_EF_SCATTER = 14.0
# Warp instructions the transport kernel issues per voxel sub-step
# (smsp__inst_executed.sum / sub-steps of the 1e7-photon ncu capture of this
# workload), and the SM's issue rate (4 warp instructions per clock).
WARP_INSTR_PER_SUBSTEP = 317_868_610_037 / 2.5583e10
ISSUE_PER_SM_CLOCK = 4.0
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one 1e8-photon
# launch of the transport kernel on this workload, captured on that launch
# (one ncu pass): 72.10 MB read, 121 KB written.  With the fluence tally
# persisting in L2 they are the first touch of the 8 MB map and the 64 MB
# tally; before it, the L2 wrote tally lines back under the atomics, about
# 29 GB per launch.
TRAFFIC_BYTES_PER_LAUNCH = 72_100_000 + 121_340
HBM_PEAK_FALLBACK_GBS = 6800.0


def _clock_sampler(stop: threading.Event, out: list, dev: int):
    q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    try:
        p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                              "-i", str(dev), "-lms", "200"], stdout=subprocess.PIPE, text=True)
    except Exception:
        return
    try:
        while not stop.is_set():
            line = p.stdout.readline()
            if not line:
                break
            out.append(line.strip())
    finally:
        p.terminate()


def _clocks_summary(lines: list) -> dict:
    import statistics

    sm, mx, reasons = [], 0.0, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for ln in lines:
        f = [x.strip() for x in ln.split(",")]
        if len(f) < 9:
            continue
        try:
            sm.append(float(f[1]))
            mx = max(mx, float(f[2]))
        except ValueError:
            continue
        for n, v in zip(names, f[5:9]):
            if v.lower() == "active":
                reasons.add(n)
    return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
            "reasons": sorted(reasons), "samples": len(sm)}


def _issue_estimate(substeps_per_s, clock_lines) -> dict | None:
    import torch

    c = _clocks_summary(clock_lines)
    mhz = c.get("sm_mhz") if isinstance(c, dict) else None
    if not substeps_per_s or not mhz:
        return None
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    per_s = substeps_per_s * WARP_INSTR_PER_SUBSTEP
    peak = sms * ISSUE_PER_SM_CLOCK * mhz * 1e6
    return {"warp_instr_per_substep": WARP_INSTR_PER_SUBSTEP, "achieved_warp_instr_per_s": per_s,
            "peak_warp_instr_per_s": peak, "frac": per_s / peak,
            "source": "instructions per sub-step from ncu (profiles/mcxyz_skinvessel_traffic.txt), "
                      "sub-step rate live, SMs x 4 issues per clock at the median sampled SM clock"}


def cpu_sample(seconds: float = 12.0, threads: int | None = None) -> dict:
    """The reference algorithm on the host cores: the oracle's FP32 restatement
    with the reference's Tausworthe generator (which reproduces the
    reference's FP32 voxel walk), with its fluence tally (the reference
    kernel always deposits into F3D), on a bounded sample of the workload.
    On one host this restatement costs what the reference's own kernel,
    compiled from its sources, costs per photon (oracle/compare_cost.py)."""
    import nmc_cases as cases
    from nmc_gb300 import abi
    from oracle import bindings

    bindings.build(ref=False)
    threads = threads or os.cpu_count() or 1
    rp, tp, v, ext = cases.skin_vessel_case(N=200, rng=abi.RNG_TAUS_REF)
    n = 64 * threads
    bindings.run(abi.SIM_MCXYZ, rp, tp, v, ext=ext, n=n, nthreads=threads, real_bits=32, tallies=True)  # warm-up
    first, photons, secs, subs = n, 0, 0.0, 0
    while secs < seconds:  # growing runs until the sample holds about `seconds` of work
        t0 = time.perf_counter()
        r = bindings.run(abi.SIM_MCXYZ, rp, tp, v, ext=ext, first=first, n=n, nthreads=threads, real_bits=32,
                         tallies=True)
        dt = time.perf_counter() - t0
        first, photons, secs, subs = first + n, photons + n, secs + dt, subs + r["substeps"]
        rate = photons / secs
        n = max(threads, min(4 * n, int(rate * max(seconds - secs, 0.5)) + 1))
    return {"photons": photons, "seconds": secs, "photons_per_s": photons / secs, "threads": threads,
            "substeps_per_photon": subs / photons}


def run_reference(args) -> dict:
    """--impl reference: the reference's photon-step algorithm on host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return {}
    threads = os.cpu_count() or 1
    per_step_s = 6.0
    samples = []
    for i in range(args.warmup + args.steps):
        s = cpu_sample(per_step_s if i >= args.warmup else 2.0, threads)
        if i >= args.warmup:
            samples.append(s)
    ph = sum(s["photons"] for s in samples)
    sec = sum(s["seconds"] for s in samples)
    v = ph / sec
    sub = sum(s["substeps_per_photon"] * s["photons"] for s in samples) / max(ph, 1)
    desc = (f"{ph} photons of the 200^3 skin-vessel workload in {args.steps} samples, FP32 restatement with "
            f"the reference's generator, {threads} threads")
    return {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "photons/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sec / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": {"workload": WORKLOAD, "photons_per_step_sampled": ph // args.steps},
        "cpu_baseline": {"value": v, "unit": "photons/s", "cores": threads, "kind": "port", "sample": desc,
                         "substeps_per_photon": sub, "substeps_per_s": v * sub},
        "e2e": {"value": v, "unit": "photons/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_ours(args) -> dict:
    import numpy as np
    import torch

    import nmc_cases as cases
    from nmc_gb300 import abi, build, engine

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    if rank == 0 or world == 1:
        build.build()
    if dist:
        dist.barrier()

    P = args.photons
    rp, tp, v, ext = cases.skin_vessel_case(N=200)
    e = engine.Engine(abi.SIM_MCXYZ, local, ext)
    e.prepare_data(rp, tp, v)
    tuned = e.autotune(args.tune) if args.tune > 0 else None
    stream = torch.cuda.ExternalStream(e.stream)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")  # > L2 (129 MB)
    base = rank * 10 ** 12  # disjoint photon ids per rank

    def step(i):
        e.run_async(base + i * P, P)

    for i in range(args.warmup):
        step(i)
        e.synchronize()
    if args.profile_only:  # the transport launches alone, for ncu captures
        for i in range(args.steps):
            step(args.warmup + i)
            e.synchronize()
        s = e.summary()
        e.close()
        print(json.dumps({"profile_only": True, "photons": s["photons"], "kernel_ms": s["kernel_ms"],
                          "launches": s["launches"]}))
        return {}
    e.reset()
    s0 = e.summary()

    # -- timed region: device time of K steps (L2 flushed before each step)
    clock_lines, stop = [], threading.Event()
    th = threading.Thread(target=_clock_sampler, args=(stop, clock_lines, local), daemon=True)
    th.start()
    times = []
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    for i in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        step(args.warmup + i)
        b.record(stream)
        e.synchronize()
        times.append(a.elapsed_time(b))
    torch.cuda.synchronize()
    stop.set()
    th.join(timeout=2)
    s1 = e.summary()
    total_ms = float(sum(times))
    if dist:
        t = torch.tensor([total_ms], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    photons_all = P * args.steps * world
    value = photons_all / (total_ms * 1e-3)
    launches = s1["launches"] - s0["launches"]
    kernel_ms = s1["kernel_ms"] - s0["kernel_ms"]
    substeps = s1["substeps"] - s0["substeps"]
    rd_mean = s1["rd_sum"] / max(s1["photons"], 1)
    rd_var = s1["rd_sumsq"] / max(s1["photons"], 1) - rd_mean ** 2
    rd_se = (rd_var / max(s1["photons"], 1)) ** 0.5
    e.close()

    # -- e2e through the C ABI with host buffers (prepare H2D + run + results D2H)
    e2 = engine.Engine(abi.SIM_MCXYZ, local, ext)
    e2_times = []
    h2d = v.nbytes + 172 + 608
    n2d = rp.Nx * rp.Ny
    d2h = rp.Nx * rp.Ny * rp.Nz * 4 + ext.photons_per_dispatch * 4 + 2 * n2d * 4
    for i in range(1 + min(args.steps, 3)):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2.prepare_data(rp, tp, v)
        e2.run(base + (10 ** 9) + i * P, P)
        res = e2.get_compute_results()
        dt = time.perf_counter() - t0
        if i > 0:
            e2_times.append(dt)
    assert np.isfinite(res["F3D"]).all()
    e2.close()
    e2e_value = P * world / (sum(e2_times) / len(e2_times))

    # -- roofline: transport kernel against the measured FP32 issue ceiling
    ffma, mufu = engine.probe_issue_peaks(local)
    kernel_s = kernel_ms * 1e-3
    achieved = substeps * OPS_PER_SUBSTEP / kernel_s / 1e12 if kernel_s > 0 else None
    peak = ffma / 1e12
    traffic = TRAFFIC_BYTES_PER_LAUNCH  # per launch: first touches of the map and the L2-resident tally
    try:
        hbm_peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
        hbm_src = "measured"
    except Exception:
        hbm_peak, hbm_src = HBM_PEAK_FALLBACK_GBS, "fallback"
    launch_s = kernel_s / max(launches, 1)
    hbm_gbs = traffic / launch_s / 1e9 if launch_s > 0 else None
    out = {
        "metric": METRIC, "value": value, "unit": "photons/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": WORKLOAD, "photons_per_step": P, "grid": [200, 200, 200], "voxel_cm": 0.005,
                   "l2": "256 MB buffer written before each timed step", "rng": "philox4x32-10",
                   "rd": rd_mean, "rd_rel_se": rd_se / rd_mean if rd_mean else None,
                   "substeps_per_photon": substeps / max(P * args.steps, 1),
                   "parallelism": f"replicas{world}",
                   "launch": ({"autotuned_on_photons": args.tune, **tuned["best"]} if tuned
                              else {"block_size": 256, "blocks_per_sm": "max resident"})},
        "e2e": {"value": e2e_value, "unit": "photons/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "roofline": {"bound": "fp32_issue", "achieved": achieved, "peak": peak, "unit": "Tlane-op/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "kernel": "mcxyz_kernel", "ops_per_substep": OPS_PER_SUBSTEP,
                     "substeps_per_s": substeps / kernel_s if kernel_s > 0 else None,
                     "mufu_peak_tlanes": mufu / 1e12,
                     "peak_source": "of measured FP32 FMA lane rate (nmc_probe_issue_peaks, live)",
                     "hbm": {"achieved_gbs": hbm_gbs, "peak_gbs": hbm_peak, "peak_source": hbm_src,
                             "frac": (hbm_gbs / hbm_peak) if hbm_gbs else None},
                     # the instruction-issue ceiling for the instruction stream the kernel
                     # executes: live sub-step rate x profiled instructions per sub-step
                     # against 4 issues per SM clock at the sampled SM clock
                     "issue": _issue_estimate(substeps / kernel_s if kernel_s > 0 else None, clock_lines)},
        "gpu_launches": launches,
        "clocks": _clocks_summary(clock_lines),
    }
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            cs = cpu_sample(12.0)
            gpu_sub_s = value * out["config"]["substeps_per_photon"]
            cpu_sub_s = cs["photons_per_s"] * cs["substeps_per_photon"]
            out["cpu_baseline"] = {"value": cs["photons_per_s"], "unit": "photons/s", "cores": cs["threads"],
                                   "kind": "port",
                                   "sample": f"{cs['photons']} photons of the same workload, FP32 restatement with "
                                             f"the reference's generator and its fluence tally "
                                             f"({cs['substeps_per_photon']:.0f} sub-steps/photon), "
                                             f"{cs['seconds']:.1f} s",
                                   "substeps_per_photon": cs["substeps_per_photon"], "substeps_per_s": cpu_sub_s,
                                   # photons/s ratio, and the ratio at equal work: the reference's FP32
                                   # walk stalls at voxel faces and takes ~4x the sub-steps per photon
                                   "photons_ratio": value / cs["photons_per_s"],
                                   "equal_work_ratio": gpu_sub_s / cpu_sub_s}
        except Exception as exc:  # noqa: BLE001
            out["cpu_baseline"] = {"value": None, "unit": "photons/s", "error": f"{type(exc).__name__}: {exc}"}
    if rank == 0 and world == 1 and not args.no_extras:
        cpu = not args.no_cpu
        for key, fn in (("batched_to_1pct_se", batched_to_target_extra), ("adjoint", adjoint_extra),
                        ("mcsub_c1", lambda: mcsub_extra(ffma, cpu)), ("layered", lambda: layered_extra(ffma, cpu)),
                        ("cbs_c5", lambda: cbs_extra(ffma, cpu))):
            try:  # an extra that fails is reported in the line, not in place of it
                out[key] = fn()
            except Exception as exc:  # noqa: BLE001
                out[key] = {"error": f"{type(exc).__name__}: {exc}"}
    if dist:
        dist.destroy_process_group()
    return out if rank == 0 else {}


def _plain_sweep(e, sets, rp, v, ext_for, target, reprepare, pilot=20000):
    """One plain run per wavelength on the same photon streams as the batched
    sweep (set s: seed 11 + (s << 32)); with a target, the batched sweep's
    pilot + top-up rule.  Returns (Rd, relative SE, photons) per set."""
    import numpy as np

    rd = np.zeros(len(sets))
    rse = np.zeros(len(sets))
    photons = 0
    for i, q in enumerate(sets):
        e.set_ext(ext_for(11 + (i << 32)))
        if reprepare:
            e.prepare_data(rp, q.tp, v)
        else:
            e.set_tissue_params(q.tp)
            e.reset()
        if target is None:
            e.run(0, q.photons)
        else:
            n1 = min(pilot, q.photons)
            e.run(0, n1)
            s1 = e.summary()
            me = s1["rd_sum"] / n1
            var = max(s1["rd_sumsq"] / n1 - me * me, 1e-30)
            need = int(np.ceil(1.15 * var / (target * max(me, 1e-30)) ** 2))
            extra = max(min(need, q.photons) - n1, 0)
            if extra:
                e.run(n1, extra)
        sm = e.summary()
        n = sm["photons"]
        photons += n
        rd[i] = sm["rd_sum"] / n
        rse[i] = np.sqrt(max(sm["rd_sumsq"] / n - rd[i] ** 2, 0) / n) / rd[i]
    return rd, rse, photons


def _timed(fn):
    import torch

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = fn()
    torch.cuda.synchronize()
    return r, time.perf_counter() - t0


def batched_to_target_extra() -> dict:
    """The 351-wavelength skin-vessel sweep brought to 1% relative SE in Rd:
    batched (pilot + top-up launches) against one plain run per wavelength
    with the same rule (table swapped in place)."""
    import numpy as np

    import nmc_cases as cases
    from nmc_gb300 import abi, engine
    from nmc_gb300 import sweep as nsweep

    lam, tables, budgets = cases.skin_vessel_spectral_tables()
    sets = [nsweep.TissueSet(t, b) for t, b in zip(tables, budgets)]
    rp, _, v, _ = cases.skin_vessel_case(N=200, d=0.005)
    ext_for = lambda seed: abi.ext_defaults(rng=abi.RNG_PHILOX, seed=seed)  # noqa: E731
    with engine.Engine(abi.SIM_MCXYZ_TT, 0, ext_for(11)) as e:
        e.prepare_data(rp, tables[0], v)
        e.run_sweep_tissues(tables[:8], [20000] * 8)
        tgt, b_s = _timed(lambda: nsweep.sweep(e, sets, target_rel_se=0.01))
        (_, p_rse, p_n), p_s = _timed(lambda: _plain_sweep(e, sets, rp, v, ext_for, 0.01, False))
    n = int(tgt["photons"].sum())
    return {"batched_s": b_s, "plain_s": p_s, "speedup": p_s / b_s, "photons": n,
            "photons_per_s": n / b_s, "max_rel_se": float((tgt["Rd_se"] / tgt["Rd"]).max()),
            "plain_max_rel_se": float(p_rse.max()), "launches": tgt["launches"],
            "workload": "skin-vessel 200^3, 351 wavelengths, two-term HG, to 1% Rd SE"}


def adjoint_extra(n: int = 10_000_000) -> dict:
    """Forward + pMC adjoint against a plain forward on the 64^3 per-voxel
    medium at 1e7 photons, for a loss on Rd(r) and for a loss on Rd(r) plus
    the fluence (absorbed weight per voxel)."""
    import numpy as np

    import nmc_cases as cases
    from nmc_gb300 import abi, engine

    rp, tp, v, ext, mua, mus, g, bins, dr = cases.adjoint_case()
    G = np.random.default_rng(3).uniform(0.5, 1.5, bins + 1).astype(np.float32)
    GF = np.random.default_rng(4).uniform(0.5, 1.5, rp.Nx * rp.Ny * rp.Nz).astype(np.float32)
    with engine.Engine(abi.SIM_MCXYZ, 0, ext) as e:
        e.prepare_data(rp, tp, v)
        e.set_radial_tally(bins, dr)
        e.set_voxel_props(mua, mus, g)
        fwd = lambda: (e.reset(), e.run(0, n))  # noqa: E731
        adj = lambda: (e.reset(), e.adjoint_forward(0, n, 8 * n), e.adjoint_backward(G))  # noqa: E731
        # a fluence loss: the forward keeps its deposit list (600 records of
        # 8 bytes per photon), so the backward needs no score replay
        adj_f = lambda: (e.reset(), e.adjoint_forward(0, n, 8 * n, 600 * n), e.adjoint_backward(G, GF))  # noqa: E731
        fwd(), adj(), adj_f()
        t_f = min(_timed(fwd)[1] for _ in range(3))
        t_a = min(_timed(adj)[1] for _ in range(3))
        t_af = min(_timed(adj_f)[1] for _ in range(3))
        list_ok = e.deposit_list_complete
    return {"forward_s": t_f, "forward_adjoint_s": t_a, "cost_ratio": t_a / t_f,
            "forward_adjoint_fluence_s": t_af, "cost_ratio_fluence": t_af / t_f, "photons": n,
            "deposit_list_complete": list_ok,
            "workload": "64^3 per-voxel medium, 1e7 photons; gradients w.r.t. all voxel mua, mus, g of a loss on "
                        "Rd(r) (cost_ratio) and on Rd(r) + fluence (cost_ratio_fluence)",
            "timing": "best of 3 host-timed synchronised calls each"}


def _unit_roofline(units: float, seconds: float, ops_per_unit: float, ffma_lanes_per_s: float, unit: str,
                   timing: str) -> dict:
    achieved = units * ops_per_unit / seconds / 1e12
    peak = ffma_lanes_per_s / 1e12
    return {"bound": "fp32_issue", "unit_of_work": unit, "units_per_s": units / seconds,
            "ops_per_unit": ops_per_unit, "achieved": achieved, "peak": peak, "unit": "Tlane-op/s",
            "frac": achieved / peak, "peak_source": "of measured FP32 FMA lane rate (nmc_probe_issue_peaks, live)",
            "timing": timing}


def mcsub_extra(ffma: float, cpu: bool = True) -> dict:
    """C1: semi-infinite medium (mua 1, mus 100 /cm, HG g 0.9, n 1.37/1.0),
    normal pencil beam, Rd(r) 100 x 0.01 cm, F(r, z) 100 x 100 x 0.01 cm,
    1e6 photons per launch (Philox seed 0), device-timed over 10 launches;
    the CPU baseline runs the full 1e6 photons through the FP32 restatement
    with the reference's generator on all host cores."""
    import nmc_cases as cases
    from nmc_gb300 import abi, engine

    rp, tp, ext = cases.mcsub_case()
    n, K = 1_000_000, 10
    with engine.Engine(abi.SIM_MCSUB, 0, ext) as e:
        e.prepare_data(rp, tp)
        e.run(0, n)
        e.reset()
        s0 = e.summary()
        (_, wall) = _timed(lambda: [e.run(i * n, n) for i in range(K)])
        s1 = e.summary()
    kernel_s = (s1["kernel_ms"] - s0["kernel_ms"]) * 1e-3
    steps = s1["substeps"] - s0["substeps"]
    out = {"value": K * n / kernel_s, "unit": "photons/s", "photons": K * n, "kernel_s": kernel_s, "wall_s": wall,
           "steps_per_photon": steps / (K * n), "rd": s1["rd_sum"] / max(s1["photons"], 1),
           "roofline": _unit_roofline(steps, kernel_s, OPS_PER_MCSUB_STEP, ffma, "mcsub step",
                                      "CUDA events around the 10 transport launches"),
           "workload": "C1 mcsub mua 1, mus 100, g 0.9, n 1.37/1.0, pencil beam, 1e6 photons per launch"}
    if cpu:
        from oracle import bindings

        bindings.build(ref=False)
        threads = os.cpu_count() or 1
        ext_c = cases.mcsub_case(rng=abi.RNG_TAUS_REF)[2]
        t0 = time.perf_counter()
        r = bindings.run(abi.SIM_MCSUB, rp, tp, ext=ext_c, n=n, nthreads=threads, real_bits=32, tallies=True)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": n / dt, "unit": "photons/s", "cores": threads, "kind": "port",
                               "sample": f"the full 1e6 photons, FP32 restatement with the reference's generator "
                                         f"and tallies, {dt:.1f} s",
                               "steps_per_photon": r["substeps"] / n}
    return out


def layered_extra(ffma: float, cpu: bool = True) -> dict:
    """Layered media: the three-layer skin stack, 1e8 photons per call."""
    import nmc_cases as cases
    from nmc_gb300 import layered

    n = 100_000_000
    kw = dict(nr=100, dr=0.01, nz=100, dz=0.01, seed=11)
    layered.run(cases.LAYERED_SKIN3, 1_000_000, **kw)
    best, r = None, None
    for _ in range(2):
        r, t = _timed(lambda: layered.run(cases.LAYERED_SKIN3, n, **kw))
        best = t if best is None else min(best, t)
    out = {"value": n / best, "unit": "photons/s", "photons": n, "seconds": best, "rd": r["rd"],
           "interactions_per_photon": r["interactions"] / n,
           "roofline": _unit_roofline(r["interactions"], best, OPS_PER_LAYERED_STEP, ffma, "layered interaction",
                                      "host clock around the call (allocation, launch, tally copies): a lower "
                                      "bound of the kernel's rate"),
           "workload": "3 layers: 0.01 cm (mua 3, mus 200, g 0.8, n 1.4), 0.2 cm (0.3, 150, 0.85, 1.4), "
                       "semi-infinite (0.1, 100, 0.9, 1.44); pencil beam; Rd(r), Tt(r), A(z)"}
    if cpu:
        from oracle import bindings as orc

        threads = os.cpu_count() or 1
        sample = 200_000
        t0 = time.perf_counter()
        orc.layered(cases.LAYERED_SKIN3, sample, real_bits=32, nthreads=threads, **kw)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": sample / dt, "unit": "photons/s", "cores": threads, "kind": "port",
                               "sample": f"{sample} photons of the same stack, FP32 CPU restatement, {dt:.1f} s"}
    return out


def cbs_extra(ffma: float, cpu: bool = True) -> dict:
    """C5: polarised E-field transport with the CBS cone and Raman, 1e8
    photons over 8 polarisation / incidence settings in one launch."""
    import nmc_cases as cases
    from nmc_gb300 import efield

    total = 100_000_000
    cfg, S633, S700, settings = cases.cbs_case(n_settings=8, photons=total // 8)
    warm = cases.cbs_case(n_settings=8, photons=20_000)[3]
    efield.run(cfg, S633, warm, S_raman=S700)
    r, t = _timed(lambda: efield.run(cfg, S633, settings, S_raman=S700))
    n = float(r["photons"].sum())
    scat = float(r["scatters"].sum())
    out = {"value": n / t, "unit": "photons/s", "photons": n, "seconds": t, "scatterings_per_photon": scat / n,
           "rd": float(r["Rd"].sum() / n),
           "co_enhancement": float(1 + r["interf_co"].sum() / r["multi_co"].sum()),
           "raman_conversions": float(r["raman_n"].sum()),
           "roofline": _unit_roofline(scat, t, OPS_PER_EF_SCATTER, ffma, "E-field scattering",
                                      "host clock around the call (tables, launch, cone transform, copies): a "
                                      "lower bound of the kernel's rate"),
           "workload": "spheres 0.5 um 1.59/1.33, 633 nm, mus 100, mua 0.01 /cm; cone 256^2 within +-5 mrad; Raman "
                       "1e-4 /cm to 700 nm; 8 settings"}
    if cpu:
        from oracle import bindings as orc

        threads = os.cpu_count() or 1
        per = 4_000
        sample = cases.cbs_case(n_settings=8, photons=per)[3]
        t0 = time.perf_counter()
        orc.efield(cfg, S633, sample, S_raman=S700, cone=True, real_bits=32, nthreads=threads)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": 8 * per / dt, "unit": "photons/s", "cores": threads, "kind": "port",
                               "sample": f"{8 * per} photons of the same 8 settings, FP32 CPU restatement of the "
                                         f"E-field model, {dt:.1f} s"}
    return out


def run_sweep_workload(args) -> dict:
    """351-wavelength batched sweep on the 200^3 skin-vessel map (two-term
    phase function, per-tissue spectra, budgets log-uniform in 1e5-1e7; the
    reference runs one `nmc` process per wavelength on this map,
    example3.ipynb cell 5).  Comparisons on the same photon streams:
    (1) every set's full budget: one persistent launch against 351 plain
        runs (swap the tissue table, run);
    (2) until every set reaches 1% relative standard error in Rd: batched
        (pilot + top-up: 2 launches) against plain runs with the same pilot
        and top-up rule per wavelength, with the table swapped in place and
        with a full nmc_prepare per wavelength (the reference's per-process
        reload of the map)."""
    import numpy as np
    import torch

    import nmc_cases as cases
    from nmc_gb300 import abi, build, engine
    from nmc_gb300 import sweep as nsweep

    build.build()
    torch.cuda.set_device(0)
    lam, tables, budgets = cases.skin_vessel_spectral_tables()
    if args.budget_scale != 1.0:
        budgets = np.maximum((budgets * args.budget_scale).astype(np.int64), 1)
    sets = [nsweep.TissueSet(t, b) for t, b in zip(tables, budgets)]
    total = int(budgets.sum())
    rp, tp0, v, ext = cases.skin_vessel_case(N=200, d=0.005, seed=11)

    def ext_for(seed):
        return abi.ext_defaults(rng=abi.RNG_PHILOX, seed=seed)

    e = engine.Engine(abi.SIM_MCXYZ_TT, 0, ext_for(11))
    e.prepare_data(rp, tables[0], v)
    e.run_sweep_tissues(tables[:8], [20000] * 8)  # warm-up

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - t0

    res, batched_s = timed(lambda: nsweep.sweep(e, sets))
    if args.profile_only:  # the batched launch alone, for ncu captures
        e.close()
        print(json.dumps({"profile_only": True, "photons": int(res["photons"].sum()), "seconds": batched_s}))
        return {}
    tgt, batched_tgt_s = timed(lambda: nsweep.sweep(e, sets, target_rel_se=0.01))
    pilot = 20000

    def plain(target, reprepare):
        return _plain_sweep(e, sets, rp, v, ext_for, target, reprepare, pilot)

    (plain_rd, _, _), plain_s = timed(lambda: plain(None, False))
    (_, plain_tgt_rse, plain_tgt_n), plain_tgt_s = timed(lambda: plain(0.01, False))
    (_, _, prep_tgt_n), prep_tgt_s = timed(lambda: plain(0.01, True))
    e.close()
    rel_se = res["Rd_se"] / res["Rd"]
    tgt_rel = tgt["Rd_se"] / tgt["Rd"]
    n_tgt = int(tgt["photons"].sum())
    return {
        "metric": "photons/s, 351-wavelength batched skin-vessel sweep vs plain per-wavelength runs",
        "unit": "photons/s", "value": total / batched_s, "plain_value": total / plain_s,
        "speedup": plain_s / batched_s, "photons": total, "batched_s": batched_s, "plain_s": plain_s,
        "n_sets": len(sets), "sets_at_1pct_se": int((rel_se <= 0.01).sum()), "max_rel_se": float(rel_se.max()),
        "rd_matches_plain": float(np.max(np.abs(plain_rd - res["Rd"]) / res["Rd"])),
        "to_1pct_se": {"batched_s": batched_tgt_s, "photons": n_tgt, "launches": tgt["launches"],
                       "max_rel_se": float(tgt_rel.max()),
                       "plain_swap_s": plain_tgt_s, "speedup_vs_plain_swap": plain_tgt_s / batched_tgt_s,
                       "plain_prepare_s": prep_tgt_s, "speedup_vs_plain_prepare": prep_tgt_s / batched_tgt_s,
                       "plain_photons": int(plain_tgt_n), "plain_max_rel_se": float(plain_tgt_rse.max()),
                       "photons_per_s_at_1pct": n_tgt / batched_tgt_s},
        "substeps_per_photon": float(res["hops"].sum() / total), "dtype": "f32", "data": "synthetic",
        "config": {"workload": "skin-vessel 200^3 @ 0.005 cm, 351 wavelengths 400-750 nm, two-term HG "
                               "(g_f 0.9, g_b -0.3, forward weight 0.9), per-tissue seeded spectra, "
                               "budgets log-uniform 1e5-1e7",
                   "kernel": "mcxyz two-term (MCXYZKernelTT semantics)", "rng": "philox4x32-10",
                   "tallies": "batched: Rd, A per set; plain: the kernel's full tallies (F3D, Rd2D, Rd, A)"},
    }


def run_sweep_mcsub_workload(args) -> dict:
    """351-wavelength batched sweep on the mcsub geometry (the C1 medium; two-term phase
    function, budgets log-uniform in 1e5-1e7).  Two comparisons on the same
    photon streams: (1) every set's full budget in one persistent launch
    against 351 plain per-wavelength runs; (2) time until every set reaches
    1% relative standard error in Rd (pilot + top-up), batched (2 launches)
    against plain (2 runs per wavelength)."""
    import numpy as np
    import torch

    import nmc_cases as cases
    from nmc_gb300 import abi, build, engine
    from nmc_gb300 import sweep as nsweep

    build.build()
    torch.cuda.set_device(0)
    lam, sets = cases.spectral_sweep_sets()
    total = int(sum(s.photons for s in sets))
    flags = abi.FLAG_SKIP_FLUENCE  # both sides tally Rd, J and totals only

    def ext_for(seed):
        return abi.ext_defaults(phase=abi.PHASE_TWO_TERM, sub_bins=101, sub_dr=0.01, sub_dz=0.01, seed=seed,
                                flags=flags)

    rp, tp, _ = cases.mcsub_case(tt=(0.9, 0.5, 0.3, 0.5, 0.9))
    e = engine.Engine(abi.SIM_MCSUB, 0, ext_for(11))
    e.prepare_data(rp, tp)
    warm = [nsweep._copy(s, photons=20000) for s in sets[:8]]
    e.run_sweep(warm)

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - t0

    res, batched_s = timed(lambda: e.run_sweep(sets))
    tgt, batched_tgt_s = timed(lambda: nsweep.sweep(e, sets, target_rel_se=0.01))

    def plain(target):
        rd = np.zeros(len(sets))
        rse = np.zeros(len(sets))
        photons = 0
        for i, q in enumerate(sets):
            e.set_ext(ext_for(11 + (i << 32)))
            tps = abi.tissue_params(mua=[q.mua], mus=[q.mus], g=[q.g], gf=[q.gf], af=[q.af], gb=[q.gb],
                                    ab=[q.ab], cc=[q.cc])
            rp.n1, rp.n2 = q.n1, q.n2
            e.prepare_data(rp, tps)
            if target is None:
                e.run(0, q.photons)
            else:  # same pilot + top-up rule as the batched sweep
                n1 = min(20000, q.photons)
                e.run(0, n1)
                s1 = e.summary()
                me = s1["E"] / n1
                var = max(s1["rd_sumsq"] / n1 - me * me, 1e-30)
                rd1 = (s1["S"] + s1["E"]) / n1
                need = int(np.ceil(1.15 * var / (target * max(rd1, 1e-30)) ** 2))
                extra = max(min(need, q.photons) - n1, 0)
                if extra:
                    e.run(n1, extra)
            sm = e.summary()
            n = sm["photons"]
            photons += n
            me = sm["E"] / n
            rd[i] = (sm["S"] + sm["E"]) / n
            rse[i] = np.sqrt(max(sm["rd_sumsq"] / n - me * me, 0) / n) / rd[i]
        return rd, rse, photons

    (plain_rd, _, _), plain_s = timed(lambda: plain(None))
    (plain_tgt_rd, plain_tgt_rse, plain_tgt_n), plain_tgt_s = timed(lambda: plain(0.01))
    e.close()
    rel_se = res["Rd_se"] / res["Rd"]
    tgt_rel = tgt["Rd_se"] / tgt["Rd"]
    return {
        "metric": "photons/s, 351-wavelength batched sweep vs plain per-wavelength runs", "unit": "photons/s",
        "value": total / batched_s, "plain_value": total / plain_s, "speedup": plain_s / batched_s,
        "photons": total, "batched_s": batched_s, "plain_s": plain_s, "n_sets": len(sets),
        "sets_at_1pct_se": int((rel_se <= 0.01).sum()), "max_rel_se": float(rel_se.max()),
        "rd_matches_plain": float(np.max(np.abs(plain_rd - res["Rd"]) / res["Rd"])),
        "to_1pct_se": {"batched_s": batched_tgt_s, "plain_s": plain_tgt_s, "speedup": plain_tgt_s / batched_tgt_s,
                       "photons": int(tgt["photons"].sum()), "plain_photons": int(plain_tgt_n),
                       "launches": tgt["launches"], "max_rel_se": float(tgt_rel.max()),
                       "plain_max_rel_se": float(plain_tgt_rse.max())},
        "hops_per_photon": float(res["hops"].sum() / total), "dtype": "f32", "data": "synthetic",
        "config": {"workload": "mcsub semi-infinite, 351 wavelengths 400-750 nm, two-term HG, budgets 1e5-1e7",
                   "rng": "philox4x32-10", "tallies": "Rd, J(r), S/A/E per set (no F(r,z) on either side)"},
    }


def run_adjoint_workload(args) -> dict:
    """Forward + pMC adjoint on the 64^3 per-voxel medium (smoothed seeded
    noise mua in [0.1, 5], mus in [50, 300] /cm, g 0.85, n 1.4, pencil beam,
    Rd(r) 128 x 0.005 cm), 1e7 photons: a plain forward against forward +
    adjoint for a loss on Rd(r), and for a loss on Rd(r) plus the absorbed
    weight per voxel."""
    import numpy as np
    import torch

    import nmc_cases as cases
    from nmc_gb300 import abi, build, engine

    build.build()
    torch.cuda.set_device(0)
    rp, tp, v, ext, mua, mus, g, bins, dr = cases.adjoint_case()
    n = args.photons if args.photons != PHOTONS_PER_STEP else 10_000_000
    e = engine.Engine(abi.SIM_MCXYZ, 0, ext)
    e.prepare_data(rp, tp, v)
    e.set_radial_tally(bins, dr)
    e.set_voxel_props(mua, mus, g)
    G = np.random.default_rng(3).uniform(0.5, 1.5, bins + 1).astype(np.float32)
    GF = np.ones(rp.Nx * rp.Ny * rp.Nz, np.float32)

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t0

    fwd = lambda: (e.reset(), e.run(0, n))
    adj = lambda: (e.reset(), e.adjoint_forward(0, n, 8 * n), e.adjoint_backward(G))
    adj_f = lambda: (e.reset(), e.adjoint_forward(0, n, 8 * n, 600 * n), e.adjoint_backward(G, GF))
    for f in (fwd, adj, adj_f):
        for _ in range(max(args.warmup, 1)):
            f()
    K = max(args.steps, 1)
    t_fwd = min(timed(fwd) for _ in range(K))
    t_adj = min(timed(adj) for _ in range(K))
    t_adj_f = min(timed(adj_f) for _ in range(K))
    sm = e.summary()
    rd = e.tally(abi.TALLY_RD_R).sum() / n
    e.close()
    return {
        "metric": "photons/s, forward + pMC adjoint vs plain forward, 64^3 per-voxel medium",
        "unit": "photons/s", "value": n / t_adj, "plain_value": n / t_fwd,
        "cost_ratio_rd": t_adj / t_fwd, "cost_ratio_rd_fluence": t_adj_f / t_fwd,
        "forward_s": t_fwd, "adjoint_rd_s": t_adj, "adjoint_rd_fluence_s": t_adj_f, "photons": n,
        "rd": rd, "substeps_per_photon": sm["substeps"] / max(sm["photons"], 1), "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": "64^3 x 0.01 cm per-voxel medium, mua 0.1-5, mus 50-300 /cm (smoothed seeded "
                               "noise), g 0.85, n 1.4, pencil beam, Rd(r) 128 x 0.005 cm",
                   "timing": f"best of {K} after {max(args.warmup, 1)} warm-up, host clock around "
                             "synchronised calls (includes the event list and gradient copies)"},
    }


def run_cbs_workload(args) -> dict:
    """Polarised E-field / CBS / Raman: monodisperse spheres a = 0.5 um, n 1.59
    in water, 633 nm, mus 100 /cm, mua 0.01 /cm, semi-infinite slab; Mie
    tables on 1801 angles; the backscattering cone on 256 x 256 angles within
    +-5 mrad; Raman conversion at 1e-4 /cm to 700 nm; 1e8 photons over 8
    polarisation / incidence settings in one launch."""
    import torch

    import nmc_cases as cases
    from nmc_gb300 import build, efield

    build.build()
    torch.cuda.set_device(0)
    total = args.photons if args.photons != PHOTONS_PER_STEP else 100_000_000
    cfg, S633, S700, settings = cases.cbs_case(n_settings=8, photons=total // 8)
    warm = cases.cbs_case(n_settings=8, photons=20_000)[3]
    efield.run(cfg, S633, warm, S_raman=S700)
    best, r = None, None
    for _ in range(max(args.steps, 1)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = efield.run(cfg, S633, settings, S_raman=S700)
        torch.cuda.synchronize()
        t = time.perf_counter() - t0
        best = t if best is None else min(best, t)
    n = float(r["photons"].sum())
    out = {
        "metric": "photons/s, polarised E-field transport with CBS cone and Raman, 8 settings",
        "unit": "photons/s", "value": n / best, "seconds": best, "photons": n,
        "scatterings_per_photon": float(r["scatters"].sum() / n),
        "rd": float(r["Rd"].sum() / n),
        "co_enhancement": float(1 + r["interf_co"].sum() / r["multi_co"].sum()),
        "cross_enhancement": float(1 + r["interf_cross"].sum() / r["multi_cross"].sum()),
        "co_fraction": float(r["co"].sum() / (r["co"].sum() + r["cross"].sum())),
        "raman_conversions": float(r["raman_n"].sum()), "raman_rd": float(r["raman_Rd"].sum() / n),
        "dtype": "f32", "data": "synthetic",
        "config": {"workload": "spheres 0.5 um 1.59/1.33, 633 nm, mus 100, mua 0.01 /cm, semi-infinite; cone "
                               "256^2 within +-5 mrad; Raman 1e-4 /cm to 700 nm; 8 settings (pol 0/45/90/135 deg "
                               "x incidence 0/10 deg)",
                   "timing": f"best of {max(args.steps, 1)} host-timed calls (tables, launch, cone transform, "
                             "result copies)"},
    }
    if not args.no_cpu:
        from oracle import bindings as orc

        threads = os.cpu_count() or 1
        per = 4_000
        sample = cases.cbs_case(n_settings=8, photons=per)[3]
        t0 = time.perf_counter()
        orc.efield(cfg, S633, sample, S_raman=S700, cone=True, real_bits=32, nthreads=threads)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": 8 * per / dt, "unit": "photons/s", "cores": threads, "kind": "port",
                               "sample": f"{8 * per} photons of the same 8 settings, FP32 CPU restatement of the "
                                         f"E-field model (sums only), {dt:.1f} s"}
    return out


def run_layered_workload(args) -> dict:
    """Layered media: a three-layer skin stack (epidermis 0.01 cm, dermis
    0.2 cm, semi-infinite subcutis; mua 3 / 0.3 / 0.1, mus 200 / 150 / 100
    /cm, g 0.8 / 0.85 / 0.9, n 1.4 / 1.4 / 1.44), normal pencil beam, Rd(r),
    Tt(r), A(z) and per-layer absorption, 1e8 photons per call; the CPU
    restatement of the same model times a bounded sample on the host cores."""
    import torch

    import nmc_cases as cases
    from nmc_gb300 import build, layered

    build.build()
    torch.cuda.set_device(0)
    n = args.photons if args.photons != PHOTONS_PER_STEP else 100_000_000
    kw = dict(nr=100, dr=0.01, nz=100, dz=0.01, seed=11)
    for _ in range(max(args.warmup, 1)):
        layered.run(cases.LAYERED_SKIN3, 1_000_000, **kw)
    best, r = None, None
    for _ in range(max(args.steps, 1)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = layered.run(cases.LAYERED_SKIN3, n, **kw)
        t = time.perf_counter() - t0
        best = t if best is None else min(best, t)
    out = {
        "metric": "photons/s, layered mcsub (3-layer skin stack)", "unit": "photons/s", "value": n / best,
        "seconds": best, "photons": n, "rd": r["rd"], "rd_se": r["rd_se"],
        "interactions_per_photon": r["interactions"] / n, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "3 layers: 0.01 cm (mua 3, mus 200, g 0.8, n 1.4), 0.2 cm (0.3, 150, 0.85, 1.4), "
                               "semi-infinite (0.1, 100, 0.9, 1.44); pencil beam; Rd(r), Tt(r) 100 x 0.01 cm, "
                               "A(z) 100 x 0.01 cm",
                   "timing": f"best of {max(args.steps, 1)} host-timed calls (allocation, launch, tally copies)"},
    }
    if not args.no_cpu:
        from oracle import bindings as orc

        threads = os.cpu_count() or 1
        sample = 200_000
        t0 = time.perf_counter()
        orc.layered(cases.LAYERED_SKIN3, sample, real_bits=32, nthreads=threads, **kw)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": sample / dt, "unit": "photons/s", "cores": threads, "kind": "port",
                               "sample": f"{sample} photons of the same stack, FP32 CPU restatement, {dt:.1f} s"}
    return out


def run_notebook_workload(args) -> dict:
    """The reference's published throughput workloads, run as the notebooks
    run them: `nmc <name>` on the files the notebook writes, with the
    reference's own random streams.
      notebook0: example0 (homogeneous 200^3 cube at 0.02, uniform beam of
        radius 1.2, mua 1, mus 100, g 0.9, n 1.4/1.001), 1e5 photons;
        recorded 7.09 s of GPU time (14,096 photons/s).
      notebook2: example2 (skin vessel, 200^3 at 0.0005 cm, 532 nm tissue
        table), 1e6 photons; recorded 209.0 s (4,783 photons/s).
    Both on an AMD Radeon Pro 5500 XT under Metal.  `value` is the same
    "Total execution time (GPU)" measure here; `wall_s` the whole process
    (start-up, file reading and writing included)."""
    import tempfile

    import numpy as np

    import nmc_cases as cases
    from nmc_gb300 import build, mci

    build.build()
    if args.workload == "notebook0":
        n, base, what = 100_000, 14096.0, "example0: 200^3 x 0.02 homogeneous cube, uniform beam r 1.2, mua 1, " \
            "mus 100, g 0.9, n 1.4/1.001, 1e5 photons"
        note = "14,096 photons/s: 1e5 photons in 7.09 s on an AMD Radeon Pro 5500 XT (example0.ipynb)"
    else:
        n, base, what = 1_000_000, 4783.0, "example2: skin vessel 200^3 x 0.0005 cm, 532 nm tissues, 1e6 photons"
        note = "4,783 photons/s: 1e6 photons in 209.0 s on an AMD Radeon Pro 5500 XT (example2.ipynb)"
    walls, kern = [], []
    with tempfile.TemporaryDirectory() as d:
        name = os.path.join(d, "test")
        if args.workload == "notebook0":
            cases.write_example0_mci(name + "_H.mci")
            mci.write_tissue(name, np.ones(200 ** 3, np.uint8))
        else:
            spec = json.load(open(os.path.join(ROOT, "tests", "golden", "spectral_tissues.json")))
            t532 = next(c for c in spec if c["nm"] == 532)["tissues"]
            cases.write_notebook_mci(name + "_H.mci", [(round(t532[str(i)]["mua"], 4), round(t532[str(i)]["mus"], 4),
                                                         round(t532[str(i)]["g"], 4)) for i in range(1, 10)])
            mci.write_tissue(name, cases.notebook_skinvessel_map())
        for i in range(max(args.warmup, 1) + max(args.steps, 1)):
            t0 = time.perf_counter()
            r = mci.run_nmc(name, "--photons", str(n))
            t = time.perf_counter() - t0
            if r.returncode != 0:
                raise RuntimeError(r.stdout[-1000:] + r.stderr[-1000:])
            rep = json.load(open(name + "_report.json"))
            if i >= max(args.warmup, 1):
                walls.append(t)
                kern.append(rep["kernel_ms"] * 1e-3)
        rd = rep["Rd"]
    k = min(kern)
    return {"metric": f"photons/s, {args.workload} through the nmc program (GPU execution time)",
            "unit": "photons/s", "value": n / k, "vs_baseline": (n / k) / base, "kernel_s": k,
            "wall_s": min(walls), "photons": n, "rd": rd, "dtype": "f32", "data": "synthetic",
            "config": {"workload": what + ", reference random streams", "baseline": note,
                       "timing": f"best of {max(args.steps, 1)} runs of the nmc program"}}


def run_mcsub_workload(args) -> dict:
    """C1 alone: the semi-infinite mcsub medium, ten 1e6-photon transport
    launches device-timed (the measurement the default line carries as its
    `mcsub_c1` extra), with the FP32 CPU restatement unless --no-cpu."""
    import torch

    from nmc_gb300 import build, engine

    build.build()
    torch.cuda.set_device(0)
    ffma, _ = engine.probe_issue_peaks(0)
    out = mcsub_extra(ffma, cpu=not args.no_cpu)
    workload = out.pop("workload")
    return {"metric": "photons/s, mcsub semi-infinite medium", **out, "dtype": "f32", "data": "synthetic",
            "config": {"workload": workload}}


def run_speckle_workload(args) -> dict:
    """CBS speckle mutual-interference post-processing (MetalMC.m:628-742):
    a 256 x 256 exit map with 64 speckle records per pixel (seeded synthetic
    maps and records of the E-field kernel's layout), on the GPU through
    nmc_speckle_mutual (host arrays in and out), against the oracle's
    single-threaded restatement of the reference's loop on the host."""
    import math

    import numpy as np

    from nmc_gb300 import abi, build, efield

    build.build()
    rng = np.random.default_rng(17)
    nx = ny = 256
    kmax = 64
    maps = np.zeros((len(abi.EF_MAPS), nx, ny), np.float32)
    det = rng.integers(1, 200, (nx, ny)).astype(np.float32)
    maps[abi.EF_MAPS.index("Det")] = det
    for k in ("XX", "XY", "YX", "YY", "Rd"):
        maps[abi.EF_MAPS.index(k)] = rng.uniform(0, 1, (nx, ny)) * det
    for k in ("Phase0", "Phase1", "Phase2", "Phase3"):
        maps[abi.EF_MAPS.index(k)] = rng.uniform(-math.pi, math.pi, (nx, ny)) * det
    rec = np.zeros((kmax, nx, ny), abi.SPECKLE_DTYPE)
    for f in ("Phase", "Path", "Scatt", "Total"):
        rec[f] = rng.uniform(-math.pi, math.pi, rec.shape)
    for f in ("XX", "XY", "Ryx"):
        rec[f] = rng.uniform(0, 0.2, rec.shape)
    counts = np.full((nx, ny), kmax, np.int32)
    lam, lc = 633e-6, 0.05
    for _ in range(max(args.warmup, 1)):
        efield.speckle_mutual(maps, rec, counts, lam, lc)
    best = None
    for _ in range(max(args.steps, 1)):
        t0 = time.perf_counter()
        out = efield.speckle_mutual(maps, rec, counts, lam, lc)
        t = time.perf_counter() - t0
        best = t if best is None else min(best, t)
    n_rec = nx * ny * kmax
    res = {"metric": "speckle records/s, CBS mutual-interference post-processing", "unit": "records/s",
           "value": n_rec / best, "seconds": best, "records": n_rec, "dtype": "f32", "data": "synthetic",
           "config": {"workload": f"{nx} x {ny} exit map, {kmax} speckle records per pixel, lambda 633 nm, "
                                  f"coherence length {lc}",
                      "timing": f"best of {max(args.steps, 1)} host-timed calls (copies in and out included)"}}
    if not args.no_cpu:
        from oracle import bindings as orc

        t0 = time.perf_counter()
        want = orc.speckle_mutual(maps, rec, counts, lam, lc, np.zeros((len(abi.EF_MAPS), nx * ny), np.float32))
        dt = time.perf_counter() - t0
        res["max_abs_diff_vs_oracle"] = float(np.abs(out.reshape(want.shape) - want).max())
        res["cpu_baseline"] = {"value": n_rec / dt, "unit": "records/s", "cores": 1, "kind": "port",
                               "sample": f"the whole workload, the oracle's restatement, 1 thread, {dt:.2f} s"}
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--photons", type=int, default=PHOTONS_PER_STEP)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the extras of the default line (sweep to 1%% SE, adjoint, C1, layered, C5)")
    ap.add_argument("--budget-scale", type=float, default=1.0,
                    help="sweep workload: scale every wavelength's photon budget (profiling on a smaller case)")
    ap.add_argument("--tune", type=int, default=2_000_000,
                    help="autotune the launch shape on this many photons before the warm-up (0: defaults)")
    ap.add_argument("--profile-only", action="store_true",
                    help="run only the warm-up and timed transport launches (for ncu)")
    ap.add_argument("--workload", default="skinvessel", choices=["skinvessel", "sweep", "sweep_mcsub", "adjoint", "cbs", "layered", "speckle",
                             "mcsub", "notebook0", "notebook2"])
    args = ap.parse_args()
    if args.workload == "sweep":
        out = run_sweep_workload(args)
    elif args.workload == "sweep_mcsub":
        out = run_sweep_mcsub_workload(args)
    elif args.workload == "adjoint":
        out = run_adjoint_workload(args)
    elif args.workload == "cbs":
        out = run_cbs_workload(args)
    elif args.workload == "layered":
        out = run_layered_workload(args)
    elif args.workload == "speckle":
        out = run_speckle_workload(args)
    elif args.workload == "mcsub":
        out = run_mcsub_workload(args)
    elif args.workload in ("notebook0", "notebook2"):
        out = run_notebook_workload(args)
    else:
        out = run_reference(args) if args.impl == "reference" else run_ours(args)
    if out:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
