#!/usr/bin/env python
"""Benchmark of the GB300 MGBF filtering path.

Workload (one "step" = forward + adjoint of the whole batch): batched
ensemble localization, 80 members x 4 variables on a 512x512 filter grid --
three 3D variables with 64, 64 and 48 levels and one 2D variable -- with 5
generations, p = 2, horizontal reaches {8, 10, 12, 16}, vertical reach 4,
FP32 storage and arithmetic.  Inputs are seeded N(0,1) fields generated on
the device (torch.Generator, seed 1000 + rank); one field set is 14.8 GB, far
larger than L2, so no flush is needed between steps.

Prints one JSON line (rank 0).  `--impl reference` times the CPU restatement
of the reference's filtering_procedure (the oracle; the Fortran reference
cannot be built on these machines) on the host cores instead.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = ("grid-pt applications/s fwd+adj (fraction of HBM roofline), "
          "batched FP32 vs plain FP64, rel-L2")
UNIT = "grid-pt applications/s"

IM = JM = 512
GM = 5
HZ = 4
P = 2
# variable groups: (levels, horizontal reach)
VARS = [(64, 8), (64, 10), (48, 12), (1, 16)]
# generation weights normalised so that L maps a constant field to itself
WEIGHTS = [4.0 ** (-g) / GM for g in range(GM)]
WORKLOAD = ("batched ensemble localization: 80 members x {64,64,48,1} levels (3D,3D,3D,2D), "
            "512x512, 5 generations, p=2, h={8,10,12,16}, hz=4, FP32, forward+adjoint")


def ampl02(h: int) -> float:
    """mg_ampl02 whose radial support has reach h (disk radius h+1/2)."""
    return (h + 0.5) ** 2 / (2 * P + 4)


def ampl01(hz: int) -> float:
    return (hz + 0.5) ** 2 / (2 * P + 3)


def groups(members: int):
    from standalone_mgbf_loc_gb300 import GroupDesc
    out = []
    for lm, h in VARS:
        out.append(GroupDesc(nk=members * lm, lm=lm, nzcol=members if lm > 1 else 0, hx=h, hy=h, hz=HZ, p=P,
                             mg_ampl01=ampl01(HZ), mg_ampl02=ampl02(h)))
    return out


# ----------------------------------------------------------------- helpers

def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi samples (200 ms) of SM clock and throttle reasons."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        # the raw samples go to MGBF_CLOCK_LOG_DIR (default: the temp dir);
        # their summary is the JSON line's "clocks" entry
        log_dir = os.environ.get("MGBF_CLOCK_LOG_DIR") or tempfile.gettempdir()
        self.path = os.path.join(log_dir, f"mgbf_clocks_rank{gpu}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names[1:], parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "samples": len(sm),
                "reasons": sorted(reasons)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ------------------------------------------------------------ CPU (oracle)

def oracle_member_cfg(group_index: int, nthreads: int):
    from oracle import oracle as O
    lm, h = VARS[group_index]
    return O.OracleConfig(I=IM, J=JM, nk=lm, hx=h, hy=h, hz=HZ, p=P, ampl01=ampl01(HZ), ampl02=ampl02(h), gm=GM,
                          weights=WEIGHTS, proc=6, lm=lm, nzcol=1 if lm > 1 else 0,
                          l_vertical_filter=lm > 1, nthreads=nthreads)


def cpu_step(x: np.ndarray, nthreads: int):
    """One sample step on the host: forward + adjoint of one member of the
    first variable (64 levels, reach 8) on the full 512x512 grid."""
    from oracle import oracle as O
    c = oracle_member_cfg(0, nthreads)
    y = O.filter_compact(c, x)
    z = O.filter_compact(c, y)  # the adjoint chain equals the forward chain
    return y, z


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    nthreads = os.cpu_count() or 1
    x = np.random.default_rng(1000).standard_normal((JM, IM, VARS[0][0]))
    pts = float(IM * JM * VARS[0][0])
    for _ in range(args.warmup):
        cpu_step(x, nthreads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cpu_step(x, nthreads)
    dt = (time.perf_counter() - t0) / args.steps
    value = 2 * pts / dt
    sample = "one member of the 64-level variable (512x512x64, reach 8, 5 generations), forward+adjoint per step"
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic: seeded N(0,1) (numpy seed 1000)",
        "config": {"workload": WORKLOAD, "sample": sample},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU restatement of the reference's filtering_procedure (FP64, OpenMP); the Fortran+MPI "
                "reference has no compiler on these machines",
    }
    print(json.dumps(out), flush=True)
    return 0


# ------------------------------------------------------------------ GPU arm

def run_gpu(args):
    import torch
    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    from __graft_entry__ import build
    build()
    from standalone_mgbf_loc_gb300 import MGBFBatch, _abi
    members = args.members
    gdesc = groups(members)
    batch = MGBFBatch(IM, JM, GM, WEIGHTS, gdesc)
    tuned = None
    if not args.no_autotune:
        batch.autotune(torch.float32)  # radial-kernel variant and tile height per generation and pass
        variant_names = {-1: "default", 0: "tma2", 1: "tma1", 2: "cp.async", 3: "tma2seq"}
        tuned = {f"lm{lm}_h{h}": [[f"{variant_names.get(v, v)}/{r}" for v, r in gen_pair] for gen_pair in per_group]
                 for (lm, h), per_group in zip(VARS, batch.tuning(torch.float32))}
    batch.use_graphs(True)  # each repeated fwd / adj call replays one captured CUDA graph
    gen = torch.Generator(device=dev)
    gen.manual_seed(1000 + rank)
    fields = [torch.randn((JM, IM, g.nk), generator=gen, device=dev, dtype=torch.float32) for g in gdesc]
    pts_op = float(sum(IM * JM * g.nk for g in gdesc))

    def step():
        batch.apply(fields, adjoint=False)
        batch.apply(fields, adjoint=True)

    # radial sides per generation or as one persistent launch per group: a
    # short timing of each (after a capturing call), the faster one is kept
    # for the timed region and the correctness sample
    def trial_ms(n=2):
        step()  # captures the graph of this launch sequence
        torch.cuda.synchronize()
        a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a0.record()
        for _ in range(n):
            step()
        a1.record()
        torch.cuda.synchronize()
        return a0.elapsed_time(a1) / n

    trials = {}
    for blocks_per_sm in (0, 1, 2, 8):  # 0: per generation; else persistent with up to that many blocks per SM
        batch.use_persistent(blocks_per_sm)
        trials[blocks_per_sm] = trial_ms()
    # per generation with the single-row TMA kernel everywhere (the rows per
    # block the autotuner chose), against the autotuner's variants: its
    # kernels are timed alone, the step runs the groups side by side
    batch.use_persistent(0)
    tuned_choice = batch.tuning(torch.float32)
    for q, per_group in enumerate(tuned_choice):
        for g, pair in enumerate(per_group):
            for p, (v, r) in enumerate(pair):
                if v >= 0:
                    batch.set_tuning(q, g, p, 1, r)
    trials["tma1"] = trial_ms()
    best = min(trials, key=trials.get)
    if best != "tma1":
        for q, per_group in enumerate(tuned_choice):  # back to the autotuner's variants
            for g, pair in enumerate(per_group):
                for p, (v, r) in enumerate(pair):
                    if v >= 0:
                        batch.set_tuning(q, g, p, v, r)
        batch.use_persistent(best)
    names = {0: "per generation", "tma1": "per generation, single-row TMA kernel everywhere"}
    radial_launch = {"ms_per_step": {names.get(k, f"persistent, <= {k} blocks/SM"): v for k, v in trials.items()},
                     "chosen": names.get(best, f"persistent, <= {best} blocks/SM")}
    # graph-node priorities of the concurrent group branches (0 none, 1
    # memory-bound kernels first, 2 radial kernels first) and the vertical
    # filter passes (2 as the reference: Bz^T first, Bz last; 1: M = Bz Bz^T
    # once, in the last prolongation -- the same operator).  They interact
    # (how the groups' stages overlap depends on both), so every pair is
    # timed and the fastest kept.
    prio_names = {0: "none", 1: "memory-bound kernels first", 2: "radial kernels first"}
    grid = {}
    for passes in (2, 1):
        batch.set_vertical_passes(passes)
        for mode in (0, 1, 2):
            batch.set_priorities(mode)
            grid[(mode, passes)] = trial_ms(3)
    best_mode, best_vp = min(grid, key=grid.get)
    batch.set_priorities(best_mode)
    batch.set_vertical_passes(best_vp)
    graph_priorities = {"ms_per_step": {prio_names[m]: grid[(m, best_vp)] for m in (0, 1, 2)},
                        "chosen": prio_names[best_mode]}
    vertical_passes = {"ms_per_step": {str(v): grid[(best_mode, v)] for v in (2, 1)}, "chosen": best_vp}
    # fresh N(0,1) inputs: the trial steps above filtered the fields in place
    for f in fields:
        f.normal_(generator=gen)

    # correctness sample (checked against the oracle after the timed legs):
    # member 0 of every variable group through one forward and, from the same
    # input, one adjoint call
    sample = {}
    if rank == 0:
        lms = [lm for lm, _ in VARS]
        x0 = [f[:, :, :lm].clone() for f, lm in zip(fields, lms)]
        batch.apply(fields, adjoint=False)
        torch.cuda.synchronize()
        y_fwd = [f[:, :, :lm].double().cpu().numpy() for f, lm in zip(fields, lms)]
        for f, x, lm in zip(fields, x0, lms):
            f[:, :, :lm].copy_(x)
        batch.apply(fields, adjoint=True)
        torch.cuda.synchronize()
        y_adj = [f[:, :, :lm].double().cpu().numpy() for f, lm in zip(fields, lms)]
        sample = {"x": [x.double().cpu().numpy() for x in x0], "fwd": y_fwd, "adj": y_adj}
        del x0
    batch.status()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    def barrier():
        if dist is not None:
            dist.barrier()

    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        barrier()
        torch.cuda.synchronize()
        e0.record(stream)
        torch.cuda.nvtx.range_push("timed_steps")  # lets a profiler keep only the timed launches
        for _ in range(args.steps):
            step()
        torch.cuda.nvtx.range_pop()
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
    from standalone_mgbf_loc_gb300.sharding import max_over_ranks
    ms = max_over_ranks(e0.elapsed_time(e1), dev)
    ms_step = ms / args.steps
    value = ws * 2 * pts_op / (ms_step * 1e-3)

    # stage timers: dominant-kernel launch durations (separate, untimed pass)
    _abi.timers_enable(True)
    nstep_t = 2
    for _ in range(nstep_t):
        step()
    torch.cuda.synchronize()
    stats = _abi.timers_read()
    _abi.timers_enable(False)
    launches_per_step = sum(v[0] for v in stats.values()) / nstep_t
    hb = [stats[k] for k in ("hfiltT", "hfilt") if k in stats]
    h_launch = sum(v[0] for v in hb)
    h_ms = sum(v[1] for v in hb)
    h_pts = sum(v[2] for v in hb)
    peak, peak_kind = measured_peaks()
    s = 4  # bytes per FP32 element
    achieved = (2 * s * h_pts) / (h_ms * 1e-3) / 1e9 if h_ms > 0 else None
    stage_ms = {k: round(v[1] / nstep_t, 3) for k, v in stats.items()}
    # FP32-pipe roofline of the radial kernel: the moment form costs 8R+3
    # scalar FP operations (adds or multiply-adds) per grid point and pass
    gen_pts = sum((IM >> g) * (JM >> g) for g in range(GM))
    fp_ops = sum(g.nk * gen_pts * (8 * g.hx + 3) for g in gdesc) * 2 * 2 * nstep_t  # 2 passes, fwd+adj
    n_sm = torch.cuda.get_device_properties(dev).multi_processor_count
    clk_sum = clk.summary()
    sm_hz = (clk_sum.get("sm_mhz") or 2070.0) * 1e6
    fp_peak = n_sm * 128 * sm_hz  # SMs x FP32 lanes x measured SM clock (one op per lane per cycle)
    traffic = (HMOM_DRAM_BYTES_PER_POINT * h_pts / h_launch) if h_launch else None

    # end to end through the host-streaming pipeline: every step copies the
    # whole field set from pinned host memory, filters it forward and adjoint,
    # and copies the result back; three device sets and three streams let the
    # copies of neighbouring steps overlap the filtering
    from standalone_mgbf_loc_gb300.pipeline import HostStream
    host = [f.to("cpu").pin_memory() for f in fields]
    outs = [torch.empty(h.shape, dtype=h.dtype).pin_memory() for h in host]
    del fields
    torch.cuda.empty_cache()
    hs = HostStream(batch, torch.float32, dev, ops=("fwd", "adj"), nsets=3)
    h2d = hs.bytes_per_step()
    e2e_steps = max(2, args.steps)
    for _ in range(hs.nsets):  # every device set once (graph capture per set)
        hs.submit(host, outs)
    hs.finish()
    torch.cuda.synchronize()
    barrier()
    e2, e3 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2.record(hs.s_h2d)
    for _ in range(e2e_steps):
        hs.submit(host, outs)
    e3.record(hs.s_d2h)
    hs.finish()
    torch.cuda.synchronize()
    ms_e2e = max_over_ranks(e2.elapsed_time(e3), dev)
    e2e_value = ws * 2 * pts_op / (ms_e2e / e2e_steps * 1e-3)
    # copy bandwidth of one whole field set, each direction alone
    c0, c1, c2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
    with torch.cuda.stream(hs.s_h2d):
        c0.record(hs.s_h2d)
        for d, h in zip(hs.sets[0], host):
            d.copy_(h, non_blocking=True)
        c1.record(hs.s_h2d)
        for d, h in zip(hs.sets[0], outs):
            h.copy_(d, non_blocking=True)
        c2.record(hs.s_h2d)
    torch.cuda.synchronize()
    copy_gbs = {"h2d": h2d / (c0.elapsed_time(c1) * 1e-3) / 1e9, "d2h": h2d / (c1.elapsed_time(c2) * 1e-3) / 1e9}
    del host, outs, hs
    batch.close()
    torch.cuda.empty_cache()

    # secondary legs (timed on the GPU; their outputs are kept for the
    # oracle checks below, which run after every timed region)
    extras, checks = {}, {}
    if rank == 0 and not args.no_extras:
        extras["cfg1"], checks["cfg1"] = cfg1_leg(torch, dev)
        extras["fp64_plain"], checks["cfg2_f64"] = plain_forward(torch, dev, torch.float64, keep=True)
        extras["fp32_plain"], checks["cfg2_f32"] = plain_forward(torch, dev, torch.float32, keep=True)
        extras["cfg3_grads_fp32"], checks["cfg3"] = cfg3_leg(torch, dev)
        extras["cfg5_bf16"], checks["cfg5"] = cfg5_leg(torch, dev, peak, args.cfg5_steps)
        extras["fast_fp32"] = fast_forward(torch, dev, torch.float32, peak)
        extras["transfers_fp32"] = transfers(torch, dev, torch.float32, peak)
        extras["rad3_fp32"] = rad3_forward(torch, dev, torch.float32)
        extras["lin2_fp32"] = lin2_forward(torch, dev, torch.float32)
        extras["lin3_fp32"] = lin3_forward(torch, dev, torch.float32)

    result = None
    if rank == 0:
        cpu = None
        parity = None
        if not args.no_extras:
            nthreads = os.cpu_count() or 1
            t0 = time.perf_counter()
            cpu_step(sample["x"][0], nthreads)
            dt = time.perf_counter() - t0
            cpu = {"value": 2 * IM * JM * VARS[0][0] / dt, "unit": UNIT, "cores": nthreads, "kind": "port",
                   "sample": "one member of the 64-level variable (512x512x64, reach 8), forward+adjoint, "
                             "FP64 CPU restatement with OpenMP"}
            checks["cfg4"] = sample
            parity = check_parity(checks, nthreads)
            extras["cfg5_bf16"]["per_generation_rel_l2"] = parity["cfg5"]["per_generation_rel_l2"]
        result = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded N(0,1) fields generated on the device (torch.Generator seed 1000+rank)",
            "config": {"workload": WORKLOAD, "members_per_gpu": members, "grid": [IM, JM], "generations": GM,
                       "points_per_op_per_gpu": pts_op, "l2": "no flush: one field set (14.8 GB) >> L2 (129 MB)",
                       "parallelism": f"replicas x{ws} (independent members per GPU, no collective)"},
            "roofline": {"bound": "fp32_pipe", "kernel": "k_hmom_tma / k_hmom_tma1 (radial beta, moment form)",
                         "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                         "traffic_source": HMOM_TRAFFIC_SOURCE,
                         "peak_source": peak_kind,
                         "algorithmic_bytes": "2 x 4 B per grid point per launch (read + write, FP32)",
                         "launches": h_launch / nstep_t, "avg_launch_ms": h_ms / h_launch if h_launch else None,
                         "note": "HBM fraction of a kernel limited by the FP32 pipe (see compute_roofline)"},
            "compute_roofline": {"bound": "fp32_pipe", "kernel": "k_hmom_tma / k_hmom_tma1",
                                 "achieved": fp_ops / (h_ms * 1e-3) if h_ms else None, "peak": fp_peak,
                                 "unit": "FP32 ops/s", "frac": fp_ops / (h_ms * 1e-3) / fp_peak if h_ms else None,
                                 "peak_from": f"{n_sm} SMs x 128 FP32 lanes x {sm_hz / 1e6:.0f} MHz (measured clock)",
                                 "ops_per_point_pass": "8R+3 (moment form; the direct disk sum costs ~pi R^2)"},
            "step_hbm_frac": (4 * 4 * pts_op) / (ms_step * 1e-3) / (peak * 1e9),
            "stages_ms_per_step": stage_ms,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": h2d,
                    "steps": e2e_steps, "ms_per_step": ms_e2e / e2e_steps, "copy_gbs": copy_gbs,
                    "numa_nodes": numa_nodes(),
                    "pipeline": "pinned host -> device, fwd+adj, device -> host per step; uploads, filtering "
                                "and downloads of adjacent steps overlap (three device field sets, three streams)"},
            "gpu_launches": int(round(launches_per_step * args.steps)),
            "radial_launch": radial_launch,
            "graph_priorities": graph_priorities,
            "vertical_passes": vertical_passes,
            "autotune": {"radial_kernel_per_generation": tuned,
                         "key": "variant/output rows per block, [pass after restriction, pass before prolongation]"},
            "clocks": clk_sum,
            "parity": parity,
        }
        result.update(extras)
        print(json.dumps(result), flush=True)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()
    return 0


# DRAM bytes (read + write) per grid point and pass of the radial moment
# kernel, measured by ncu (dram__bytes_read.sum + dram__bytes_write.sum) on
# one k_hmom_tma1 launch of 134.2 M points (8 members of the 64-level,
# reach-8 variable, FP32: 1093.0 MB); traffic grows in proportion to the
# points of a launch.
HMOM_DRAM_BYTES_PER_POINT = 8.15
HMOM_TRAFFIC_SOURCE = ("scaled from an ncu capture of one 8-member launch (8.15 B per point); "
                       "not measured in this run")


def timed_calls(torch, fn, n=5, warm=2):
    """Mean CUDA-event time (ms) of n calls of fn after warm untimed ones."""
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(n):
        fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / n


def plain_cfg(**kw):
    """One 3D field on 768x768x64 (16x16 ranks of 48x48), 5 generations, h=12, hz=4."""
    from standalone_mgbf_loc_gb300 import MGBFConfig
    d = dict(nxPE=16, nyPE=16, im_filt=48, jm_filt=48, lm=64, km3=1, km2=0, n_ens=1, gm_max=5,
             hx=12, hy=12, hz=4, p=2, mg_ampl02=ampl02(12), mg_ampl01=ampl01(4),
             mg_weig1=1.0, mg_weig2=0.5, mg_weig3=0.25, mg_weig4=0.125, mg_weig5=0.0625, layout=1)
    d.update(kw)
    return MGBFConfig(**d)


def plain_forward(torch, dev, dtype, keep=False):
    """Plain unbatched forward of one 3D field, 768x768x64, 5 generations,
    reach 12, vertical reach 4 (filtering_procedure(1)); input seeded N(0,1)
    from numpy (seed 2).  keep: also return (config, input, output) for the
    oracle check."""
    from standalone_mgbf_loc_gb300 import MGBF
    cfg = plain_cfg()
    op = MGBF(cfg)
    x_np = np.random.default_rng(2).standard_normal(op.field_shape())
    x0 = torch.from_numpy(x_np).to(device=dev, dtype=dtype)
    x = x0.clone()
    ms = timed_calls(torch, lambda: op.filtering_procedure(1, x))
    x.copy_(x0)
    op.filtering_procedure(1, x)
    torch.cuda.synchronize()
    op.status()
    out = x.double().cpu().numpy() if keep else None
    pts = float(np.prod(op.field_shape()))
    op.close()
    res = {"workload": "plain forward, one 3D field 768x768x64, 5 generations, h=12, hz=4",
           "dtype": str(dtype).replace("torch.", ""), "ms": ms, "value": pts / (ms * 1e-3), "unit": UNIT}
    if keep:
        return res, {"cfg": cfg, "proc": 1, "x": x_np, "y": out, "dtype": res["dtype"]}
    return res


def cfg1_leg(torch, dev):
    """256x256x32 (8x8 ranks of 32x32), 4 generations, h=6, hz=3, weights
    1, .5, .25, .125; filtering_procedure(1) in FP64 and FP32 on seeded
    N(0,1) noise (numpy seed 0) and on a unit impulse at Fortran (128,128,16)."""
    from standalone_mgbf_loc_gb300 import MGBF, MGBFConfig
    cfg = MGBFConfig(nxPE=8, nyPE=8, im_filt=32, jm_filt=32, lm=32, km3=1, km2=0, n_ens=1, gm_max=4,
                     hx=6, hy=6, hz=3, p=2, mg_ampl02=ampl02(6), mg_ampl01=ampl01(3),
                     mg_weig1=1.0, mg_weig2=0.5, mg_weig3=0.25, mg_weig4=0.125, layout=1)
    op = MGBF(cfg)
    noise = np.random.default_rng(0).standard_normal(op.field_shape())
    imp = np.zeros(op.field_shape())
    imp[127, 127, 15] = 1.0
    pts = float(np.prod(op.field_shape()))
    res = {"workload": "plain forward, 256x256x32, 4 generations, h=6, hz=3, weights 1,.5,.25,.125"}
    outs = {}
    for dtype in (torch.float64, torch.float32):
        name = str(dtype).replace("torch.", "")
        xn = torch.from_numpy(noise).to(device=dev, dtype=dtype)
        x = xn.clone()
        ms = timed_calls(torch, lambda: op.filtering_procedure(1, x), n=10)
        res[name] = {"ms": ms, "value": pts / (ms * 1e-3), "unit": UNIT}
        for tag, inp in (("noise", noise), ("impulse", imp)):
            t = torch.from_numpy(inp).to(device=dev, dtype=dtype)
            op.filtering_procedure(1, t)
            torch.cuda.synchronize()
            outs[(name, tag)] = t.double().cpu().numpy()
    op.status()
    op.close()
    return res, {"cfg": cfg, "proc": 1, "inputs": {"noise": noise, "impulse": imp}, "outs": outs}


def cfg3_leg(torch, dev):
    """Differentiation: 512x512x64 (16x16 ranks of 32x32), 5 generations,
    h=10, hz=4, FP32.  One step = the torch.autograd.Function's forward plus
    its backward (hand-written adjoint chain; gradients for the field and the
    five generation weights; coarse generations recomputed in the backward).
    Kept for the oracle check: y, dL/dx, dL/da, the dot-product residual of
    forward and adjoint, and central finite differences (step 1e-3) of the
    weights, each from GPU FP32 calls."""
    from standalone_mgbf_loc_gb300 import MGBF
    from standalone_mgbf_loc_gb300.autograd import mgbf_apply
    cfg = plain_cfg(im_filt=32, jm_filt=32, hx=10, hy=10, mg_ampl02=ampl02(10))
    op = MGBF(cfg)
    rng = np.random.default_rng(3)
    x_np = rng.standard_normal(op.field_shape())
    r_np = rng.standard_normal(op.field_shape())
    y2_np = rng.standard_normal(op.field_shape())
    x = torch.from_numpy(x_np).to(device=dev, dtype=torch.float32)
    r = torch.from_numpy(r_np).to(device=dev, dtype=torch.float32)
    w0 = [1.0, 0.5, 0.25, 0.125, 0.0625]

    def step():
        xg = x.clone().requires_grad_(True)
        w = torch.tensor(w0, dtype=torch.float64, device=dev, requires_grad=True)
        loss = (mgbf_apply(op, xg, w, 1) * r).sum()
        loss.backward()
        return xg, w

    ms = timed_calls(torch, step, n=5)
    xg, w = step()
    y = mgbf_apply(op, x, torch.tensor(w0, dtype=torch.float64, device=dev), 1)
    out = {"y": y.double().cpu().numpy(), "gx": xg.grad.double().cpu().numpy(),
           "ga": w.grad.double().cpu().numpy()}
    # dot-product test of the forward and the adjoint call
    op.set_weights(w0)
    ly = torch.from_numpy(y2_np).to(device=dev, dtype=torch.float32)
    op.filtering_procedure_adjoint(1, ly)
    lx = y.double()
    a = float((lx * torch.from_numpy(y2_np).to(dev)).sum())
    b = float((x.double() * ly.double()).sum())
    out["dot_residual"] = abs(a - b) / (float(lx.norm()) * float(np.linalg.norm(y2_np)))
    # central finite differences of <r, L(a) x> in the weights, step 1e-3
    h = 1e-3
    fd = []
    for g in range(5):
        f = []
        for sgn in (1, -1):
            wg = list(w0)
            wg[g] += sgn * h
            op.set_weights(wg)
            t = x.clone()
            op.filtering_procedure(1, t)
            f.append(float((t.double() * r.double()).sum()))
        fd.append((f[0] - f[1]) / (2 * h))
    out["fd"] = np.array(fd)
    torch.cuda.synchronize()
    op.status()
    pts = float(np.prod(op.field_shape()))
    op.close()
    res = {"workload": "autograd forward + backward (field and 5 weight gradients), 512x512x64, 5 generations, "
                       "h=10, hz=4, FP32",
           "dtype": "float32", "ms": ms, "value": 2 * pts / (ms * 1e-3), "unit": UNIT,
           "note": "value counts 2 operator applications per step (forward and adjoint)"}
    return res, {"cfg": cfg, "proc": 1, "x": x_np, "r": r_np, "w": w0, **out}


CFG5 = dict(members=30, n=1536, lm=64, gm=6, h=24, hz=5, weights=[1.0, 0.5, 0.25, 0.125, 0.0625, 0.0625])


def numa_nodes():
    """NUMA nodes the host exposes (pinned buffers land on one of them)."""
    try:
        return sum(1 for d in os.listdir("/sys/devices/system/node") if re.fullmatch(r"node\d+", d))
    except OSError:
        return None


def cfg5_leg(torch, dev, peak_gbs, steps, members=None):
    """Large batched run: 30 members (or `members`, for small profiling
    cases) x one 3D variable on 1536x1536x64,
    6 generations, h=24, hz=5, BF16 storage with FP32 arithmetic, FP64
    coefficient setup; seeded N(0,1) inputs (numpy seed 5 for member 0,
    torch.Generator for the others).  One step = forward + adjoint of the
    batch (the adjoint recomputes every coarse generation; nothing is stored
    between the calls).  Kept for the oracle check: member 0's output with
    every weight and with one generation's weight at a time (the
    per-generation terms of the operator)."""
    from standalone_mgbf_loc_gb300 import MGBFBatch, GroupDesc, _abi
    c = dict(CFG5, members=members or CFG5["members"])
    n, lm, nk = c["n"], c["lm"], c["members"] * c["lm"]
    gd = [GroupDesc(nk=nk, lm=lm, nzcol=c["members"], hx=c["h"], hy=c["h"], hz=c["hz"], p=P,
                    mg_ampl01=ampl01(c["hz"]), mg_ampl02=ampl02(c["h"]))]
    b = MGBFBatch(n, n, c["gm"], c["weights"], gd)
    b.autotune(torch.bfloat16)
    b.use_graphs(True)
    gen = torch.Generator(device=dev)
    gen.manual_seed(55)
    x0 = torch.randn((n, n, nk), generator=gen, device=dev, dtype=torch.float32).to(torch.bfloat16)
    m0 = np.random.default_rng(5).standard_normal((n, n, lm))
    x0[:, :, :lm] = torch.from_numpy(m0).to(device=dev, dtype=torch.bfloat16)
    f = [x0.clone()]

    def step():
        b.apply(f, adjoint=False)
        b.apply(f, adjoint=True)

    for _ in range(3):
        step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(steps):
        step()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    b.status()
    # radial-kernel launch durations from the stage timers
    _abi.timers_enable(True)
    step()
    torch.cuda.synchronize()
    st = _abi.timers_read()
    _abi.timers_enable(False)
    hb = [st[k] for k in ("hfiltT", "hfilt") if k in st]
    h_ms, h_pts, h_n = sum(v[1] for v in hb), sum(v[2] for v in hb), sum(v[0] for v in hb)
    achieved = 2 * 2 * h_pts / (h_ms * 1e-3) / 1e9 if h_ms else None
    gen_pts = sum((n >> g) * (n >> g) for g in range(c["gm"]))
    fp_ops = nk * gen_pts * (8 * c["h"] + 3) * 2 * 2  # 2 passes, forward + adjoint
    # member 0: every weight, then one generation at a time
    outs = []
    for g in range(-1, c["gm"]):
        w = c["weights"] if g < 0 else [c["weights"][q] if q == g else 0.0 for q in range(c["gm"])]
        b.set_weights(w)
        f[0].copy_(x0)
        b.apply(f, adjoint=False)
        torch.cuda.synchronize()
        outs.append(f[0][:, :, :lm].float().cpu().numpy())
    b.status()
    x_m0 = x0[:, :, :lm].double().cpu().numpy()  # the BF16-rounded input the GPU filtered
    pts = float(n * n * nk)
    b.close()
    del f, x0
    torch.cuda.empty_cache()
    res = {"workload": f"{c['members']} members x 1536x1536x64, 6 generations, h=24, hz=5, BF16 storage, "
                       "FP32 arithmetic, forward + adjoint",
           "dtype": "bf16", "ms": ms, "value": 2 * pts / (ms * 1e-3), "unit": UNIT, "steps": steps,
           "field_gb": pts * 2 / 1e9, "stages_ms_per_step": {k: v[1] for k, v in st.items()},
           "roofline": {"bound": "fp32_pipe", "kernel": "k_hmom_tma / k_hmom_tma1 (reach 24, BF16)",
                        "achieved": achieved, "peak": peak_gbs, "unit": "GB/s",
                        "frac": achieved / peak_gbs if achieved else None,
                        "algorithmic_bytes": "2 x 2 B per grid point per launch (BF16)",
                        "launches": h_n, "avg_launch_ms": h_ms / h_n if h_n else None,
                        "fp32_ops_per_s": fp_ops / (h_ms * 1e-3) if h_ms else None}}
    return res, {"x": x_m0, "outs": outs}


def check_parity(checks, nthreads):
    """Relative L2 errors of the kept GPU outputs against the FP64 oracle
    (the oracle is only the checker here; nothing of it is timed above)."""
    from oracle import oracle as O
    t_start = time.perf_counter()

    def rel(a, b):
        d = float(np.linalg.norm(b))
        return float(np.linalg.norm(np.asarray(a, dtype=np.float64) - b) / (d if d > 0 else 1.0))

    def ocfg(c, proc, **kw):
        gm = c.gm_max
        w = [c.mg_weig1, c.mg_weig2, c.mg_weig3, c.mg_weig4, c.mg_weig5][:gm]
        d = dict(I=c.nxPE * c.im_filt, J=c.nyPE * c.jm_filt, nk=c.lm * c.km3 + c.km2, hx=c.hx, hy=c.hy, hz=c.hz,
                 p=c.p, ampl01=c.mg_ampl01, ampl02=c.mg_ampl02, gm=gm, weights=w, proc=proc, lm=c.lm,
                 nzcol=c.km3, l_vertical_filter=True, nthreads=nthreads)
        d.update(kw)
        return O.OracleConfig(**d)

    out = {"tolerance": {"f64": 1e-12, "f32": 1e-5, "bf16": "reported (2^-8 storage rounding)",
                         "dot_residual_f32": 1e-6, "fd_vs_oracle_grad": 1e-3}}
    c1 = checks["cfg1"]
    oc = ocfg(c1["cfg"], 1)
    refs = {tag: O.filter_compact(oc, x) for tag, x in c1["inputs"].items()}
    out["cfg1"] = {f"{dt}_{tag}": rel(y, refs[tag]) for (dt, tag), y in c1["outs"].items()}
    c2 = checks["cfg2_f64"]
    ref2 = O.filter_compact(ocfg(c2["cfg"], 1), c2["x"])
    out["cfg2"] = {"float64_fwd": rel(c2["y"], ref2), "float32_fwd": rel(checks["cfg2_f32"]["y"], ref2)}
    c3 = checks["cfg3"]
    oc3 = ocfg(c3["cfg"], 1)
    ga = O.weight_grads(oc3, c3["x"], c3["r"])
    out["cfg3"] = {"float32_fwd": rel(c3["y"], O.filter_compact(oc3, c3["x"])),
                   "float32_grad_x": rel(c3["gx"], O.filter_compact(oc3, c3["r"])),
                   "float32_grad_weights": rel(c3["ga"], ga),
                   "float32_fd_weights_vs_oracle": rel(c3["fd"], ga),
                   "float32_dot_residual": c3["dot_residual"]}
    c4 = checks["cfg4"]
    out["cfg4"] = {}
    for q, (lm, h) in enumerate(VARS):
        oc4 = O.OracleConfig(I=IM, J=JM, nk=lm, hx=h, hy=h, hz=HZ, p=P, ampl01=ampl01(HZ), ampl02=ampl02(h), gm=GM,
                             weights=WEIGHTS, proc=6, lm=lm, nzcol=1 if lm > 1 else 0, l_vertical_filter=lm > 1,
                             nthreads=nthreads)
        ref = O.filter_compact(oc4, c4["x"][q])  # L is self-adjoint: the adjoint's reference too
        out["cfg4"][f"group{q}_lm{lm}_h{h}"] = {"float32_fwd": rel(c4["fwd"][q], ref),
                                              "float32_adj": rel(c4["adj"][q], ref)}
    c5 = checks["cfg5"]
    k = CFG5
    oc5 = O.OracleConfig(I=k["n"], J=k["n"], nk=k["lm"], hx=k["h"], hy=k["h"], hz=k["hz"], p=P,
                         ampl01=ampl01(k["hz"]), ampl02=ampl02(k["h"]), gm=k["gm"], weights=k["weights"], proc=6,
                         lm=k["lm"], nzcol=1, l_vertical_filter=True, nthreads=nthreads)
    ys = O.contributions(oc5, c5["x"])
    out["cfg5"] = {"bf16_fwd": rel(c5["outs"][0], sum(ys)),
                   "per_generation_rel_l2": [rel(c5["outs"][1 + g], ys[g]) for g in range(k["gm"])],
                   "sample": "member 0 (1536x1536x64); per generation: the operator with only that generation's "
                             "weight, against the oracle's term of that generation"}
    out["checker_seconds"] = time.perf_counter() - t_start
    return out


def fast_forward(torch, dev, dtype, peak_gbs):
    """The fast 1D+1D filter, filtering_procedure(3), on the plain-forward
    field (768x768x64, 5 generations, hz=4) with line reach 12
    (mg_ampl02 = sqrt(2p+3)/12.5).  Its line passes are HBM-bound: each
    reads and writes the generation once (2 x 4 B per point, FP32)."""
    from standalone_mgbf_loc_gb300 import MGBF, MGBFConfig, _abi
    cfg = MGBFConfig(nxPE=16, nyPE=16, im_filt=48, jm_filt=48, lm=64, km3=1, km2=0, n_ens=1, gm_max=5,
                     hx=12, hy=12, hz=4, p=2, mg_ampl02=np.sqrt(2 * P + 3) / 12.5, mg_ampl01=ampl01(4),
                     mg_weig1=1.0, mg_weig2=0.5, mg_weig3=0.25, mg_weig4=0.125, mg_weig5=0.0625, layout=1)
    op = MGBF(cfg)
    gen = torch.Generator(device=dev)
    gen.manual_seed(8)
    x = torch.randn(op.field_shape(), generator=gen, device=dev, dtype=dtype)
    for _ in range(2):
        op.filtering_procedure(3, x)
    torch.cuda.synchronize()
    n = 5
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(n):
        op.filtering_procedure(3, x)
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / n
    # line-pass bandwidth from the library's stage timers (two passes per
    # hfiltT / hfilt call, each 2 x 4 B per point of its generation)
    _abi.timers_enable(True)
    op.filtering_procedure(3, x)
    torch.cuda.synchronize()
    st = _abi.timers_read()
    _abi.timers_enable(False)
    line_ms = sum(st[k][1] for k in ("hfiltT", "hfilt") if k in st)
    line_pts = sum(st[k][2] for k in ("hfiltT", "hfilt") if k in st)
    gbs = 2 * 2 * 4 * line_pts / (line_ms * 1e-3) / 1e9 if line_ms > 0 else None
    pts = float(np.prod(op.field_shape()))
    op.close()
    return {"workload": "fast 1D+1D filter (proc 3), one 3D field 768x768x64, 5 generations, line reach 12, hz=4",
            "dtype": str(dtype).replace("torch.", ""), "ms": ms, "value": pts / (ms * 1e-3), "unit": UNIT,
            "line_kernel": {"bound": "hbm", "ms_per_call": line_ms, "achieved": gbs, "peak": peak_gbs,
                            "unit": "GB/s", "frac": gbs / peak_gbs if gbs else None,
                            "algorithmic_bytes": "2 passes x 2 x 4 B per point of each generation"}}


def rad3_forward(torch, dev, dtype):
    """filtering_procedure(4) (filtering_rad3) on a 768x768 field with one
    64-level 3D variable (3D ball, mg_ampl03 = 1: reach 2) and one 2D
    variable (disk reach 4), 5 generations.  The ball is a direct sum
    (~120 taps per point); the stage timers give its share."""
    from standalone_mgbf_loc_gb300 import MGBF, MGBFConfig, _abi
    cfg = MGBFConfig(nxPE=16, nyPE=16, im_filt=48, jm_filt=48, lm=64, km3=1, km2=1, n_ens=1, gm_max=5,
                     hx=4, hy=4, hz=4, p=2, mg_ampl02=ampl02(4), mg_ampl01=ampl01(4), mg_ampl03=1.0,
                     mg_weig1=1.0, mg_weig2=0.5, mg_weig3=0.25, mg_weig4=0.125, mg_weig5=0.0625, layout=1)
    op = MGBF(cfg)
    gen = torch.Generator(device=dev)
    gen.manual_seed(10)
    x = torch.randn(op.field_shape(), generator=gen, device=dev, dtype=dtype)
    for _ in range(2):
        op.filtering_procedure(4, x)
    torch.cuda.synchronize()
    n = 5
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(n):
        op.filtering_procedure(4, x)
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / n
    _abi.timers_enable(True)
    op.filtering_procedure(4, x)
    torch.cuda.synchronize()
    st = _abi.timers_read()
    _abi.timers_enable(False)
    pts = float(np.prod(op.field_shape()))
    op.close()
    return {"workload": "filtering_rad3 (proc 4), 768x768, one 64-level 3D variable (ball reach 2) + one 2D "
                        "variable (disk reach 4), 5 generations",
            "dtype": str(dtype).replace("torch.", ""), "ms": ms, "value": pts / (ms * 1e-3), "unit": UNIT,
            "stages_ms": {k: v[1] for k, v in st.items()}}


def lin2_forward(torch, dev, dtype):
    """filtering_procedure(2) (filtering_lin2_bckg) on one 768x768x64 field,
    5 generations, hz=4, mg_ampl02 = 0.3: per generation three dibeta line
    filters, half-span 3 along x and y and the identity on the diagonal
    (the triad of the Cholesky factor of the inverse aspect)."""
    from standalone_mgbf_loc_gb300 import MGBF, MGBFConfig, _abi
    cfg = MGBFConfig(nxPE=16, nyPE=16, im_filt=48, jm_filt=48, lm=64, km3=1, km2=0, n_ens=1, gm_max=5,
                     hx=12, hy=12, hz=4, p=2, mg_ampl02=0.3, mg_ampl01=ampl01(4), mgbf_line=True,
                     mg_weig1=1.0, mg_weig2=0.5, mg_weig3=0.25, mg_weig4=0.125, mg_weig5=0.0625, layout=1)
    op = MGBF(cfg)
    gen = torch.Generator(device=dev)
    gen.manual_seed(11)
    x = torch.randn(op.field_shape(), generator=gen, device=dev, dtype=dtype)
    for _ in range(2):
        op.filtering_procedure(2, x)
    torch.cuda.synchronize()
    n = 5
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(n):
        op.filtering_procedure(2, x)
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / n
    _abi.timers_enable(True)
    op.filtering_procedure(2, x)
    torch.cuda.synchronize()
    st = _abi.timers_read()
    _abi.timers_enable(False)
    pts = float(np.prod(op.field_shape()))
    op.close()
    return {"workload": "filtering_lin2_bckg (proc 2), one 3D field 768x768x64, 5 generations, line half-span 3",
            "dtype": str(dtype).replace("torch.", ""), "ms": ms, "value": pts / (ms * 1e-3), "unit": UNIT,
            "stages_ms": {k: v[1] for k, v in st.items()}}


def lin3_forward(torch, dev, dtype):
    """filtering_procedure(5) (filtering_lin3) on one 768x768x64 field, 5
    generations: per generation the seven colors of the hexad's 3D line
    filters (x, y and z lines of half-span 2 at mg_ampl03 = 0.6, three
    identity diagonals, color 7 null) on both sides, restriction and
    prolongation as procedure 1."""
    from standalone_mgbf_loc_gb300 import MGBF, MGBFConfig, _abi
    cfg = MGBFConfig(nxPE=16, nyPE=16, im_filt=48, jm_filt=48, lm=64, km3=1, km2=0, n_ens=1, gm_max=5,
                     hx=12, hy=12, hz=3, p=2, mg_ampl02=0.3, mg_ampl01=ampl01(3), mg_ampl03=0.6, mgbf_line=True,
                     mg_weig1=1.0, mg_weig2=0.5, mg_weig3=0.25, mg_weig4=0.125, mg_weig5=0.0625,
                     layout=_abi.MGBF_LAYOUT_COMPACT)
    op = MGBF(cfg)
    gen = torch.Generator(device=dev)
    gen.manual_seed(12)
    x = torch.randn(op.field_shape(), generator=gen, device=dev, dtype=dtype)
    for _ in range(2):
        op.filtering_procedure(5, x)
    torch.cuda.synchronize()
    n = 5
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(n):
        op.filtering_procedure(5, x)
    b.record()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b) / n
    _abi.timers_enable(True)
    op.filtering_procedure(5, x)
    torch.cuda.synchronize()
    st = _abi.timers_read()
    _abi.timers_enable(False)
    op.status()
    pts = float(np.prod(op.field_shape()))
    op.close()
    return {"workload": "filtering_lin3 (proc 5), one 3D field 768x768x64, 5 generations, 3D line half-span 2",
            "dtype": str(dtype).replace("torch.", ""), "ms": ms, "value": pts / (ms * 1e-3), "unit": UNIT,
            "stages_ms": {k: v[1] for k, v in st.items()}}


def transfers(torch, dev, dtype, peak_gbs, half=False):
    """anal_to_filt_all2 / filt_to_anal_all2 on the shipped namelist's grids:
    analysis 1440x960, filter 20x20 ranks of 64x32 (1280x640), 4 3D
    variables of 65 levels (lm_a = lm), lsqr interpolation.  HBM-bound:
    each direction reads one field and writes the other once.  `half`:
    both grids halved in x and y (720x480 <-> 10x10 ranks), for profiles."""
    from standalone_mgbf_loc_gb300 import MGBF, MGBFConfig
    d = 2 if half else 1
    cfg = MGBFConfig(nxPE=20 // d, nyPE=20 // d, im_filt=64, jm_filt=32, nm0=1440 // d, mm0=960 // d, lm=65, lm_a=65,
                     km3=4, km2=0,
                     n_ens=1, gm_max=4, hx=6, hy=6, hz=4, p=2, mg_ampl02=ampl02(6), mg_ampl01=ampl01(4),
                     layout=0)  # VALL with its halo, as the reference holds it
    op = MGBF(cfg)
    gen = torch.Generator(device=dev)
    gen.manual_seed(9)
    v = torch.randn(op.field_shape(), generator=gen, device=dev, dtype=dtype)
    w = torch.randn(op.analysis_shape(), generator=gen, device=dev, dtype=dtype)
    es = v.element_size()
    out = {"workload": f"transfers, analysis {1440 // d}x{960 // d} <-> filter {1280 // d}x{640 // d} "
                       f"({20 // d}x{20 // d} ranks of 64x32), 260 levels, lsqr, VALL with halo 6",
           "dtype": str(dtype).replace("torch.", "")}
    for name, fn in (("anal_to_filt", lambda: op.anal_to_filt(w, v)), ("filt_to_anal", lambda: op.filt_to_anal(v, w))):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        n = 10
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(n):
            fn()
        b.record()
        torch.cuda.synchronize()
        ms = a.elapsed_time(b) / n
        nbytes = (v.numel() + w.numel()) * es  # one field read, the other written
        gbs = nbytes / (ms * 1e-3) / 1e9
        out[name] = {"ms": ms, "achieved": gbs, "peak": peak_gbs, "unit": "GB/s", "frac": gbs / peak_gbs,
                     "algorithmic_bytes": nbytes}
    op.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--members", type=int, default=80)
    ap.add_argument("--no-extras", action="store_true", help="skip the plain-forward and CPU-baseline legs")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default radial-kernel tiles")
    ap.add_argument("--cfg5-steps", type=int, default=5, help="timed steps of the large BF16 leg")
    ap.add_argument("--cfg5-members", type=int, default=None,
                    help="members of the large BF16 leg run alone with --leg cfg5 (default 30; fewer for profiles)")
    ap.add_argument("--leg", choices=sorted(LEGS), help="run one secondary leg alone (fp32) and print its JSON line")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.leg:
        return run_leg(args.leg, args)
    if args.impl == "reference":
        return run_reference(args)
    return run_gpu(args)


# secondary legs, each runnable alone (used for kernel profiles)
LEGS = {
    "fast": lambda torch, dev, peak: fast_forward(torch, dev, torch.float32, peak),
    "transfers": lambda torch, dev, peak: transfers(torch, dev, torch.float32, peak),
    "transfers_half": lambda torch, dev, peak: transfers(torch, dev, torch.float32, peak, half=True),
    "rad3": lambda torch, dev, peak: rad3_forward(torch, dev, torch.float32),
    "lin2": lambda torch, dev, peak: lin2_forward(torch, dev, torch.float32),
    "lin3": lambda torch, dev, peak: lin3_forward(torch, dev, torch.float32),
    "plain": lambda torch, dev, peak: plain_forward(torch, dev, torch.float32),
    "cfg1": lambda torch, dev, peak: cfg1_leg(torch, dev)[0],
    "cfg3": lambda torch, dev, peak: cfg3_leg(torch, dev)[0],
    "cfg5": lambda torch, dev, peak: cfg5_leg(torch, dev, peak, 5, LEG_ARGS.get("cfg5_members"))[0],
}
LEG_ARGS = {}


def run_leg(name, args=None):
    import torch
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    peak, _ = measured_peaks()
    if args is not None:
        LEG_ARGS["cfg5_members"] = args.cfg5_members
    print(json.dumps({"leg": name, **LEGS[name](torch, dev, peak)}), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
