"""Benchmark of the GCMC energy hot path on GB300.

Headline workload: the framework energy grid of the large triclinic
supercell: a 24 Å base cell (angles 70/80/100 degrees, 422 atoms) replicated
4x4x4 (27 008 atoms), 0.2 Å spacing (457 x 437 x 437 nodes), the two LJ site
types of rigid CO2 as guest species, truncated-shifted LJ with rc = 12.8 Å,
FP32 pair terms with FP64 accumulation. The metric is energy-grid pair
evaluations per second, counted as the reference's loop counts them
(framework_energy_grid.cc:221-242): nodes x framework atoms x guest species.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

* ``value``: K timed grid builds with every input resident in HBM
  (alea_grid_rebuild), L2 flushed between steps; CUDA events on the launching
  stream; max over ranks.
* ``e2e``: the same metric through the public C-ABI call a user makes
  (alea_grid_build_to_host: the grid from host arrays with both tables copied
  into pinned host memory as the build's z-slabs finish), host<->device copies
  inside the timed region.
* ``roofline``: the build kernel against the FP32 FMA peak measured in the
  same run, scalar and packed (the kernel is FP32-pipe bound; the peaks file
  has no FP32 figure).
* ``fp32_error``: every node of the timed FP32-form grid against the FP64 form
  of the same grid, by node class (built after the timed region).
* ``cpu_baseline``: the CPU restatement of the reference's grid loop on a
  bounded sample of the same nodes, on all host cores.
* ``--impl reference``: the reference's CPU algorithm (the oracle port; the
  reference tree is not present on the GPU host) on all host cores, the same
  metric on a bounded node sample per step.
Multi-GPU: one replica of the workload per rank (weak scaling, no data-path
collective); the barrier and the max-over-ranks time reduction are control.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

SPACING = 0.2
CUTOFF = 12.8
REPS = 4
# Roofline unit: the reference's operation count per pair evaluation (node,
# atom image, guest species): 3 sub, 3 rint + 3 FMA min-image, 5 for r^2,
# 1 rcp, 1 s^2, 2 s^6, 1 s^12, 3 for 4 eps (s^12 - s^6) - V(rc), 1 accumulate,
# 1 compare/select = 24 FLOP, counted over the pairs the kernel evaluates.
FLOPS_PER_PAIR = 24
# What the FP32 sweep itself issues per evaluated node-image pair (an FMA
# counts 2): displacement 3, r^2 5, reciprocal 1, r^-6 2, and per guest
# species two FMAs (t = A r^-6 - B; sum += r^-6 t) = 4.
KERNEL_FLOPS_PER_NODE_IMAGE = 11
KERNEL_FLOPS_PER_SPECIES = 4
# DRAM bytes (read + write) of one sweep launch on this workload, from a
# single-pass ncu capture of the full workload (profiles/grid_build_f32_c5_dram.md)
SWEEP_DRAM_BYTES_PER_LAUNCH = 1422016256


def fp32_error_stats(t32, t64, kt=298.0, cap=1e5):
    """Error of an FP32-form grid table against the FP64 form of the same grid,
    over every node: pure relative |dE|/|E|, against max(kT, |E|), and the
    nodes above 1e-5 pure relative (with the largest |E| among them). Nodes at
    the cap in the FP64 form are counted too: their FP32 value is the cap, or
    a value just below it whose exact energy is just above it."""
    d = np.abs(t32 - t64)
    mag = np.abs(t64)
    with np.errstate(divide="ignore", invalid="ignore"):
        pure = np.where(mag > 0, d / mag, np.where(d > 0, np.inf, 0.0))
    floored = d / np.maximum(kt, mag)
    capped = t64 >= cap
    big = mag >= kt
    over = pure > 1e-5
    hot = (t64 > 1e4) & ~capped
    return {
        "nodes": int(t64.size),
        "capped_nodes": int(capped.sum()),
        "max_pure_rel_capped": float(pure[capped].max()) if capped.any() else 0.0,
        "max_abs_err_K": float(d.max()),
        "max_pure_rel": float(pure.max()),
        "max_rel_kT_floor": float(floored.max()),
        "max_pure_rel_abs_E_ge_kT": float(pure[big].max()) if big.any() else 0.0,
        "nodes_above_1e-5_pure_rel": int(over.sum()),
        "max_abs_E_above_1e-5_pure_rel_K": float(mag[over].max()) if over.any() else 0.0,
        "nodes_1e4_to_1e5_K": int(hot.sum()),
        "max_pure_rel_1e4_to_1e5_K": float(pure[hot].max()) if hot.any() else 0.0,
    }


def fp32_error(A, ff, parts, fw, guests, grid32):
    """The timed FP32-form grid against the FP64 form of the same grid, built
    after the timed region (the FP64 form equals the reference's loop to
    1e-10, tested)."""
    t0 = time.perf_counter()
    g64 = A.FrameworkEnergyGrid(ff, parts, fw.lattice, guests, SPACING, A.FP64)
    build_s = time.perf_counter() - t0
    st64 = g64.stats()
    out = {"kT_K": 298.0, "fp64_build_s": build_s, "reference": "FP64 form of the same grid",
           # the parity form's own rate on this workload (its one build, CUDA-event timed)
           "fp64_form_kernel_ms": float(st64["last_kernel_ms"]),
           "fp64_form_pair_evals_per_s":
               float(st64["algorithmic_pairs"]) / (float(st64["last_kernel_ms"]) * 1e-3)}
    for s in guests:
        out[f"guest_species_{s}"] = fp32_error_stats(grid32.table(s), g64.table(s))
    del g64
    return out


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    return ws, rank


def max_over_ranks(x: float, dist, device: str = "cuda") -> float:
    """The slowest rank's figure (every rank gets it): the replicas' job ends
    when the last one does. dist is None for one process."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(world: int, units_per_step: float, steps: int, seconds: float) -> float:
    """Whole-job throughput of `world` independent replicas, each doing
    units_per_step per step, timed by the slowest one."""
    return world * units_per_step * steps / seconds


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-i", str(self.gpu), "-lms", "200"], stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() in ("active", "1", "0x1"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def make_workload(reps: int = REPS):
    """reps=4: the benchmark workload; reps=2: the same cell 2x2x2 (8x fewer
    nodes and atoms, tables still larger than L2) used for profiler captures."""
    from aleator_gb300 import workloads as W
    fw = W.triclinic_supercell(reps=reps)
    guests = [fw.guest_species["CO2_C"], fw.guest_species["CO2_O"]]
    return fw, guests


def cpu_grid_rate(fw, guests, seconds_target=12.0, threads=None):
    """Reference grid loop (CPU restatement) on a bounded node sample."""
    import oracle as O
    orc = O.Oracle()
    threads = threads or os.cpu_count() or 1
    ff = dict(eps=fw.eps, sigma=fw.sigma, cutoff=CUTOFF, truncation=O.SHIFTED)
    counts = orc.grid_point_counts(fw.lattice, SPACING)
    total = counts[0] * counts[1] * counts[2]
    # calibrate on a small sample, then size the measured sample
    probe = max(threads, 16)
    t0 = time.perf_counter()
    orc.grid_build(ff, fw.lattice, fw.x, fw.y, fw.z, fw.species, guests[0], SPACING, 0, probe,
                   threads)
    dt = max(time.perf_counter() - t0, 1e-6)
    per_node = dt / probe
    nodes = int(min(total, max(probe, seconds_target / per_node / len(guests))))
    start = (total // 2) - nodes // 2  # a slab through the middle of the cell
    t0 = time.perf_counter()
    for g in guests:
        orc.grid_build(ff, fw.lattice, fw.x, fw.y, fw.z, fw.species, g, SPACING, start,
                       start + nodes, threads)
    dt = time.perf_counter() - t0
    pairs = nodes * fw.n_atoms * len(guests)
    return pairs / dt, dict(nodes=nodes, pairs=pairs, seconds=dt, threads=threads,
                            sample=f"{nodes} grid nodes x {fw.n_atoms} atoms x {len(guests)} species "
                                   f"(node range [{start}, {start + nodes}) of {total})")


def run_reference(args):
    ws, rank = _dist()
    if rank != 0:
        return 0
    fw, guests = make_workload()
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_grid_rate(fw, guests, seconds_target=2.0, threads=threads)
    t0 = time.perf_counter()
    rates, info = [], None
    for _ in range(args.steps):
        r, info = cpu_grid_rate(fw, guests, seconds_target=8.0, threads=threads)
        rates.append(r)
    wall = time.perf_counter() - t0
    value = float(np.mean(rates))
    line = {
        "impl": "reference", "metric": "energy-grid pair evals/s", "value": value,
        "unit": "pair evals/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": wall * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": _config(fw, guests),
        "cpu_baseline": {"value": value, "unit": "pair evals/s", "cores": threads, "kind": "port",
                         "sample": info["sample"] + " per step"},
        "e2e": {"value": value, "unit": "pair evals/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "the reference tree is not present on the GPU host, so its compiled code "
                "(oracle/_ref) cannot be rebuilt there; this is the C restatement of the same "
                "loop, checked bit-exact against the reference's own build in the test suite",
    }
    print(json.dumps(line), flush=True)
    return 0


def _config(fw, guests, counts=(457, 437, 437), reps=REPS):
    return {"workload": f"framework energy grid, {reps}x{reps}x{reps} triclinic supercell "
                        "(a=b=c=24 Å, 70/80/100 deg) of 422 atoms, CO2 guest site types, "
                        "0.2 Å spacing" + ("" if reps == REPS else " [profiling case]"),
            "framework_atoms": int(fw.n_atoms), "guest_species": len(guests),
            "grid_points": "x".join(str(c) for c in counts), "cutoff_angstrom": CUTOFF,
            "spacing_angstrom": SPACING,
            "truncation": "shifted", "l2": "256 MB buffer written between timed steps; each "
                                          "step also writes 1.4 GB of tables (> L2)",
            "parallelism": "replica per GPU"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--no-henry", action="store_true",
                    help="leave out the learned-vs-uniform half (profiling runs of the grid)")
    ap.add_argument("--workload", default="full", choices=["full", "small"],
                    help="small: 2x2x2 supercell for profiler captures (not a bench line)")
    ap.add_argument("--henry-scatter", action="store_true",
                    help="the learned K_H over six proposal seeds and three uniform shares")
    ap.add_argument("--henry-judge", type=float, default=None, metavar="SECONDS",
                    help="run the uniform-insertion judge of the learned Henry coefficient for "
                         "SECONDS and print one JSON line (no bench line)")
    ap.add_argument("--loading", type=float, default=None, metavar="SECONDS",
                    help="the C4 loading comparison at 0.1, 1, 10 and 30 bar, SECONDS per arm, "
                         "one JSON line (no bench line)")
    ap.add_argument("--orientation-trials", type=int, default=6)
    ap.add_argument("--c5-isotherm", type=float, default=None, metavar="SECONDS",
                    help="run the C5 isotherm's 64 chains for SECONDS and print one JSON line")
    ap.add_argument("--kernel-case", default=None, choices=["gcmc", "gcmc_c5", "widom", "widom_q32", "interp", "ewald"],
                    help="one small case of a non-grid kernel for profiler captures, then exit "
                         "(no bench line)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.kernel_case:
        return kernel_case(args.kernel_case)
    if args.c5_isotherm:
        import torch
        import aleator_gb300 as A
        A.load_library()
        print(json.dumps(c5_isotherm(A, torch, args.c5_isotherm)), flush=True)
        return 0
    if args.loading:
        import torch
        import aleator_gb300 as A
        A.load_library()
        print(json.dumps(loading_comparison(A, torch, seconds=args.loading,
                                            orient=args.orientation_trials,
                                            arms=("uniform", "uniform_orient", "learned"))),
              flush=True)
        return 0
    if args.henry_scatter:
        import torch
        import aleator_gb300 as A
        A.load_library()
        henry_scatter(A, torch)
        return 0
    if args.henry_judge:
        import torch
        import aleator_gb300 as A
        A.load_library()
        print(json.dumps(henry_judge(A, torch, args.henry_judge)), flush=True)
        return 0

    import torch
    import aleator_gb300 as A

    ws, rank = _dist()
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    A.load_library()

    fw, guests = make_workload(REPS if args.workload == "full" else 2)
    ff = A.LennardJones(fw.eps, fw.sigma, CUTOFF, A.SHIFTED)
    parts = A.ParticleData.from_framework(fw)
    grid = A.FrameworkEnergyGrid(ff, parts, fw.lattice, guests, SPACING, A.FP32)
    st = grid.stats()
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    for _ in range(args.warmup):
        grid.rebuild(sp)
    torch.cuda.synchronize()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    sweep_ms, launches = [], 0
    with ClockSampler(local) as clocks:
        t0 = time.perf_counter()
        for i in range(args.steps):
            flush.fill_(float(i))
            starts[i].record(stream)
            grid.rebuild(sp)
            ends[i].record(stream)
            st_i = grid.stats()  # the build synchronises; its launch's event time
            sweep_ms.append(st_i["last_kernel_ms"])
            launches += st_i["launches"]
        torch.cuda.synchronize()
        region_s = time.perf_counter() - t0
    if dist:
        dist.barrier()
    kernel_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    step_ms = float(np.mean(kernel_ms))
    st = grid.stats()
    total_ms = max_over_ranks(float(np.sum(kernel_ms)), dist)
    pairs_step = st["algorithmic_pairs"]
    value = replica_value(ws, pairs_step, args.steps, total_ms * 1e-3)

    # e2e through the public call with host buffers (pinned host output)
    nodes = st["nodes"]
    pinned = [torch.empty(nodes, dtype=torch.float64, pin_memory=True) for _ in guests]
    h2d = st["images"] * 32 + (fw.n_atoms * (4 * 8 + 4))
    d2h = nodes * 8 * len(guests)
    e2e_steps = max(2, min(args.steps, 5))

    def e2e_step():  # alea_grid_build_to_host: the build with the table copies overlapped
        A.FrameworkEnergyGrid.build_to_host(ff, parts, fw.lattice, guests, SPACING, A.FP32,
                                            [t.data_ptr() for t in pinned], keep=False)

    e2e_step()  # untimed warm-up: the first copy into freshly pinned pages runs at half speed
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_step()
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, dist)
    e2e_value = replica_value(ws, pairs_step, e2e_steps, e2e_s)

    if rank == 0:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) \
            if (ROOT / "MEASURED_PEAKS.json").exists() else {}
        scalar_peak = A.fp32_fma_tflops()
        packed_peak = A.fp32_fma_tflops(packed=True)
        fp32_peak = max(scalar_peak, packed_peak)  # the device's FP32 FMA peak
        ng = len(guests)
        node_image = st["executed_pairs"] / ng
        sweep = float(np.mean(sweep_ms))
        achieved = st["executed_pairs"] * FLOPS_PER_PAIR / (sweep * 1e-3) / 1e12
        kflops = node_image * (KERNEL_FLOPS_PER_NODE_IMAGE + KERNEL_FLOPS_PER_SPECIES * ng)
        kachieved = kflops / (sweep * 1e-3) / 1e12
        line = {
            "metric": "energy-grid pair evals/s", "value": value, "unit": "pair evals/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32 pair terms, fp64 accumulation", "data": "synthetic",
            "config": _config(fw, guests, grid.point_counts(),
                              REPS if args.workload == "full" else 2),
            "region_ms": region_s * 1e3,
            "gpu_launches": launches,
            "roofline": {
                "bound": "fp32", "achieved": achieved, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": achieved / fp32_peak,
                "peak_source": "the larger of two FP32 FMA loops measured in this run: scalar "
                               "fmaf (alea_probe_fp32_fma_tflops) and packed fma.rn.f32x2 "
                               "(alea_probe_fp32x2_fma_tflops), the instruction the sweep issues",
                "peak_scalar_fma": scalar_peak, "peak_packed_fma": packed_peak,
                "frac_vs_scalar_peak": achieved / scalar_peak,
                "frac_vs_packed_peak": achieved / packed_peak,
                "traffic": SWEEP_DRAM_BYTES_PER_LAUNCH if args.workload == "full" else None,
                "kernel": "grid_build_f32_kernel<2,SHIFTED>, timed with the grid_plan_kernel "
                          "launch before it (the bricks' row plans, ~1 % of the time)",
                "kernel_ms": sweep,
                "flops_per_pair": FLOPS_PER_PAIR,
                "executed_pairs_per_step": int(st["executed_pairs"]),
                "kernel_issued_flops_per_node_image_pair":
                    KERNEL_FLOPS_PER_NODE_IMAGE + KERNEL_FLOPS_PER_SPECIES * ng,
                "kernel_issued_achieved": kachieved,
                "kernel_issued_frac": kachieved / fp32_peak,
                "kernel_issued_frac_vs_scalar_peak": kachieved / scalar_peak,
                "kernel_issued_frac_vs_packed_peak": kachieved / packed_peak,
            },
            "e2e": {"value": e2e_value, "unit": "pair evals/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h), "steps": e2e_steps},
            "clocks": clocks.summary(),
            "peaks_file": {k: peaks.get(k) for k in ("hbm_gbs", "bf16_tflops")},
        }
        line["fp32_error"] = fp32_error(A, ff, parts, fw, guests, grid)
        if not args.no_cpu_baseline:
            rate, info = cpu_grid_rate(fw, guests, seconds_target=12.0)
            line["cpu_baseline"] = {"value": rate, "unit": "pair evals/s",
                                    "cores": info["threads"], "kind": "port",
                                    "sample": info["sample"]}
        if not args.no_henry:
            line["henry_time_to_1pct"] = henry_time_to_1pct(A, torch, gcmc=not args.no_extras)
        if not args.no_extras:
            line["extra"] = extras(A, torch, peaks)
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def combine_widom(chunks, temperature):
    """K_H and its relative standard error over consecutive chunks of one
    trial stream, from each chunk's (trials, log mean weight, relative s.e.):
    the chunks' first and second moments of the weight, combined in log
    space (the weights reach e^40 and more on this framework)."""
    n = np.array([c["n_trials"] for c in chunks], dtype=np.float64)
    lm = np.array([c["log_mean_weight"] for c in chunks])
    rel = np.array([c["rel_std_error"] for c in chunks])
    ln = np.log(n)
    lm2 = 2.0 * lm + np.log1p(rel * rel * n)  # log E[w^2] of each chunk
    big_n = n.sum()

    def lse(v):
        m = v.max()
        return m + np.log(np.exp(v - m).sum())

    l1 = lse(lm + ln) - np.log(big_n)
    l2 = lse(lm2 + ln) - np.log(big_n)
    var_rel = max(np.expm1(l2 - 2.0 * l1), 0.0)
    return {"trials": int(big_n), "henry": float(np.exp(l1) / temperature),
            "log_mean_weight": float(l1), "rel_std_error": float(np.sqrt(var_rel / big_n))}


def run_to_target(torch, run_chunk, temperature, target, cap_s, first_chunk, max_chunk):
    """Consecutive chunks of one trial stream until the combined relative
    standard error reaches the target or the time cap passes; wall time
    measured (device synchronised)."""
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    chunks, first, size = [], 0, first_chunk
    while True:
        chunks.append(run_chunk(first, size))
        first += size
        comb = combine_widom(chunks, temperature)
        torch.cuda.synchronize()
        elapsed = time.perf_counter() - t0
        if comb["rel_std_error"] <= target or elapsed >= cap_s:
            break
        size = min(2 * size, max_chunk)
    comb.update(seconds=elapsed, reached=comb["rel_std_error"] <= target,
                chunks=[(int(c["n_trials"]), float(c["log_mean_weight"]), float(c["rel_std_error"]))
                        for c in chunks])
    return comb


def henry_setup(A):
    """The C4 workload: the charged 424-atom cubic cell, rigid 3-site CO2,
    Ewald for 1e-6 relative precision (alpha and kMax from the rule), rc 12 Å,
    LJ shifted at 12.8 Å, 298 K."""
    from aleator_gb300 import workloads as W
    fw = W.cubic_framework(charged=True)
    alpha, kmax = W.ewald_parameters(fw.lattice, 12.0)
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    ew = A.Ewald(alpha, 12.0, kmax)
    return fw, ff, p, ew, W.co2_guest(fw), 298.0, alpha, kmax


# the learned proposal's training budget: 2e6 Boltzmann-weighted Widom samples
# over three adaptive rounds (each round's rows drawn from the previous table)
TRAIN_SAMPLES = 2_000_000
TRAIN_ROUNDS = 3


def fit_proposal(A, widom, seed=2, stream=7, epochs=8, cells=128):
    """The learned proposal of the Henry workload, tabulated on cells^3 cells:
    the deep wells are narrower than a 64^3 cell (0.4 A), so within such a cell
    the Boltzmann weight still varies by orders of magnitude; 128^3 cells cut
    the trials to a 1 % K_H about 7x against 64^3 (measured over three seeds)."""
    prop = A.Proposal(seed=seed)
    prop.fit(widom, n_samples=TRAIN_SAMPLES // TRAIN_ROUNDS, rounds=TRAIN_ROUNDS, epochs=epochs,
             cells=cells, stream=stream)
    return prop


def henry_time_to_1pct(A, torch, gcmc=True, cap_s=60.0):
    """The second half of the metric: wall time to a 1 % relative-error Henry
    coefficient, learned proposal against uniform insertion, on the C4
    workload (henry_setup), both in the FP32 form (its per-trial energies are
    within 1e-5 of the FP64 form's, tested).

    Both arms are measured, not extrapolated: each runs consecutive chunks of
    one trial stream until its relative standard error reaches 1 % or the time
    cap passes. The learned arm's time includes fitting the proposal on the
    GPU (2e6 training samples). Where uniform insertion does not reach 1 %
    within the cap, the speed-up is a measured lower bound (cap over the
    learned time). The uniform estimate's own standard error is unreliable on
    this heavy-tailed weight distribution (rare deep electrostatic wells), so
    the two estimates are also compared in combined standard errors."""
    fw, ff, p, ew, guest, T, alpha, kmax = henry_setup(A)
    widom = A.Widom(ff, p, fw.lattice, guest, T, ewald=ew, precision=A.FP32)
    widom.run(1, 0, 4096)  # warm-up
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    prop = fit_proposal(A, widom)
    torch.cuda.synchronize()
    t_fit = time.perf_counter() - t0
    learned = run_to_target(torch, lambda f, n: widom.run_biased(prop, 42, 0, n, first_trial=f),
                            T, 0.01, cap_s, 1 << 20, 1 << 24)
    learned["fit_seconds"] = t_fit
    learned["time_to_1pct_s"] = t_fit + learned["seconds"] if learned["reached"] else None
    uniform = run_to_target(torch, lambda f, n: widom.run(42, 1, n, first_trial=f), T, 0.01, cap_s,
                            1 << 22, 1 << 26)
    uniform["time_to_1pct_s"] = uniform["seconds"] if uniform["reached"] else None
    se = np.hypot(learned["rel_std_error"] * learned["henry"],
                  uniform["rel_std_error"] * uniform["henry"])
    tl = learned["time_to_1pct_s"]
    out = {
        "workload": "charged 424-atom cubic cell (25.832 A), rigid 3-site CO2, Ewald 1e-6 "
                    f"(alpha {alpha:.4f}, kMax {kmax}), 298 K, FP32 form; proposal trained on "
                    f"{TRAIN_SAMPLES} Widom samples",
        "learned": learned, "uniform": uniform, "uniform_cap_s": cap_s,
        "speedup": (uniform["time_to_1pct_s"] / tl) if (tl and uniform["reached"]) else None,
        "speedup_lower_bound": (uniform["seconds"] / tl) if (tl and not uniform["reached"]) else None,
        "henry_difference_in_combined_se": abs(learned["henry"] - uniform["henry"]) / se,
    }
    if gcmc:
        out["gcmc_loading"] = loading_comparison(A, torch, pressures_bar=(10.0,), seconds=15.0,
                                                 arms=("uniform", "uniform_orient", "learned"))
    return out


def henry_judge(A, torch, seconds):
    """The plain method as the judge of the learned K_H: uniform insertion for
    `seconds` of FP32 trials, and an independent learned run (another seed,
    stream and proposal) to 0.5 %; one JSON line."""
    fw, ff, p, ew, guest, T, alpha, kmax = henry_setup(A)
    widom = A.Widom(ff, p, fw.lattice, guest, T, ewald=ew, precision=A.FP32)
    prop = fit_proposal(A, widom, seed=5, stream=21)
    learned = run_to_target(torch, lambda f, n: widom.run_biased(prop, 77, 3, n, first_trial=f),
                            T, 0.005, 600.0, 1 << 22, 1 << 24)
    uniform = run_to_target(torch, lambda f, n: widom.run(77, 4, n, first_trial=f), T, 0.0,
                            seconds, 1 << 24, 1 << 27)
    se = np.hypot(learned["rel_std_error"] * learned["henry"],
                  uniform["rel_std_error"] * uniform["henry"])
    return {"henry_judge": {"learned": learned, "uniform": uniform,
                            "difference_in_combined_se": abs(learned["henry"] - uniform["henry"]) / se,
                            "difference_in_uniform_se":
                                abs(learned["henry"] - uniform["henry"]) /
                                (uniform["rel_std_error"] * uniform["henry"])}}


def henry_scatter(A, torch, seeds=(1, 3, 5, 8, 13, 21), shares=(0.05, 0.2, 0.4)):
    """The learned K_H across proposals: for each proposal seed (training
    stream 100 + seed) and uniform share, a run to 1 % (trial seed 900 + seed,
    stream 3) and a run of 2^25 trials (seed 500 + seed, stream 5). One JSON
    line per run."""
    fw, ff, p, ew, guest, T, alpha, kmax = henry_setup(A)
    widom = A.Widom(ff, p, fw.lattice, guest, T, ewald=ew, precision=A.FP32)
    for seed in seeds:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        prop = fit_proposal(A, widom, seed=seed, stream=100 + seed)
        torch.cuda.synchronize()
        fit_s = time.perf_counter() - t0
        for share in shares:
            prop.tabulate(128, share)
            r = run_to_target(torch, lambda f, n: widom.run_biased(prop, 900 + seed, 3, n, first_trial=f),
                              T, 0.01, 20.0, 1 << 20, 1 << 22)
            big = widom.run_biased(prop, 500 + seed, 5, 1 << 25)
            print(json.dumps({"seed": seed, "share": share, "fit_s": fit_s,
                              "to1pct_trials": r["trials"], "to1pct_s": r["seconds"],
                              "to1pct_henry": r["henry"], "to1pct_se": r["rel_std_error"],
                              "big_henry": big["henry"], "big_se": big["rel_std_error"]}), flush=True)


def loading_run(A, torch, ff, p, fw, guest, ew, T, pressure_pa, learned, seconds, n=152,
                block=5000, refits=3, proposal=None, orient=1, seed0=2000):
    """One arm of the loading comparison: n FP32 chains of charged CO2 from an
    empty cell at one pressure (Peng-Robinson fugacity), blocks of `block`
    moves until `seconds` of wall time. The learned arm starts from `proposal`
    (trained on the empty framework; its fit time is counted) and refits at
    loading before each of its first `refits` blocks (timed). Returns the
    per-block trajectory: (wall time, per-chain mean N over the block)."""
    from aleator_gb300 import workloads as W
    fug = A.peng_robinson_fugacity(*W.CO2_CRITICAL, T, pressure_pa)
    ch = A.GcmcChains(ff, p, fw.lattice, guest, T, [fug] * n, list(range(seed0, seed0 + n)),
                      [7] * n, ewald=ew, max_molecules=800, precision=A.FP32)
    if orient > 1:
        ch.set_orientation_trials(orient)
    prop, t_total, fit_s = None, 0.0, 0.0
    if learned:
        prop, fit_s = proposal
        t_total += fit_s
        ch.set_proposal(prop)
    prev = np.array([ch.info(c)["sum_molecules"] for c in range(n)])
    traj, b = [], 0
    while t_total < seconds:
        if learned and b < refits:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            prop.fit_at_loading(ch, ff, p, fw.lattice, guest, T, ewald=ew, chain_ids=range(8),
                                n_samples=1 << 17, rounds=1, epochs=10, cells=48,
                                uniform_share=0.2, seed=100 + b, stream=10 * b)
            ch.set_proposal(prop)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            fit_s += dt
            t_total += dt
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ch.run(block)
        torch.cuda.synchronize()
        t_total += time.perf_counter() - t0
        cur = np.array([ch.info(c)["sum_molecules"] for c in range(n)])
        traj.append((t_total, (cur - prev) / block))
        prev = cur
        b += 1
    att = np.array([ch.info(c)["attempted"] for c in range(n)]).sum(0)
    acc = np.array([ch.info(c)["accepted"] for c in range(n)]).sum(0)
    return {"traj": traj, "fit_seconds": fit_s, "moves_per_chain": block * b,
            "insert_acceptance": float(acc[2] / max(att[2], 1)),
            "delete_acceptance": float(acc[3] / max(att[3], 1))}


def loading_metrics(traj, ref, n):
    """For each block end t: the loading estimate over the second half of the
    blocks so far (the first half discarded as burn-in) and its standard error
    over the independent chains. Time to 1 %: the first t at which the
    estimate is within 1 % of the reference loading `ref` and its standard
    error is at most 1 % of it."""
    t_hit, est = None, None
    for k in range(1, len(traj) + 1):
        half = traj[k // 2:k]
        per_chain = np.mean([m for _, m in half], axis=0)
        est = float(per_chain.mean())
        se = float(per_chain.std(ddof=1) / np.sqrt(n))
        if t_hit is None and abs(est - ref) <= 0.01 * ref and se <= 0.01 * ref:
            t_hit = traj[k - 1][0]
    return t_hit, est


def loading_comparison(A, torch, pressures_bar=(0.1, 1.0, 10.0, 30.0), seconds=30.0, n=152,
                       orient=6, arms=("uniform", "learned")):
    """GCMC loading on the C4 workload at each pressure, the learned form
    (learned insertion proposal and `orient` orientation trials per insertion
    and deletion) against the reference's moves (uniform insertion, one
    orientation); arm "uniform_orient" adds the orientation trials alone. All
    arms run for the same wall time from an empty cell; the reference loading
    is the mean over the arms' last quarter of blocks (their final estimates
    agree within their standard errors when they have equilibrated); each
    arm's time to a 1 %-accurate loading with a 1 % standard error
    (loading_metrics), and the ratio uniform / learned."""
    fw, ff, p, ew, guest, T, alpha, kmax = henry_setup(A)
    widom = A.Widom(ff, p, fw.lattice, guest, T, ewald=ew, precision=A.FP32)
    out = {"workload": "charged 424-atom cubic cell, rigid CO2, Ewald 1e-6, 298 K, FP32 chains, "
                       f"{n} chains per arm from an empty cell, {seconds:.0f} s per arm",
           "orientation_trials": orient}
    for P_bar in pressures_bar:
        res = {}
        for arm in arms:
            learned = arm == "learned"
            prop = None
            if learned:
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                pr = fit_proposal(A, widom)
                torch.cuda.synchronize()
                prop = (pr, time.perf_counter() - t0)
            res[arm] = loading_run(A, torch, ff, p, fw, guest, ew, T, P_bar * 1e5, learned, seconds,
                                   n=n, proposal=prop, orient=1 if arm == "uniform" else orient)
        tail = [m for arm in res.values() for _, m in arm["traj"][-max(1, len(arm["traj"]) // 4):]]
        ref = float(np.mean(tail))
        row = {"reference_loading": ref}
        for name, arm in res.items():
            t_hit, est = loading_metrics(arm["traj"], ref, n)
            traj = arm.pop("traj")
            arm.update(time_to_1pct_s=t_hit, final_estimate=est,
                       wall_s=float(traj[-1][0]) if traj else 0.0,
                       trajectory=[(round(t, 2), round(float(m.mean()), 2)) for t, m in traj[::3]])
            row[name] = arm
        tu, tl = row["uniform"]["time_to_1pct_s"], row["learned"]["time_to_1pct_s"]
        wu = row["uniform"]["wall_s"]

        def ratio(t_other):  # uniform's time over the arm's; a lower bound when uniform never got there
            if not t_other:
                return None, None
            return (tu / t_other, None) if tu else (None, wu / t_other)

        row["speedup"], row["speedup_lower_bound"] = ratio(tl)
        if "uniform_orient" in row:  # the orientation trials alone
            row["speedup_orientation_trials"], row["speedup_orientation_trials_lower_bound"] = \
                ratio(row["uniform_orient"]["time_to_1pct_s"])
        out[f"{P_bar:g} bar"] = row
    return out


def kernel_case(case):
    """Small cases of the non-grid kernels for ncu captures (each a few
    launches, tens of milliseconds):
      gcmc:   152 FP32 charged-CO2 chains (kMax 10) in the charged 424-atom cell,
              1 bar, a 2000-move launch then a 300-move launch;
      widom:  2^20 FP32 CH4 trials (424-atom cell), then 2^16 FP64 charged-CO2
              trials (kMax 10);
      interp: 2^24 random queries on the FP32-form grid of the 2x2x2 supercell
              (0.2 A, 174 MB table), then the same on its FP64-form grid;
      widom_q32: charged CO2 in the charged 424-atom cell (kMax 10), FP32 form:
              2^16 then 2^18 trials;
      gcmc_c5: the large isotherm case (64 FP32 chains of charged CO2 in the
              27 008-atom supercell with its 0.2 A grid, kMax 34), a 200-move
              launch then a 100-move launch;
      ewald:  the EwaldIncrementalState of the charged 2x2x2 supercell (3 376
              atoms, alpha and kMax for 1e-6, rc 12 A): the S(k) build, then 8
              CO2 insertion proposals and commits (6 sites per move proposal)."""
    import torch
    import aleator_gb300 as A
    from aleator_gb300 import workloads as W
    A.load_library()
    if case == "gcmc":
        fw = W.cubic_framework(charged=True)
        alpha, kmax = W.ewald_parameters(fw.lattice, 12.0)
        ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
        fug = A.peng_robinson_fugacity(*W.CO2_CRITICAL, 298.0, 1e5)
        ch = A.GcmcChains(ff, A.ParticleData.from_framework(fw), fw.lattice, W.co2_guest(fw), 298.0,
                          [fug] * 152, list(range(152)), [0] * 152, ewald=A.Ewald(alpha, 12.0, kmax),
                          max_molecules=600, precision=A.FP32)
        ch.run(2000)
        ch.run(300)
    elif case == "widom":
        fw = W.cubic_framework()
        ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
        A.Widom(ff, A.ParticleData.from_framework(fw), fw.lattice, W.ch4_guest(fw), 298.0,
                precision=A.FP32).run(42, 0, 1 << 20)
        fq = W.cubic_framework(charged=True)
        alpha, kmax = W.ewald_parameters(fq.lattice, 12.0)
        A.Widom(A.LennardJones(fq.eps, fq.sigma, 12.8, A.SHIFTED), A.ParticleData.from_framework(fq),
                fq.lattice, W.co2_guest(fq), 298.0, ewald=A.Ewald(alpha, 12.0, kmax)).run(42, 0, 1 << 16)
    elif case == "widom_q32":
        fq = W.cubic_framework(charged=True)
        alpha, kmax = W.ewald_parameters(fq.lattice, 12.0)
        w = A.Widom(A.LennardJones(fq.eps, fq.sigma, 12.8, A.SHIFTED), A.ParticleData.from_framework(fq),
                    fq.lattice, W.co2_guest(fq), 298.0, ewald=A.Ewald(alpha, 12.0, kmax),
                    precision=A.FP32)
        w.run(42, 0, 1 << 16)
        w.run(42, 0, 1 << 18)
    elif case == "gcmc_c5":
        fw, guests = make_workload()
        alpha, kmax = W.ewald_parameters(fw.lattice, 12.0)
        ff = A.LennardJones(fw.eps, fw.sigma, CUTOFF, A.SHIFTED)
        p = A.ParticleData.from_framework(fw)
        grid = A.FrameworkEnergyGrid(ff, p, fw.lattice, guests, SPACING, A.FP32)
        pressures = np.logspace(np.log10(0.01), np.log10(50.0), 64)
        fugs = [A.peng_robinson_fugacity(*W.CO2_CRITICAL, 298.0, P * 1e5) for P in pressures]
        ch = A.GcmcChains(ff, p, fw.lattice, W.co2_guest(fw), 298.0, fugs, list(range(64)),
                          list(range(64)), ewald=A.Ewald(alpha, 12.0, kmax), max_molecules=4000,
                          precision=A.FP32)
        ch.set_grid(grid)
        ch.run(200)
        ch.run(100)
    elif case == "ewald":
        fw = W.triclinic_supercell(reps=2)
        alpha, kmax = W.ewald_parameters(fw.lattice, 12.0)
        p = A.ParticleData.from_framework(fw)
        st = A.EwaldIncrementalState(A.Ewald(alpha, 12.0, kmax), p, fw.lattice)
        rng = np.random.default_rng(1)
        mols = []
        for i in range(8):
            c = rng.uniform(0.0, 1.0, 3) @ fw.lattice
            m = np.array([[c[0], c[1], c[2] - 1.16, -0.35], [c[0], c[1], c[2], 0.7],
                          [c[0], c[1], c[2] + 1.16, -0.35]])
            st.propose_insertion(m)
            st.commit_insertion(m)
            mols.append(m)
        for m in mols:
            st.propose_move(m, m + np.array([0.3, -0.2, 0.1, 0.0]))
        print(f"terms {st.term_count()} atoms {fw.n_atoms}")
    else:
        fw, guests = make_workload(2)
        ff = A.LennardJones(fw.eps, fw.sigma, CUTOFF, A.SHIFTED)
        n = 1 << 24
        xyz = (torch.rand(n, 3, dtype=torch.float64, device="cuda")
               @ torch.tensor(fw.lattice, device="cuda")).contiguous()
        res = torch.empty(n, dtype=torch.float64, device="cuda")
        for prec in (A.FP32, A.FP64):
            g = A.FrameworkEnergyGrid(ff, A.ParticleData.from_framework(fw), fw.lattice, guests[:1],
                                      SPACING, prec)
            g.interpolate_device(guests[0], xyz.data_ptr(), n, res.data_ptr(), 0)
            del g
    torch.cuda.synchronize()
    print(f"kernel case {case}: done")
    return 0


def c5_isotherm_sample(A, torch, moves=1000, n=64):
    """The large batched isotherm: the 4x4x4 triclinic supercell (27 008 charged
    atoms), 64 rigid-CO2 chains at pressures log-spaced over 0.01-50 bar in one
    launch, FP32 form, dispersion from the 0.2 A FP32 energy grid of the CO2
    site types, Ewald at 1e-6 (alpha and kMax from the rule, rc 12 A, FP64
    S(k) per chain), insertions from the learned proposal fitted on the
    supercell's own Widom trials. A bounded sample: `moves` moves per chain
    (the chains are not equilibrated); reported are the costs and the loadings
    reached."""
    from aleator_gb300 import workloads as W
    T = 298.0
    fw, guests = make_workload()
    alpha, kmax = W.ewald_parameters(fw.lattice, 12.0)
    ff = A.LennardJones(fw.eps, fw.sigma, CUTOFF, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    ew = A.Ewald(alpha, 12.0, kmax)
    guest = W.co2_guest(fw)

    def timed(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return r, time.perf_counter() - t0

    grid, t_grid = timed(lambda: A.FrameworkEnergyGrid(ff, p, fw.lattice, guests, SPACING, A.FP32))
    widom = A.Widom(ff, p, fw.lattice, guest, T, ewald=ew, precision=A.FP32)
    prop = A.Proposal(seed=2)
    _, t_fit = timed(lambda: prop.fit(widom, n_samples=1 << 16, rounds=2, epochs=15, cells=64))
    pressures = np.logspace(np.log10(0.01), np.log10(50.0), n)
    fugs = [A.peng_robinson_fugacity(*W.CO2_CRITICAL, T, P * 1e5) for P in pressures]
    ch, t_create = timed(lambda: A.GcmcChains(ff, p, fw.lattice, guest, T, fugs, list(range(n)),
                                              list(range(n)), ewald=ew, max_molecules=4000,
                                              precision=A.FP32))
    ch.set_grid(grid)
    ch.set_proposal(prop)
    _, t_run = timed(lambda: ch.run(moves))
    mol = [ch.molecules(c) for c in range(n)]
    terms = int(A.EwaldIncrementalState(ew, p, fw.lattice).term_count())
    return {"workload": f"4x4x4 triclinic supercell, {len(fw.x)} charged atoms, rigid CO2, {n} chains "
                        f"at 0.01-50 bar, Ewald kMax {kmax} ({terms} terms), 0.2 A FP32 grid, learned "
                        "proposal, FP32 form",
            "grid_build_s": t_grid, "proposal_fit_s": t_fit, "chains_create_s": t_create,
            "moves_per_chain": moves, "run_s": t_run,
            "us_per_move_per_chain": t_run / moves * 1e6,
            "chain_moves_per_s": n * moves / t_run,
            "molecules_after": {f"{P:.3g} bar": m for P, m in list(zip(pressures, mol))[::9]}}


def c5_isotherm(A, torch, seconds, n=64, block=2000):
    """The C5 isotherm itself: the 64 chains of c5_isotherm_sample (learned
    proposal, 0.2 A FP32 grid, kMax 34, FP32 form) run in blocks of `block`
    moves for `seconds` of wall time. Per pressure: the mean loading over the
    second half of the blocks and its standard error from the block means
    (blocks of 2000 moves; the chain is one replica per pressure), and the
    drift between the two quarters of that half (an equilibration check)."""
    from aleator_gb300 import workloads as W
    T = 298.0
    fw, guests = make_workload()
    alpha, kmax = W.ewald_parameters(fw.lattice, 12.0)
    ff = A.LennardJones(fw.eps, fw.sigma, CUTOFF, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    ew = A.Ewald(alpha, 12.0, kmax)
    guest = W.co2_guest(fw)
    grid = A.FrameworkEnergyGrid(ff, p, fw.lattice, guests, SPACING, A.FP32)
    widom = A.Widom(ff, p, fw.lattice, guest, T, ewald=ew, precision=A.FP32)
    prop = A.Proposal(seed=2)
    prop.fit(widom, n_samples=1 << 18, rounds=2, epochs=10, cells=64)
    pressures = np.logspace(np.log10(0.01), np.log10(50.0), n)
    fugs = [A.peng_robinson_fugacity(*W.CO2_CRITICAL, T, P * 1e5) for P in pressures]
    ch = A.GcmcChains(ff, p, fw.lattice, guest, T, fugs, list(range(n)), list(range(n)), ewald=ew,
                      max_molecules=8000, precision=A.FP32)
    ch.set_grid(grid)
    ch.set_proposal(prop)
    t0 = time.perf_counter()
    prev = np.array([ch.info(c)["sum_molecules"] for c in range(n)])
    means = []
    while time.perf_counter() - t0 < seconds:
        ch.run(block)
        cur = np.array([ch.info(c)["sum_molecules"] for c in range(n)])
        means.append((cur - prev) / block)
        prev = cur
    wall = time.perf_counter() - t0
    m = np.array(means)  # blocks x chains
    nb = len(m)
    half = m[nb // 2:]
    q1, q2 = half[:len(half) // 2], half[len(half) // 2:]
    V = abs(np.linalg.det(np.asarray(fw.lattice)))
    rows = []
    for c in range(n):
        mean = float(half[:, c].mean())
        se = float(half[:, c].std(ddof=1) / np.sqrt(len(half))) if len(half) > 1 else None
        rows.append({"bar": float(pressures[c]), "molecules": mean, "se": se,
                     "drift": float(q2[:, c].mean() - q1[:, c].mean()) if len(q1) else None,
                     "mmol_per_cm3": mean / V * 1e24 / 6.02214076e23 * 1e3})
    info = [ch.info(c) for c in range(n)]
    return {"workload": f"4x4x4 triclinic supercell, {fw.n_atoms} charged atoms, rigid CO2, {n} chains "
                        f"at 0.01-50 bar, Ewald kMax {kmax}, 0.2 A FP32 grid, learned proposal, FP32",
            "moves_per_chain": nb * block, "wall_s": wall,
            "us_per_move_per_chain": wall / (nb * block) * 1e6,
            "resyncs_max": int(max(i["resyncs"] for i in info)), "isotherm": rows}


def batched_screening(A, torch, n_frameworks=256, trials=1_000_000):
    """Batched screening: 256 uneven synthetic triclinic frameworks (a, b, c
    uniform in 10-40 A, angles in 60-120 deg, 50-2000 atoms, each replicated so
    the cutoff fits; 978k atoms in all), CH4 probe. Their 0.3 A FP32 grids are
    built in one persistent launch replayed from a CUDA graph (the
    first build autotunes the launch shape and captures), then Widom insertions
    for every framework in one persistent launch (FP32 pair terms, FP64
    accumulation), `trials` (1e6) per framework."""
    from aleator_gb300 import workloads as W
    t0 = time.perf_counter()
    fws = W.random_triclinic_frameworks(n_frameworks)
    gen_s = time.perf_counter() - t0
    ffs = [A.LennardJones(fw.eps, fw.sigma, CUTOFF, A.SHIFTED) for fw in fws]
    ps = [A.ParticleData.from_framework(fw) for fw in fws]
    lats = [fw.lattice for fw in fws]
    guests = [[fw.guest_species["CH4"]] for fw in fws]
    batch = A.GridBatch(ffs, ps, lats, guests, 0.3)
    batch.build()  # autotune + capture
    first = batch.stats()
    ms = []
    for _ in range(3):
        batch.build()
        ms.append(batch.stats()["last_ms"])
    st = batch.stats()
    grid_ms = float(np.median(ms))
    wb = A.WidomBatch(ffs, ps, lats, [W.ch4_guest(fw) for fw in fws], 298.0, precision=A.FP32)
    seeds, streams = [42] * n_frameworks, list(range(n_frameworks))
    wb.run(seeds, streams, trials)  # capture
    res = wb.run(seeds, streams, trials)
    w_ms = res[0]["kernel_ms"]
    atoms = sum(len(fw.x) for fw in fws)
    return {
        "workload": f"{n_frameworks} triclinic frameworks, {atoms} atoms, CH4, 0.3 A grids, "
                    f"{trials} Widom trials each (FP32)",
        "generate_s": gen_s,
        "grid": {"nodes": st["nodes"], "ms": grid_ms,
                 "pair_evals_per_s": st["algorithmic_pairs"] / (grid_ms * 1e-3),
                 "executed_pairs": st["executed_pairs"], "graph_launches": st["graph_launches"],
                 "autotuned_variant": first["variant"], "autotune_ms": first["tune_ms"],
                 "variants": "0: 3 sweep blocks/SM, 1: 4 sweep blocks/SM"},
        "widom": {"trials": trials * n_frameworks, "ms": w_ms,
                  "trials_per_s": trials * n_frameworks / (w_ms * 1e-3),
                  "pair_evals_per_s": trials * atoms / (w_ms * 1e-3),
                  "median_rel_std_error": float(np.median([r["rel_std_error"] for r in res]))},
    }


def extras(A, torch, peaks):
    """Secondary measurements of the other hot-path kernels (not the headline)."""
    from aleator_gb300 import workloads as W
    out = {}
    # 424-atom cubic cell, 52^3 grid at 0.5 Å, CH4 (the CPU-runnable configuration)
    fw = W.cubic_framework()
    ff = A.LennardJones(fw.eps, fw.sigma, 12.8, A.SHIFTED)
    p = A.ParticleData.from_framework(fw)
    for prec, name in ((A.FP64, "fp64"), (A.FP32, "fp32")):
        g = A.FrameworkEnergyGrid(ff, p, fw.lattice, [fw.guest_species["CH4"]], 0.5, prec)
        ms = []
        for _ in range(5):
            g.rebuild(0)
            ms.append(g.stats()["last_kernel_ms"])
        st = g.stats()
        out[f"grid_424atoms_52cube_{name}_pair_evals_per_s"] = st["algorithmic_pairs"] / (min(ms) * 1e-3)
    # Widom, CH4 and charged CO2 (kMax 10 from the 1e-6 rule), FP64
    alpha, kmax = W.ewald_parameters(fw.lattice, 12.0)
    fwq = W.cubic_framework(charged=True)
    pq = A.ParticleData.from_framework(fwq)
    w = A.Widom(ff, p, fw.lattice, W.ch4_guest(fw), 298.0)
    w.run(42, 0, 10000)
    r = w.run(42, 0, 1_000_000)
    out["widom_ch4_trials_per_s"] = 1_000_000 / (r["kernel_ms"] * 1e-3)
    wq = A.Widom(ff, pq, fwq.lattice, W.co2_guest(fwq), 298.0, ewald=A.Ewald(alpha, 12.0, kmax))
    wq.run(42, 0, 2000)
    r = wq.run(42, 0, 100_000)
    out["widom_co2_kmax10_trials_per_s"] = 100_000 / (r["kernel_ms"] * 1e-3)
    out["widom_co2_kmax10_terms"] = int(A.EwaldIncrementalState(A.Ewald(alpha, 12.0, kmax), pq,
                                                                fwq.lattice).term_count())
    # trilinear interpolation (HBM-bound gather) on the 0.2 Å supercell grid
    big, guests = make_workload()
    gi = A.FrameworkEnergyGrid(A.LennardJones(big.eps, big.sigma, CUTOFF, A.SHIFTED),
                               A.ParticleData.from_framework(big), big.lattice, guests[:1],
                               SPACING, A.FP32)
    n = 64 * 1024 * 1024
    u = torch.rand(n, 3, dtype=torch.float64, device="cuda")
    xyz = (u @ torch.tensor(big.lattice, device="cuda")).contiguous()
    res = torch.empty(n, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream()
    for _ in range(3):
        gi.interpolate_device(guests[0], xyz.data_ptr(), n, res.data_ptr(), s.cuda_stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(s)
    gi.interpolate_device(guests[0], xyz.data_ptr(), n, res.data_ptr(), s.cuda_stream)
    e1.record(s)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    algo_bytes = n * (24 + 8 * 8 + 8)
    gbs = algo_bytes / (ms * 1e-3) / 1e9
    out["interpolate_queries_per_s"] = n / (ms * 1e-3)
    out["batched_screening"] = batched_screening(A, torch)
    out["c5_isotherm_sample"] = c5_isotherm_sample(A, torch)
    out["interpolate_roofline"] = {
        "bound": "hbm", "achieved": gbs, "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
        "frac": gbs / peaks["hbm_gbs"] if peaks.get("hbm_gbs") else None, "bytes_per_query": 96,
        "note": "96 algorithmic bytes per query (8 corner loads of 8 B + 24 B in + 8 B out), random "
                "queries over a 0.7 GB table of an FP32-form grid, against the HBM copy peak. The "
                "transform and lerps run in double-float on the FP32 pipe (operands split by integer "
                "operations); each query reads its eight corners as one aligned 64-byte block of a "
                "per-node corner copy (made on the first interpolation after a build), so the "
                "kernel is bound by random 64-byte DRAM reads. The FP64-form grids keep the "
                "reference's FP64 arithmetic (3 IEEE divisions) for bit-equal values"}
    return out


if __name__ == "__main__":
    sys.exit(main())
