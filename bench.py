"""Benchmark of the GB300 self-gravity engine.

Headline workload (one JSON line on rank 0): LBVH Barnes-Hut KDK steps on a
1,000,000-particle exponential stellar disk (M = 5e10 Msun, Rd = 3 kpc,
sech^2 z0 = 0.3 kpc, 10% dispersion, seed 0, galactic units), theta = 0.5,
eps = 0.05 kpc, 30-bit Morton keys, dt = 1e-4.  A step is one full KDK step:
fused kick+drift, bounding box, keys, radix sort, Karras build, bottom-up
summaries, traversal with the closing kick.  Metric: particle-steps/s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb|reference]

Timing: W untimed steps, then K steps; each step is bracketed by CUDA events
on the launching stream, and a 512 MiB memset between steps (outside the
events) flushes the 129 MB L2.  Under torchrun every rank runs an
independent replica (the tree build is global: replicas only) and the
slowest rank's time sets the aggregate.  Secondary results (direct N^2
Plummer, FP32/Kahan/FP64 precision on a two-Plummer merger, batching,
adjoint) run on rank 0 at N = 1 and are reported under "secondary".
"""
from __future__ import annotations

import argparse
import ctypes
import hashlib
import importlib
import json
import os
import re
import subprocess
import sys
import tempfile
import time

import numpy as np
import torch

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
PKG = "real-astronomy-simulation_gb300"

BH_N = 1_000_000
BH_THETA = 0.5
BH_EPS = 0.05
BH_BITS = 10
BH_DT = 1e-4
FLUSH_BYTES = 512 << 20
METRIC = "BH particle-steps/s (LBVH theta=0.5, 1M exponential disk, KDK step)"


# ---------------------------------------------------------------- helpers
def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _git_blob(path: str) -> str:
    """git's blob hash of a file (sha1 of "blob <size>\\0" + content), so a
    profile note can name the exact kernel source it measured."""
    with open(path, "rb") as f:
        data = f.read()
    return hashlib.sha1(b"blob %d\0" % len(data) + data).hexdigest()


def _profile_current(summary: str, source: str) -> bool:
    """True when profiles/<summary> records the git blob hash of the kernel
    source it measured and that hash is the current file's."""
    try:
        with open(os.path.join(ROOT, "profiles", summary)) as f:
            txt = f.read()
    except OSError:
        return False
    m = re.search(r"git blob `([0-9a-f]{40})`", txt)
    return bool(m) and m.group(1) == _git_blob(os.path.join(ROOT, PKG, "csrc", source))


def _profiled_traffic(summary: str):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum)
    of the ncu capture summarised in profiles/<summary>, taken on the same
    workload as the bench line; None when the summary is absent."""
    try:
        with open(os.path.join(ROOT, "profiles", summary)) as f:
            txt = f.read()
    except OSError:
        return None
    m = re.search(r"traffic per launch[^|]*\|\s*([0-9]+) bytes", txt)
    return int(m.group(1)) if m else None


def _profiled_metric(summary: str, metric: str):
    """One metric's value from the table of the ncu summary in
    profiles/<summary>; None when absent."""
    try:
        with open(os.path.join(ROOT, "profiles", summary)) as f:
            txt = f.read()
    except OSError:
        return None
    m = re.search(r"`" + re.escape(metric) + r"`\s*\|\s*([0-9.]+)", txt)
    return float(m.group(1)) if m else None


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                    power.append(float(parts[3]))
                except ValueError:
                    continue
                for nm, val in zip(names, parts[5:9]):
                    if val.lower().startswith("active"):
                        reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)),
                "power_w_max": float(max(power)), "samples": len(sm),
                "reasons": sorted(reasons)}


def max_over_ranks(value: float, dist, device) -> float:
    """The slowest rank's time (all ranks get it); identity without a
    process group."""
    if not dist:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _events(k):
    return ([torch.cuda.Event(enable_timing=True) for _ in range(k)],
            [torch.cuda.Event(enable_timing=True) for _ in range(k)])


def _f32(a):
    return np.asarray(a, np.float64).astype(np.float32).astype(np.float64)


def _xm(pos, mass, dev):
    return torch.tensor(np.column_stack((pos, mass)), dtype=torch.float32, device=dev)


def _v4(vel, dev):
    v = torch.zeros((vel.shape[0], 4), dtype=torch.float32, device=dev)
    v[:, :3] = torch.tensor(vel, dtype=torch.float32)
    return v


def _rel_stats(a, ref):
    rel = np.linalg.norm(a - ref, axis=1) / np.maximum(np.linalg.norm(ref, axis=1), 1e-300)
    return {"rms": float(np.sqrt((rel ** 2).mean())), "max": float(rel.max()),
            "median": float(np.median(rel))}


def fp32_peak_tflops(lib_mod, dev):
    """Measured FP32 CUDA-core peak (best of scalar FFMA and packed FFMA2)."""
    buf = torch.zeros(1 << 16, device=dev)
    fl = ctypes.c_double()
    s = torch.cuda.current_stream().cuda_stream
    best = 0.0
    for packed in (0, 1):
        for _ in range(2):
            lib_mod.call("gb_calib_fp32", buf.data_ptr(), 2000, packed, ctypes.byref(fl), s)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(5):
            lib_mod.call("gb_calib_fp32", buf.data_ptr(), 2000, packed, ctypes.byref(fl), s)
        e1.record()
        torch.cuda.synchronize()
        best = max(best, fl.value * 5 / (e0.elapsed_time(e1) / 1e3) / 1e12)
    return best


# --------------------------------------------------------------- headline
def bench_bh(args, dev, rank, world, dist):
    ic = importlib.import_module(PKG + ".ic")
    bhmod = importlib.import_module(PKG + ".solvers.barnes_hut")
    units = importlib.import_module(PKG + ".units")
    pos, vel, mass = ic.exponential_disk(BH_N, seed=rank)
    xm, v4 = _xm(pos, mass, dev), _v4(vel, dev)
    a4 = torch.zeros_like(xm)
    bh = bhmod.BarnesHut(BH_N, theta=BH_THETA, softening=BH_EPS, key_bits=BH_BITS,
                         G=units.G, device=dev)
    bh.set_traversal(args.bh_traversal)
    bh.compute(xm, a4)
    for _ in range(args.warmup):
        bh.kdk(xm, v4, a4, BH_DT, 1)
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=dev)
    starts, ends = _events(args.steps)
    torch.cuda.synchronize()
    bh.diag(reset=True)
    bh.timing(True)
    bh.stage_times()
    launches0 = bh.launch_count()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(dev.index).start()
    for k in range(args.steps):
        flush.zero_()
        starts[k].record()
        bh.kdk(xm, v4, a4, BH_DT, 1)
        ends[k].record()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    launches = bh.launch_count() - launches0
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    stages, nst = bh.stage_times()
    bh.timing(False)
    diag = bh.diag(reset=True)
    total_ms = max_over_ranks(float(sum(step_ms)), dist, dev)
    value = world * BH_N * args.steps / (total_ms / 1e3)
    res = {"value": value, "ms_per_step": total_ms / args.steps, "clocks": clk,
           "gpu_launches": int(launches), "diag": diag,
           "stages_ms_per_step": {k: v / max(nst, 1) for k, v in stages.items()}}

    # Tree forces of the final state against FP64 direct sums on 4,096 seeded
    # targets (untimed).
    grav = importlib.import_module(PKG + ".solvers.gravity")
    targets = np.random.default_rng(1234).choice(BH_N, 4096, replace=False)
    ref = grav.acc_fp64_targets(xm, targets, units.G, BH_EPS * BH_EPS)
    got = a4[torch.as_tensor(targets, device=dev), :3].double().cpu().numpy()
    rel = np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)
    res["force_error_vs_fp64_direct"] = {"targets": 4096, "median": float(np.median(rel)),
                                         "p99": float(np.percentile(rel, 99)), "max": float(rel.max()),
                                         "rms": float(np.sqrt((rel ** 2).mean()))}

    # Work of one traversal, counted by an extra untimed evaluation with the
    # counting kernel variant on the final state of the timed steps.
    tmp = torch.zeros_like(a4)
    bh.compute(xm, tmp, count_work=True)
    per_step = {k: v for k, v in bh.diag(reset=True).items()
                if k in ("warp_node_reads", "warp_root_reads", "lane_interactions", "lane_tests")}
    del tmp
    # Roofline of the dominant kernel (traversal): algorithmic bytes per launch
    # = node records read per warp (48 B two-children record per expansion,
    # 32 B root record) + per particle: own leaf 16 B, order 4 B, velocity
    # 16 B read + 16 B write, acceleration 16 B write.
    trav_ms = res["stages_ms_per_step"]["traverse"]
    # The group walk (shape 3) also reads a 4 B group size per particle.
    bytes_launch = (48 * per_step["warp_node_reads"] + 32 * per_step["warp_root_reads"]
                    + BH_N * (16 + 4 + 16 + 16 + 16 + (4 if args.bh_traversal == 3 else 0)))
    hbm, src = _peaks()
    achieved = bytes_launch / (trav_ms / 1e3) / 1e9
    res["roofline"] = {"kernel": "bh_traverse_kernel", "bound": "hbm", "achieved": achieved,
                       "peak": hbm, "peak_source": f"{src} (MEASURED_PEAKS.json hbm_gbs)"
                       if src == "measured" else "fallback 6800 GB/s",
                       "unit": "GB/s", "frac": achieved / hbm, "traffic": None,
                       "algorithmic_bytes_per_launch": bytes_launch,
                       "launch_ms": trav_ms}
    traffic = _profiled_traffic("bh_traverse_1M_disk.md")
    if traffic is not None and not _profile_current("bh_traverse_1M_disk.md", "gb_bh_traverse.cuh"):
        # The capture measured another revision of the kernel source: its
        # figures are not this kernel's.
        res["roofline"]["traffic_source"] = ("none: profiles/bh_traverse_1M_disk.md was captured on "
                                             "another revision of csrc/gb_bh_traverse.cuh")
        traffic = None
    if traffic is not None and BH_N == 1_000_000 and BH_BITS == 10:
        res["roofline"]["traffic"] = traffic
        res["roofline"]["traffic_source"] = ("ncu dram bytes of one launch on this workload "
                                             "(profiles/bh_traverse_1M_disk.md)")
        # The kernel's actual limit is instruction issue, not HBM: the same
        # capture's issue-slot and pipe utilisation.
        res["roofline"]["observed_limit"] = {
            "issue_active_pct": _profiled_metric("bh_traverse_1M_disk.md",
                                                 "smsp__issue_active.avg.pct_of_peak_sustained_active"),
            "alu_pipe_pct": _profiled_metric("bh_traverse_1M_disk.md",
                                             "sm__pipe_alu_cycles_active.avg.pct_of_peak_sustained_active"),
            "fma_pipe_pct": _profiled_metric("bh_traverse_1M_disk.md",
                                             "sm__pipe_fma_cycles_active.avg.pct_of_peak_sustained_active"),
            "source": "ncu --set full capture of one launch (profiles/bh_traverse_1M_disk.md)"}
    # The same launch seen as FP32 work: 20 flop per monopole term, 10 per
    # acceptance test.
    flops = 20 * per_step["lane_interactions"] + 10 * per_step["lane_tests"]
    res["work_per_step"] = per_step
    res["traverse_fp32_tflops"] = flops / (trav_ms / 1e3) / 1e12

    # e2e: the same step through the C ABI with host buffers; pinned host
    # state is copied in before and read back after every step.
    hx = xm.detach().cpu().pin_memory()
    hv = v4.detach().cpu().pin_memory()
    ha = a4.detach().cpu().pin_memory()
    e_s, e_e = _events(args.steps)
    torch.cuda.synchronize()
    for k in range(args.steps):
        flush.zero_()
        e_s[k].record()
        xm.copy_(hx, non_blocking=True)
        v4.copy_(hv, non_blocking=True)
        a4.copy_(ha, non_blocking=True)
        bh.kdk(xm, v4, a4, BH_DT, 1)
        hx.copy_(xm, non_blocking=True)
        hv.copy_(v4, non_blocking=True)
        ha.copy_(a4, non_blocking=True)
        e_e[k].record()
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(float(sum(s.elapsed_time(e) for s, e in zip(e_s, e_e))), dist, dev)
    nbytes = 3 * BH_N * 16
    res["e2e"] = {"value": world * BH_N * args.steps / (e2e_ms / 1e3),
                  "unit": "particle-steps/s", "h2d_bytes_per_step": nbytes,
                  "d2h_bytes_per_step": nbytes,
                  "path": "gb_bh_kdk via the C ABI, pinned host state copied in/out each step"}

    # energies() right after a step (untimed for the headline): wall clock of
    # one step, of one step whose traversal also writes the tree potential,
    # and of that step plus the FP64 energy reductions read back to the host.
    phi = torch.zeros(BH_N, dtype=torch.float32, device=dev)

    def wall(fn, reps=20):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / reps * 1e3

    sync = torch.cuda.synchronize
    t_step = wall(lambda: (bh.kdk(xm, v4, a4, BH_DT, 1), sync()))
    t_phi = wall(lambda: (bh.kdk(xm, v4, a4, BH_DT, 1, phi=phi), sync()))
    t_e = wall(lambda: (bh.kdk(xm, v4, a4, BH_DT, 1, phi=phi), bh.energies_from_phi(xm, v4, phi)))
    res["energies_after_step"] = {
        "step_ms": t_step, "step_with_tree_potential_ms": t_phi,
        "tree_potential_over_step": (t_phi - t_step) / t_step,
        "energies_ms": t_e - t_phi, "energies_over_step": (t_e - t_phi) / t_phi,
        "note": "wall clock per call at N=1M, each waited for: gb_bh_kdk; gb_bh_kdk_phi (the step also "
                "writes the tree potential); gb_bh_kdk_phi + gb_bh_energy read back to the host"}
    bh.close()
    if args.bh_traversal == 3:
        res["roofline"].update(kernel="bh_group_kernel", traffic=None,
                               traffic_source="none: the headline ran the group walk")
        res["roofline"].pop("observed_limit", None)
    if not args.no_secondary and args.bh_traversal != 3:
        res["group_walk"] = bench_group_walk(args, dev, rank, world, dist, flush, hbm, src)
    return res


def bench_group_walk(args, dev, rank, world, dist, flush, hbm, src):
    """The opt-in group walk (traversal shape 3) on the same workload and
    initial state as the headline: KDK step throughput (device and e2e),
    stage split, traversal roofline and force error against FP64 direct sums
    on the same 4,096 seeded targets at its own final state."""
    ic = importlib.import_module(PKG + ".ic")
    bhmod = importlib.import_module(PKG + ".solvers.barnes_hut")
    units = importlib.import_module(PKG + ".units")
    grav = importlib.import_module(PKG + ".solvers.gravity")
    pos, vel, mass = ic.exponential_disk(BH_N, seed=rank)
    xm, v4 = _xm(pos, mass, dev), _v4(vel, dev)
    a4 = torch.zeros_like(xm)
    bh = bhmod.BarnesHut(BH_N, theta=BH_THETA, softening=BH_EPS, key_bits=BH_BITS,
                         G=units.G, device=dev)
    bh.set_traversal(3)
    bh.compute(xm, a4)
    for _ in range(args.warmup):
        bh.kdk(xm, v4, a4, BH_DT, 1)
    starts, ends = _events(args.steps)
    torch.cuda.synchronize()
    bh.diag(reset=True)
    bh.timing(True)
    bh.stage_times()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    for k in range(args.steps):
        flush.zero_()
        starts[k].record()
        bh.kdk(xm, v4, a4, BH_DT, 1)
        ends[k].record()
    torch.cuda.synchronize()
    total_ms = max_over_ranks(float(sum(s.elapsed_time(e) for s, e in zip(starts, ends))), dist, dev)
    stages, nst = bh.stage_times()
    bh.timing(False)
    diag = bh.diag(reset=True)
    out = {"traversal": 3, "value": world * BH_N * args.steps / (total_ms / 1e3),
           "unit": "particle-steps/s", "ms_per_step": total_ms / args.steps,
           "stages_ms_per_step": {k: v / max(nst, 1) for k, v in stages.items()},
           "diag": {k: diag[k] for k in ("stack_overflow", "nonfinite", "bad_tree")}}
    targets = np.random.default_rng(1234).choice(BH_N, 4096, replace=False)
    ref = grav.acc_fp64_targets(xm, targets, units.G, BH_EPS * BH_EPS)
    got = a4[torch.as_tensor(targets, device=dev), :3].double().cpu().numpy()
    rel = np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)
    out["force_error_vs_fp64_direct"] = {"targets": 4096, "median": float(np.median(rel)),
                                         "p99": float(np.percentile(rel, 99)), "max": float(rel.max()),
                                         "rms": float(np.sqrt((rel ** 2).mean()))}
    # Traversal roofline: node records read (48 B each, one per lane per
    # popped internal node; 32 B root record per group) + per particle own
    # leaf 16 B, order 4 B, group size 4 B, velocity 16 B read + 16 B write,
    # acceleration 16 B write.
    tmp = torch.zeros_like(a4)
    bh.compute(xm, tmp, count_work=True)
    work = bh.diag(reset=True)
    del tmp
    trav_ms = out["stages_ms_per_step"]["traverse"]
    bytes_launch = (48 * work["warp_node_reads"] + 32 * work["warp_root_reads"]
                    + BH_N * (16 + 4 + 4 + 16 + 16 + 16))
    achieved = bytes_launch / (trav_ms / 1e3) / 1e9
    out["roofline"] = {"kernel": "bh_group_kernel", "bound": "hbm", "achieved": achieved, "peak": hbm,
                       "peak_source": f"{src} (MEASURED_PEAKS.json hbm_gbs)" if src == "measured"
                       else "fallback 6800 GB/s", "unit": "GB/s", "frac": achieved / hbm,
                       "algorithmic_bytes_per_launch": bytes_launch, "launch_ms": trav_ms, "traffic": None}
    note = "bh_group_walk_1M_disk.md"
    if BH_N == 1_000_000 and BH_BITS == 10 and _profile_current(note, "gb_bh_traverse.cuh"):
        out["roofline"]["traffic"] = _profiled_traffic(note)
        out["roofline"]["traffic_source"] = f"ncu dram bytes of one launch on this workload (profiles/{note})"
    else:
        out["roofline"]["traffic_source"] = f"none: profiles/{note} was captured on another revision of csrc/gb_bh_traverse.cuh"
    # FP32 work: 20 flop per monopole term (list entry x target), 10 per
    # box-acceptance test (two per record).
    out["work_per_step"] = {"node_reads": work["warp_node_reads"], "groups": work["warp_root_reads"],
                            "interactions": work["lane_interactions"], "tests": work["lane_tests"]}
    out["traverse_fp32_tflops"] = (20 * work["lane_interactions"] + 10 * work["lane_tests"]) / (trav_ms / 1e3) / 1e12
    # e2e through the C ABI with host buffers, as the headline's.
    hx, hv, ha = (t_.detach().cpu().pin_memory() for t_ in (xm, v4, a4))
    e_s, e_e = _events(args.steps)
    torch.cuda.synchronize()
    for k in range(args.steps):
        flush.zero_()
        e_s[k].record()
        xm.copy_(hx, non_blocking=True)
        v4.copy_(hv, non_blocking=True)
        a4.copy_(ha, non_blocking=True)
        bh.kdk(xm, v4, a4, BH_DT, 1)
        hx.copy_(xm, non_blocking=True)
        hv.copy_(v4, non_blocking=True)
        ha.copy_(a4, non_blocking=True)
        e_e[k].record()
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(float(sum(s.elapsed_time(e) for s, e in zip(e_s, e_e))), dist, dev)
    nbytes = 3 * BH_N * 16
    out["e2e"] = {"value": world * BH_N * args.steps / (e2e_ms / 1e3), "unit": "particle-steps/s",
                  "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                  "path": "gb_bh_kdk (traversal 3) via the C ABI, pinned host state copied in/out each step"}
    bh.close()
    return out


# ------------------------------------------------------------ CPU oracle
def cpu_bh_step(budget_s: float = 20.0):
    """One KDK step of the same workload with the float64 oracle (OpenMP, all
    host threads): tree build over all particles, traversal of a seeded
    target sample sized to the budget, scaled to the full particle count."""
    from oracle import oracle

    ic = importlib.import_module(PKG + ".ic")
    units = importlib.import_module(PKG + ".units")
    pos, vel, mass = ic.exponential_disk(BH_N, seed=0)
    pos, vel, mass = _f32(pos), _f32(vel), _f32(mass)
    acc = np.zeros_like(pos)
    oracle.build()
    rng = np.random.default_rng(0)
    probe = rng.choice(BH_N, 20000, replace=False)
    t0 = time.perf_counter()
    tree = oracle.bh_tree(pos, mass, bits=BH_BITS)
    t_build = time.perf_counter() - t0
    t0 = time.perf_counter()
    oracle.traverse(pos, tree["order"], tree["com"], tree["nmass"], tree["nmin"], tree["nmax"],
                    tree["left"], tree["right"], BH_THETA, BH_EPS ** 2, units.G, targets=probe)
    per_target = (time.perf_counter() - t0) / probe.size
    sample = int(min(BH_N, max(20000, (budget_s - t_build) / max(per_target, 1e-9))))
    targets = np.sort(rng.choice(BH_N, sample, replace=False)) if sample < BH_N else None
    t0 = time.perf_counter()
    vh = vel + acc * (0.5 * BH_DT)
    p1 = pos + vh * BH_DT
    t_kick = time.perf_counter() - t0
    t0 = time.perf_counter()
    tree = oracle.bh_tree(p1, mass, bits=BH_BITS)
    t_build = time.perf_counter() - t0
    t0 = time.perf_counter()
    a1, _ = oracle.traverse(p1, tree["order"], tree["com"], tree["nmass"], tree["nmin"],
                            tree["nmax"], tree["left"], tree["right"], BH_THETA, BH_EPS ** 2,
                            units.G, targets=targets)
    t_trav = time.perf_counter() - t0
    nt = BH_N if targets is None else targets.size
    t_step = 2 * t_kick + t_build + t_trav * BH_N / nt
    return {"value": BH_N / t_step, "unit": "particle-steps/s", "cores": oracle.max_threads(),
            "kind": "port",
            "sample": (f"one KDK step: kick/drift and tree build over all {BH_N} particles, "
                       f"traversal of {nt} seeded targets scaled to {BH_N}"),
            "seconds": {"build": t_build, "traverse": t_trav, "kick": t_kick}}


def bench_sharded_bh(args, dev, rank, world, dist):
    """The tree path with the tree replicated and the targets split across
    the ranks (ShardedBarnesHut) on the headline workload: every rank kicks,
    drifts and builds the whole tree, walks its slice of the key order, and
    one all-reduce of the accelerations (16 B per particle) joins the slices.
    Total work fixed as ranks are added (strong scaling)."""
    sh = importlib.import_module(PKG + ".sharded")
    ic = importlib.import_module(PKG + ".ic")
    units = importlib.import_module(PKG + ".units")
    pos, vel, mass = ic.exponential_disk(BH_N, seed=0)
    s = sh.ShardedBarnesHut(pos, vel, mass, theta=BH_THETA, softening=BH_EPS, G=units.G, key_bits=BH_BITS,
                            device=dev)
    s.run(BH_DT, args.warmup)
    steps = max(1, args.steps)
    st, en = _events(1)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    st[0].record()
    s.run(BH_DT, steps)
    en[0].record()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms = max_over_ranks(st[0].elapsed_time(en[0]), dist, dev)
    s.close()
    return {"workload": f"LBVH Barnes-Hut KDK, exponential disk N={BH_N}, theta {BH_THETA}, replicated tree, "
                        f"key-order targets split over {world} rank(s)",
            "value": BH_N * steps / (ms / 1e3), "unit": "particle-steps/s", "n_ranks": world,
            "scaling": "strong", "ms_per_step": ms / steps, "steps": steps,
            "allreduce_bytes_per_step": 16 * BH_N,
            "path": "ShardedBarnesHut: gb_kick/gb_drift, gb_bh_build, gb_bh_accel_range, all-reduce, gb_kick"}


# ------------------------------------------------------------- secondary
def bench_sharded_direct(args, dev, rank, world, dist, n=262_144, dt=5e-4):
    """Direct N^2 with the targets split across the ranks (ShardedDirect):
    one Plummer sphere of n = 262,144 (G = 1, eps = 0.01), each step one
    all-gather of the 16 B position records and a range force pass per
    rank.  Total work is fixed as ranks are added (strong scaling)."""
    sh = importlib.import_module(PKG + ".sharded")
    ic = importlib.import_module(PKG + ".ic")
    pos, vel, mass = ic.plummer(n, seed=0)
    s = sh.ShardedDirect(pos, vel, mass, G=1.0, softening=0.01, device=dev)
    s.run(dt, args.warmup)
    steps = max(1, args.steps)
    st, en = _events(1)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    st[0].record()
    s.run(dt, steps)
    en[0].record()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms = max_over_ranks(st[0].elapsed_time(en[0]), dist, dev)
    s.close()
    return {"workload": f"direct N^2 Plummer N={n}, G=1, eps=0.01, dt={dt}, targets split over {world} rank(s)",
            "value": n * n * steps / (ms / 1e3) / 1e9, "unit": "G interactions/s", "n_ranks": world,
            "scaling": "strong", "ms_per_step": ms / steps, "steps": steps,
            "allgather_bytes_per_step": 16 * n,
            "path": "ShardedDirect: gb_kick/gb_drift on the own slice, all-gather, gb_direct_acc_range"}


# FP32 work of one unordered pair in the symmetric pass, FMA = 2 flop: 3 sub,
# 3 FMA for |d|^2 + eps^2, 2 mul for rsqrt^3, 2 mul for the two mass
# factors, 6 FMA for the two sides' sums (the rsqrt is on the MUFU pipe).
SYM_PAIR_FLOP = 3 + 6 + 2 + 2 + 12


def cpu_direct_step(n=20000, budget_s=10.0):
    """One direct-sum KDK step of the Plummer workload (N = 20,000, G = 1,
    eps = 0.01) with the float64 oracle (OpenMP over all host threads): the
    force sum of a seeded target sample sized to the budget, scaled to all
    N targets; the kick/drift halves are O(N) and timed on all particles."""
    from oracle import oracle

    ic = importlib.import_module(PKG + ".ic")
    pos, vel, mass = ic.plummer(n, seed=0)
    pos, vel, mass = _f32(pos), _f32(vel), _f32(mass)
    oracle.build()
    rng = np.random.default_rng(0)
    probe = rng.choice(n, 500, replace=False)
    t0 = time.perf_counter()
    oracle.direct_acc(pos, mass, 1.0, 1e-4, probe)
    per_target = (time.perf_counter() - t0) / probe.size
    sample = int(min(n, max(500, budget_s / max(per_target, 1e-9))))
    targets = np.sort(rng.choice(n, sample, replace=False))
    acc = np.zeros_like(pos)
    t0 = time.perf_counter()
    vh = vel + acc * 5e-4
    p1 = pos + vh * 1e-3
    t_kick = time.perf_counter() - t0
    t0 = time.perf_counter()
    oracle.direct_acc(p1, mass, 1.0, 1e-4, targets)
    t_force = time.perf_counter() - t0
    t_step = 2 * t_kick + t_force * n / sample
    return {"value": n * n / t_step / 1e9, "unit": "G interactions/s", "cores": oracle.max_threads(),
            "kind": "port", "ms_per_step": t_step * 1e3,
            "sample": (f"one KDK step of the N={n} Plummer workload: kick/drift over all particles, "
                       f"force sum of {sample} seeded targets over all {n} sources scaled to {n} targets")}


def bench_direct(dev, lib_mod, peak_tflops, cpu=True):
    """Direct N^2 Plummer, N = 20,000, G = 1, eps = 0.01, dt = 1e-3, 100 KDK
    steps through the Engine (symmetric pass); the same step through the C
    ABI with host buffers (e2e); energies() right after a step; the CPU
    baseline; plus the per-target force kernel's own FP32 fraction at
    N = 20k and 262k, and the symmetric pass at the same sizes."""
    pkg = importlib.import_module(PKG)
    ic = importlib.import_module(PKG + ".ic")
    grav = importlib.import_module(PKG + ".solvers.gravity")
    n, steps = 20000, 100
    pos, vel, mass = ic.plummer(n, seed=0)
    pos, vel, mass = _f32(pos), _f32(vel), _f32(mass)
    eng = pkg.Engine(softening=0.01, G=1.0, device=dev)
    eng.load_state(pkg.State.from_arrays(pos, vel, mass))
    targets = np.random.default_rng(0).choice(n, 2048, replace=False)
    ref = grav.acc_fp64_targets(eng.xm, targets, 1.0, 1e-4)
    err = _rel_stats(eng.acc.to_numpy()[targets], ref)
    eng.run(1e-3, 3)
    eng.load_state(pkg.State.from_arrays(pos, vel, mass))
    e0 = eng.energies()
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    eng.run(1e-3, steps)
    e.record()
    torch.cuda.synchronize()
    t = s.elapsed_time(e) / 1e3
    e1 = eng.energies()
    gint = n * n * steps / t / 1e9
    out = {"workload": "direct N^2 Plummer N=20000, G=1, eps=0.01, dt=1e-3, 100 KDK steps",
           "gint_per_s": gint, "ms_per_step": t / steps * 1e3,
           # Delivered interactions (N^2 per step) x 20 flop over the
           # measured FP32 peak: a throughput; the symmetric pass evaluates
           # N^2 / 2 pairs to deliver them.
           "delivered_20flop_rate_over_fp32_peak": gint * 20 / 1e3 / peak_tflops,
           "energy_drift": abs((e1[2] - e0[2]) / e0[2]), "acc_err_vs_fp64_2048_targets": err}

    # energies() right after a step (the reference's print cadence), wall
    # clock: the step alone, the step plus energies() from the potential the
    # step wrote, and the step plus an exact O(N^2) potential pass.
    def wall(fn, reps=50):
        fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / reps * 1e3

    sync = torch.cuda.synchronize

    def engine(fused):
        e_ = pkg.Engine(softening=0.01, G=1.0, fused_potential=fused, device=dev)
        e_.load_state(pkg.State.from_arrays(pos, vel, mass))
        return e_

    eng_plain, eng_fused, eng_auto = engine(False), engine(True), engine("auto")
    t_plain = wall(lambda: (eng_plain.step(1e-3), sync()))
    t_fused = wall(lambda: (eng_fused.step(1e-3), sync()))
    t_fused_e = wall(lambda: (eng_fused.step(1e-3), eng_fused.energies()))
    t_exact = wall(lambda: (eng_plain.step(1e-3), eng_plain.energies(exact=True)))

    def loop10(e_, energies):
        for _ in range(10):
            e_.step(1e-3)
        if energies:
            e_.energies()
        sync()

    t10_plain = wall(lambda: loop10(eng_plain, False), reps=10)
    t10_auto = wall(lambda: loop10(eng_auto, True), reps=10)
    out["energies_after_step"] = {
        "step_ms": t_plain, "step_writing_potential_ms": t_fused,
        "potential_over_step": (t_fused - t_plain) / t_plain,
        "energies_ms": t_fused_e - t_fused, "energies_over_step": (t_fused_e - t_fused) / t_plain,
        "energies_exact_pass_ms": t_exact - t_plain,
        "print_every_10_steps_overhead": (t10_auto - t10_plain) / t10_plain,
        "note": "wall clock per Engine.step(dt) call at N=20000, each waited for: without the potential, "
                "writing it (fused_potential=True), and followed by energies(); the last figure is 10 steps "
                "plus energies() with fused_potential='auto' against 10 plain steps"}

    # e2e: the KDK step through the C ABI with host buffers: pinned host
    # state copied in before and read back after every step.
    g = grav.DirectGravity(n, dev)
    g.set_variant(2)
    xm, v4 = _xm(pos, mass, dev), _v4(vel, dev)
    a4 = torch.zeros_like(xm)
    g.acc(xm, a4, 1.0, 1e-4)
    hx, hv, ha = (t_.detach().cpu().pin_memory() for t_ in (xm, v4, a4))
    reps = 50
    for _ in range(3):
        g.kdk(xm, v4, a4, 1.0, 1e-4, 1e-3, 1, graph=True)
    torch.cuda.synchronize()
    s.record()
    for _ in range(reps):
        xm.copy_(hx, non_blocking=True)
        v4.copy_(hv, non_blocking=True)
        a4.copy_(ha, non_blocking=True)
        g.kdk(xm, v4, a4, 1.0, 1e-4, 1e-3, 1, graph=True)
        hx.copy_(xm, non_blocking=True)
        hv.copy_(v4, non_blocking=True)
        ha.copy_(a4, non_blocking=True)
    e.record()
    torch.cuda.synchronize()
    te = s.elapsed_time(e) / reps / 1e3
    out["e2e"] = {"value": n * n / te / 1e9, "unit": "G interactions/s", "h2d_bytes_per_step": 3 * n * 16,
                  "d2h_bytes_per_step": 3 * n * 16, "ms_per_step": te * 1e3,
                  "path": "gb_direct_kdk (symmetric pass, graph replay) via the C ABI, pinned host state "
                          "copied in/out each step"}
    g.close()
    if cpu:
        out["cpu_baseline"] = cpu_direct_step(n)
        out["gpu_over_cpu"] = gint / out["cpu_baseline"]["value"]
        out["e2e_over_cpu"] = out["e2e"]["value"] / out["cpu_baseline"]["value"]

    kern = {}
    for nk in (20000, 262144):
        p2, _, m2 = ic.plummer(nk, seed=1)
        xm = _xm(p2, m2, dev)
        acc = torch.zeros_like(xm)
        g = grav.DirectGravity(nk, dev)
        for _ in range(3):
            g.acc(xm, acc, 1.0, 1e-4)
        reps = max(3, int(3e11 / nk / nk))
        s.record()
        for _ in range(reps):
            g.acc(xm, acc, 1.0, 1e-4)
        e.record()
        torch.cuda.synchronize()
        tk = s.elapsed_time(e) / reps / 1e3
        tf = 20.0 * nk * nk / tk / 1e12
        kern[str(nk)] = {"ms": tk * 1e3, "gint_per_s": nk * nk / tk / 1e9, "tflops_20flop": tf,
                         "frac_of_fp32_peak": tf / peak_tflops}
        # Symmetric variant (the Engine's default): N^2 / 2 pair evaluations.
        # gint_per_s counts the N^2 ordered interactions it delivers; the
        # achieved FLOP/s counts the FP32 work it executes per pair.
        g.set_variant(2)
        for _ in range(3):
            g.acc(xm, acc, 1.0, 1e-4)
        s.record()
        for _ in range(reps):
            g.acc(xm, acc, 1.0, 1e-4)
        e.record()
        torch.cuda.synchronize()
        ts = s.elapsed_time(e) / reps / 1e3
        achieved = SYM_PAIR_FLOP * nk * nk / 2 / ts / 1e12
        kern[str(nk)]["symmetric"] = {"ms": ts * 1e3, "gint_per_s": nk * nk / ts / 1e9,
                                      "delivered_20flop_rate_over_fp32_peak":
                                          20.0 * nk * nk / ts / 1e12 / peak_tflops,
                                      "achieved_fp32_tflops": achieved,
                                      "achieved_frac_of_fp32_peak": achieved / peak_tflops,
                                      "speedup_vs_per_target": tk / ts}
        g.close()
    out["force_kernel"] = kern
    return out


def bench_merger(dev, drift_steps=1000):
    """Precision: two Plummer spheres (2 x 131,072, G = 1, a = 1, M = 1) 10
    apart on a parabolic orbit, eps = 0.01.  FP32+Kahan (per-target and
    symmetric passes) vs plain FP32 vs FP64 on 8,192 targets; FP64 energy
    drift over Engine KDK steps (symmetric pass) at dt = 5e-4."""
    pkg = importlib.import_module(PKG)
    ic = importlib.import_module(PKG + ".ic")
    grav = importlib.import_module(PKG + ".solvers.gravity")
    pos, vel, mass = ic.plummer_pair(131072)
    pos, vel, mass = _f32(pos), _f32(vel), _f32(mass)
    n = pos.shape[0]
    xm = _xm(pos, mass, dev)
    targets = np.random.default_rng(0).choice(n, 8192, replace=False)
    ref = grav.acc_fp64_targets(xm, targets, 1.0, 1e-4)
    g = grav.DirectGravity(n, dev)
    acc = torch.zeros_like(xm)
    g.acc(xm, acc, 1.0, 1e-4)
    kahan = _rel_stats(acc[:, :3].double().cpu().numpy()[targets], ref)
    g.acc(xm, acc, 1.0, 1e-4, plain=True)
    plain = _rel_stats(acc[:, :3].double().cpu().numpy()[targets], ref)
    g.set_variant(2)  # the symmetric pass (the Engine's), Kahan-merged slots
    g.acc(xm, acc, 1.0, 1e-4)
    sym = _rel_stats(acc[:, :3].double().cpu().numpy()[targets], ref)
    g.close()
    eng = pkg.Engine(softening=0.01, G=1.0, device=dev)
    eng.load_state(pkg.State.from_arrays(pos, vel, mass))
    e0 = eng.energies()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    eng.run(5e-4, drift_steps)
    e.record()
    torch.cuda.synchronize()
    t = s.elapsed_time(e) / 1e3
    e1 = eng.energies()
    return {"workload": f"two-Plummer merger 2x131072, eps=0.01, dt=5e-4, {drift_steps} KDK steps",
            "impact_parameter": 2.0, "kahan_vs_fp64": kahan, "plain_fp32_vs_fp64": plain,
            "symmetric_kahan_vs_fp64": sym,
            "energy_drift": abs((e1[2] - e0[2]) / e0[2]), "E0": e0, "E1": e1,
            "gint_per_s": n * n * drift_steps / t / 1e9}


def bench_batch(dev, steps=200, loop_steps=20):
    """512 independent Plummer spheres (N_s = round(exp(U(ln 256, ln 16384))),
    seed s), G = 1, eps = 0.02, dt = 1e-3: 200 KDK steps as one persistent
    launch per step replayed from a CUDA graph, tile shape and force-pass
    form (per target or symmetric) from the autotuner; compared with the
    batched launches without the graph, with the other form, and with a loop
    over systems of the single-system kernel."""
    batch = importlib.import_module(PKG + ".batch")
    ic = importlib.import_module(PKG + ".ic")
    tune = importlib.import_module(PKG + ".autotune")
    systems = [(_f32(p), _f32(v), _f32(m)) for p, v, m in ic.plummer_batch(512)]
    b = batch.DirectBatch(systems, G=1.0, softening=0.02, device=dev)
    shape, tune_ms = tune.tune_batch(b, use_cache=False)
    inter = b.interactions_per_step()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        torch.cuda.synchronize()
        s.record()
        fn()
        e.record()
        torch.cuda.synchronize()
        return s.elapsed_time(e) / 1e3

    b.run(1e-3, steps, graph=True)  # capture + first replay (warm-up)
    saved = b.state_arrays()
    l0 = b.launch_count()
    t_graph = timed(lambda: b.run(1e-3, steps, graph=True))
    launches = b.launch_count() - l0
    b.restore(saved)
    t_plain = timed(lambda: b.run(1e-3, loop_steps, graph=False))
    # The other force-pass form, for comparison: best per-target tile shape
    # against the symmetric pass.
    per_target = min((k for k in tune_ms if k.endswith(",0")), key=tune_ms.get)
    forms = {}
    for v in (0, 1):
        if v == 0:
            kk, ww, _ = (int(x) for x in per_target.split(","))
            b.set_tiles(kk, ww)
        b.set_variant(v)
        b.restore(saved)
        b.run(1e-3, steps, graph=True)
        b.restore(saved)
        forms[v] = inter * steps / timed(lambda: b.run(1e-3, steps, graph=True)) / 1e9
    b.set_tiles(shape[0], shape[1])
    b.set_variant(shape[2])
    b.restore(saved)
    b.run_loop(1e-3, 2)
    b.restore(saved)
    t_loop = timed(lambda: b.run_loop(1e-3, loop_steps))
    out = {"workload": "512 Plummer spheres, N log-uniform in [256, 16384] (seed s), G=1, eps=0.02, "
                       f"dt=1e-3, {steps} KDK steps",
           "n_total": b.n_total, "interactions_per_step": inter, "tiles": list(shape),
           "autotune_ms_per_step": tune_ms,
           "graph_gint_per_s": inter * steps / t_graph / 1e9, "graph_ms_per_step": t_graph / steps * 1e3,
           "gpu_launches_graph": launches,
           "graph_gint_per_s_per_target_pass": forms[0], "graph_gint_per_s_symmetric_pass": forms[1],
           "batched_no_graph_gint_per_s": inter * loop_steps / t_plain / 1e9,
           "per_system_loop_gint_per_s": inter * loop_steps / t_loop / 1e9,
           "per_system_loop_ms_per_step": t_loop / loop_steps * 1e3}
    out["speedup_vs_loop"] = out["graph_gint_per_s"] / out["per_system_loop_gint_per_s"]
    b.close()
    return out


def bench_adjoint(dev, n=65536, steps=200, every=20):
    """Adjoint of 200 direct-sum KDK steps on a 65,536-particle exponential
    disk (Rd = 3, eps = 0.05, dt = 1e-3, galactic G), checkpoint every 20.
    Loss: MSE of the final positions against a target snapshot made with
    masses x lognormal(sigma = 0.05).  Reports forward and backward time per
    step (backward = segment recompute + adjoint kernels)."""
    adj = importlib.import_module(PKG + ".adjoint")
    ic = importlib.import_module(PKG + ".ic")
    grav = importlib.import_module(PKG + ".solvers.gravity")
    units = importlib.import_module(PKG + ".units")
    lib_mod = importlib.import_module(PKG + "._lib")
    p, v, m = ic.exponential_disk(n, seed=0)
    p, v, m = _f32(p), _f32(v), _f32(m)
    solver = grav.DirectGravity(n, dev)
    mt = m * np.random.default_rng(1).lognormal(0.0, 0.05, size=n)
    with torch.no_grad():
        xt, _ = adj.simulate(torch.tensor(p, device=dev, dtype=torch.float32),
                             torch.tensor(v, device=dev, dtype=torch.float32),
                             torch.tensor(mt, device=dev, dtype=torch.float32),
                             G=units.G, softening=0.05, dt=1e-3, nsteps=steps, solver=solver)
    target = xt.detach()
    # Warm-up: one short differentiable run (module loading and autograd
    # set-up happen on first use and are not part of a step).
    xw = torch.tensor(p, device=dev, dtype=torch.float32, requires_grad=True)
    xa, _ = adj.simulate(xw, torch.tensor(v, device=dev, dtype=torch.float32),
                         torch.tensor(m, device=dev, dtype=torch.float32), G=units.G, softening=0.05,
                         dt=1e-3, nsteps=2 * every, checkpoint_every=every, solver=solver)
    (xa ** 2).mean().backward()
    torch.cuda.synchronize()
    x0 = torch.tensor(p, device=dev, dtype=torch.float32, requires_grad=True)
    v0 = torch.tensor(v, device=dev, dtype=torch.float32, requires_grad=True)
    m0 = torch.tensor(m, device=dev, dtype=torch.float32, requires_grad=True)
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    s.record()
    xT, vT = adj.simulate(x0, v0, m0, G=units.G, softening=0.05, dt=1e-3, nsteps=steps,
                          checkpoint_every=every, solver=solver)
    e.record()
    torch.cuda.synchronize()
    t_fwd = s.elapsed_time(e) / 1e3
    loss = ((xT - target) ** 2).mean()
    torch.cuda.synchronize()
    s.record()
    loss.backward()
    e.record()
    torch.cuda.synchronize()
    t_bwd = s.elapsed_time(e) / 1e3
    # One adjoint step alone (no recompute) against one forward step.
    xm = torch.zeros((n, 4), device=dev)
    xm[:, :3] = x0.detach()
    xm[:, 3] = m0.detach()
    v4 = torch.zeros_like(xm)
    a4 = torch.zeros_like(xm)
    lx, lv, la = torch.ones_like(xm), torch.ones_like(xm), torch.ones_like(xm)
    lm = torch.zeros(n, device=dev)
    st = torch.cuda.current_stream().cuda_stream
    reps = 10

    lib_mod.call("gb_adjoint_set_variant", solver.handle, 2)

    def adj_step():
        lib_mod.call("gb_adjoint_step", solver.handle, xm.data_ptr(), lx.data_ptr(), lv.data_ptr(),
                     la.data_ptr(), lm.data_ptr(), n, units.G, 0.0025, 1e-3, 0, st)

    adj_step()
    solver.kdk(xm.clone(), v4, a4, units.G, 0.0025, 1e-3, 1)
    xs = xm.clone()
    s.record()
    for _ in range(reps):
        solver.kdk(xs, v4, a4, units.G, 0.0025, 1e-3, 1)
    e.record()
    torch.cuda.synchronize()
    t_f1 = s.elapsed_time(e) / reps
    solver.set_variant(2)  # the symmetric force pass, for comparison
    solver.kdk(xs, v4, a4, units.G, 0.0025, 1e-3, 1)
    s.record()
    for _ in range(reps):
        solver.kdk(xs, v4, a4, units.G, 0.0025, 1e-3, 1)
    e.record()
    torch.cuda.synchronize()
    t_f1s = s.elapsed_time(e) / reps
    solver.set_variant(0)
    s.record()
    for _ in range(reps):
        adj_step()
    e.record()
    torch.cuda.synchronize()
    t_b1 = s.elapsed_time(e) / reps
    g = [t.grad for t in (x0, v0, m0)]

    def backward_time(symmetric, packed):
        """The same backward with another pair evaluation, for comparison."""
        x1 = x0.detach().clone().requires_grad_(True)
        xT1, _ = adj.simulate(x1, v0.detach(), m0.detach(), G=units.G, softening=0.05, dt=1e-3,
                              nsteps=steps, checkpoint_every=every, solver=solver, symmetric=symmetric,
                              packed=packed)
        loss1 = ((xT1 - target) ** 2).mean()
        torch.cuda.synchronize()
        s.record()
        loss1.backward()
        e.record()
        torch.cuda.synchronize()
        return s.elapsed_time(e) / 1e3

    t_bwd_pt = backward_time(False, True)
    t_bwd_sc = backward_time(True, False)
    lib_mod.call("gb_adjoint_set_variant", solver.handle, 2)
    # The same run with the symmetric force pass in the forward steps and the
    # backward's segment recompute.
    solver.set_variant(2)
    xs0 = x0.detach().clone().requires_grad_(True)
    torch.cuda.synchronize()
    s.record()
    xTs, _ = adj.simulate(xs0, v0.detach(), m0.detach(), G=units.G, softening=0.05, dt=1e-3,
                          nsteps=steps, checkpoint_every=every, solver=solver)
    e.record()
    torch.cuda.synchronize()
    t_fwd_s = s.elapsed_time(e) / 1e3
    loss_s = ((xTs - target) ** 2).mean()
    torch.cuda.synchronize()
    s.record()
    loss_s.backward()
    e.record()
    torch.cuda.synchronize()
    t_bwd_s = s.elapsed_time(e) / 1e3
    solver.set_variant(0)
    return {"workload": f"adjoint of {steps} KDK steps, exponential disk N={n}, eps=0.05, dt=1e-3, "
                        f"checkpoint every {every}; loss = MSE of final positions",
            "forward_ms_per_step": t_fwd / steps * 1e3, "backward_ms_per_step": t_bwd / steps * 1e3,
            "backward_over_forward": t_bwd / t_fwd,
            "backward_over_forward_per_target_form": t_bwd_pt / t_fwd,
            "backward_over_forward_scalar_symmetric_form": t_bwd_sc / t_fwd,
            "adjoint_kernel_over_force_step": t_b1 / t_f1,
            "adjoint_kernel_over_symmetric_force_step": t_b1 / t_f1s,
            "with_symmetric_force_pass": {"forward_ms_per_step": t_fwd_s / steps * 1e3,
                                          "backward_ms_per_step": t_bwd_s / steps * 1e3,
                                          "backward_over_forward": t_bwd_s / t_fwd_s},
            "loss": float(loss.detach()),
            "grad_finite": bool(all(torch.isfinite(t).all().item() for t in g))}


def bench_grid(dev, n=1_000_000, reps=20):
    """SPH neighbour-grid rebuild (NeighborGrid.rebuild) of a 1M exponential
    disk with 30% stars: device rebuild alone (CUDA events, L2 flushed), the
    call with its gas-count readback, and the oracle's C restatement on one
    host core (the reference's rebuild is host numpy)."""
    ic = importlib.import_module(PKG + ".ic")
    ngm = importlib.import_module(PKG + ".solvers.neighbor_grid")
    pos, _, mass = ic.exponential_disk(n, seed=5)
    rng = np.random.default_rng(6)
    h = rng.lognormal(np.log(0.05), 0.5, n).astype(np.float32)
    star = (rng.random(n) < 0.3).astype(np.int32)
    xm = _xm(pos, mass, dev)
    hs = torch.tensor(h, device=dev)
    st = torch.tensor(star, device=dev)
    grid = ngm.NeighborGrid(n, min_radius=0.02, device=dev)
    for _ in range(3):
        ngas = grid.rebuild(xm, hs, st)
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device=dev)
    starts, ends = _events(reps)
    l0 = grid.launch_count()
    for k in range(reps):
        flush.zero_()
        starts[k].record()
        grid.rebuild_async(xm, hs, st)
        ends[k].record()
    torch.cuda.synchronize()
    launches = (grid.launch_count() - l0) // reps
    dev_ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends)) / reps
    t0 = time.perf_counter()
    for _ in range(reps):
        grid.rebuild(xm, hs, st)
    sync_ms = (time.perf_counter() - t0) / reps * 1e3
    from oracle import oracle as orc
    orc.build()
    pos64 = pos.astype(np.float32).astype(np.float64)
    t0 = time.perf_counter()
    ref = orc.grid_rebuild(pos64, h.astype(np.float64), star, 0.02)
    cpu_ms = (time.perf_counter() - t0) * 1e3
    same = bool(ref["ngas"] == ngas and np.array_equal(ref["gsort"], grid.gsort.cpu().numpy())
                and np.array_equal(ref["cell_start"], grid.cell_start.cpu().numpy()))
    grid.close()
    return {"workload": f"NeighborGrid.rebuild, exponential disk N={n}, 30% stars, h lognormal(0.05, 0.5), "
                        "min_radius 0.02", "ngas": int(ngas), "dims": [grid.nx, grid.ny, grid.nz],
            "rebuild_ms": dev_ms, "rebuild_with_gas_count_readback_ms": sync_ms,
            "launches_per_rebuild": int(launches),
            "cpu_port_ms": cpu_ms, "cpu_port": "oracle C restatement, 1 host core",
            "identical_to_oracle": same}


def bench_snapshot(dev, n=1_000_000, steps=100, every=20):
    """Snapshot cost in the step loop: the 1M-disk BH engine runs `steps`
    KDK steps with a snapshot every `every` steps, written (a) the
    reference's way (to_state, then the file, the loop waiting) and (b) by
    snapshot.run_with_snapshots (device copy on the compute stream, copy
    stream + host thread for the rest); (c) without snapshots.  Files are
    .npz in a temporary directory (h5py is not installed here)."""
    pkg = importlib.import_module(PKG)
    snap = importlib.import_module(PKG + ".snapshot")
    ic = importlib.import_module(PKG + ".ic")
    st = importlib.import_module(PKG + ".state")
    pos, vel, mass = ic.exponential_disk(n, seed=0)
    s0 = st.State.from_arrays(pos, vel, mass)
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        for mode in ("none", "sync", "async"):
            eng = pkg.Engine(softening=BH_EPS, gravity_mode="bh", theta=BH_THETA, key_bits=BH_BITS,
                             device=dev)
            eng.load_state(s0)
            eng.run(BH_DT, 3)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if mode == "async":
                snap.run_with_snapshots(eng, BH_DT, steps, os.path.join(tmp, mode), snap_every=every)
            else:
                os.makedirs(os.path.join(tmp, mode), exist_ok=True)
                frame = 0
                if mode == "sync":
                    eng.to_state().save_npz(os.path.join(tmp, mode, f"snap_{frame:04d}.npz"))
                for k in range(steps // every):
                    eng.run(BH_DT, every)
                    if mode == "sync":
                        frame += 1
                        eng.to_state().save_npz(os.path.join(tmp, mode, f"snap_{frame:04d}.npz"))
                torch.cuda.synchronize()
            out[f"{mode}_s"] = time.perf_counter() - t0
    return {"workload": f"BH engine, 1M exponential disk, {steps} KDK steps, snapshot every {every} "
                        f"({steps // every + 1} files of {n} particles, .npz)",
            "wall_s_no_snapshots": out["none_s"], "wall_s_synchronous_snapshots": out["sync_s"],
            "wall_s_async_snapshots": out["async_s"],
            "snapshot_cost_per_file_ms": {"synchronous": (out["sync_s"] - out["none_s"]) / (steps // every + 1) * 1e3,
                                          "async": (out["async_s"] - out["none_s"]) / (steps // every + 1) * 1e3}}


def bench_scaling(dev, sizes=(10_000, 100_000, 1_000_000, 4_000_000, 16_000_000)):
    """BH KDK step time and force error against N (exponential disk, theta
    0.5, eps 0.05, 30-bit keys; error against FP64 direct sums on 256 seeded
    targets), and one direct N^2 force evaluation at N = 1M (per-target and
    symmetric passes; the symmetric one runs in bands of tile rows)."""
    ic = importlib.import_module(PKG + ".ic")
    bhmod = importlib.import_module(PKG + ".solvers.barnes_hut")
    grav = importlib.import_module(PKG + ".solvers.gravity")
    units = importlib.import_module(PKG + ".units")
    rows = []
    direct_ms = None
    for n in sizes:
        pos, vel, mass = ic.exponential_disk(n, seed=1)
        xm, v4 = _xm(pos, mass, dev), _v4(vel, dev)
        a4 = torch.zeros_like(xm)
        bh = bhmod.BarnesHut(n, theta=BH_THETA, softening=BH_EPS, key_bits=BH_BITS, G=units.G, device=dev)
        bh.compute(xm, a4)
        targets = np.random.default_rng(2).choice(n, 256, replace=False)
        ref = grav.acc_fp64_targets(xm, targets, units.G, BH_EPS * BH_EPS)
        got = a4[torch.as_tensor(targets, device=dev), :3].double().cpu().numpy()
        rel = np.linalg.norm(got - ref, axis=1) / np.linalg.norm(ref, axis=1)
        reps = 10 if n <= 4_000_000 else 3
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

        def timed_steps():
            for _ in range(3):
                bh.kdk(xm, v4, a4, BH_DT, 1)
            torch.cuda.synchronize()
            s.record()
            bh.kdk(xm, v4, a4, BH_DT, reps)
            e.record()
            torch.cuda.synchronize()
            return s.elapsed_time(e) / reps

        ms = timed_steps()
        d = bh.diag(reset=True)
        row = {"n": n, "bh_step_ms": ms, "particle_steps_per_s": n / ms * 1e3,
               "force_error_median": float(np.median(rel)), "p99": float(np.percentile(rel, 99)),
               "max": float(rel.max()), "stack_drops": d["stack_drops"], "bad_tree": d["bad_tree"]}
        # The opt-in group walk on the same state: step time and its force
        # error on the same targets (against FP64 sums of the same positions).
        bh.set_traversal(3)
        p0 = xm.clone()
        a3 = torch.zeros_like(xm)
        bh.compute(p0, a3)
        ref3 = grav.acc_fp64_targets(p0, targets, units.G, BH_EPS * BH_EPS)
        got3 = a3[torch.as_tensor(targets, device=dev), :3].double().cpu().numpy()
        rel3 = np.linalg.norm(got3 - ref3, axis=1) / np.linalg.norm(ref3, axis=1)
        ms3 = timed_steps()
        d3 = bh.diag(reset=True)
        row["group_walk"] = {"bh_step_ms": ms3, "particle_steps_per_s": n / ms3 * 1e3,
                             "force_error_median": float(np.median(rel3)), "p99": float(np.percentile(rel3, 99)),
                             "max": float(rel3.max()), "stack_overflow": d3["stack_overflow"],
                             "bad_tree": d3["bad_tree"]}
        rows.append(row)
        del p0, a3
        bh.close()
        if n == 1_000_000:
            g = grav.DirectGravity(n, dev)
            acc = torch.zeros_like(xm)
            direct_ms = {}
            for name, variant in (("per_target", 0), ("symmetric", 2)):
                g.set_variant(variant)
                g.acc(xm, acc, units.G, BH_EPS * BH_EPS)
                s.record()
                g.acc(xm, acc, units.G, BH_EPS * BH_EPS)
                e.record()
                torch.cuda.synchronize()
                direct_ms[name] = s.elapsed_time(e)
            g.close()
        del xm, v4, a4
        torch.cuda.empty_cache()
    return {"workload": "BH KDK step against N, exponential disk, theta 0.5, eps 0.05, 30-bit keys",
            "rows": rows, "direct_force_ms_at_1m": direct_ms}


# ------------------------------------------------------------------- main
def run_reference(args):
    """Reference arm: the float64 CPU restatement of the reference's BH path
    (oracle, OpenMP over all host threads) on the same workload."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    steps = []
    info = None
    for k in range(args.warmup + args.steps):
        r = cpu_bh_step(budget_s=8.0)
        if k >= args.warmup:
            steps.append(BH_N / r["value"])
            info = r
    t = float(sum(steps))
    value = BH_N * args.steps / t
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "particle-steps/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": _config(),
            "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": info["cores"],
                             "kind": "port", "sample": info["sample"]},
            "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def _config():
    return {"workload": "LBVH Barnes-Hut KDK step, exponential disk N=1,000,000 (M=5, Rd=3, "
                        "sech2 z0=0.3, G=43009.1725), theta=0.5, eps=0.05, 30-bit Morton keys, "
                        "dt=1e-4",
            "n": BH_N, "theta": BH_THETA, "eps": BH_EPS, "key_bits": 3 * BH_BITS, "dt": BH_DT,
            "l2": "flushed: 512 MiB memset between timed steps, outside the step events"}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=("gb", "reference"), default="gb")
    ap.add_argument("--no-secondary", action="store_true")
    ap.add_argument("--drift-steps", type=int, default=1000)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU oracle baseline")
    ap.add_argument("--bh-traversal", type=int, default=-1, choices=(-1, 0, 1, 2, 3),
                    help="traversal shape of the headline step (default -1: the per-particle walk)")
    ap.add_argument("--only", choices=("direct", "merger", "batch", "adjoint", "grid", "snapshot", "scaling"),
                    help="run one secondary workload alone (profiling runs)")
    args = ap.parse_args(argv)
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference(args)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("NCCL_NVLS_ENABLE", "0")
        dist.init_process_group("nccl", device_id=dev)
    pkg = importlib.import_module(PKG)
    pkg.load_library()
    lib_mod = importlib.import_module(PKG + "._lib")
    if args.only:
        peak = fp32_peak_tflops(lib_mod, dev)
        fn = {"direct": lambda: bench_direct(dev, lib_mod, peak),
              "merger": lambda: bench_merger(dev, args.drift_steps),
              "batch": lambda: bench_batch(dev),
              "adjoint": lambda: bench_adjoint(dev),
              "grid": lambda: bench_grid(dev),
              "snapshot": lambda: bench_snapshot(dev),
              "scaling": lambda: bench_scaling(dev)}[args.only]
        print(json.dumps({"only": args.only, "fp32_peak_tflops_measured": peak,
                          "result": fn()}), flush=True)
        return 0

    res = bench_bh(args, dev, rank, world, dist)
    line = {"metric": METRIC, "value": res["value"], "unit": "particle-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": res["ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (FP64 key quantisation)",
            "data": "synthetic (seeded exponential disk; one replica per rank)",
            "config": _config(), "roofline": res["roofline"], "e2e": res["e2e"],
            "gpu_launches": res["gpu_launches"], "clocks": res["clocks"],
            "stages_ms_per_step": res["stages_ms_per_step"],
            "traverse_work_per_step": res["work_per_step"],
            "traverse_fp32_tflops": res["traverse_fp32_tflops"],
            "force_error_vs_fp64_direct": res["force_error_vs_fp64_direct"],
            "energies_after_step": res["energies_after_step"],
            "diag": {k: res["diag"][k] for k in ("stack_drops", "stack_overflow", "nonfinite",
                                                  "bad_tree")}}
    if "group_walk" in res:
        line["group_walk"] = res["group_walk"]
    if not args.no_secondary:
        line["sharded_direct"] = bench_sharded_direct(args, dev, rank, world, dist)
        line["sharded_bh"] = bench_sharded_bh(args, dev, rank, world, dist)
    if rank == 0 and world == 1:
        if not args.no_cpu:
            line["cpu_baseline"] = cpu_bh_step()
        if not args.no_secondary:
            peak = fp32_peak_tflops(lib_mod, dev)
            sec = {"fp32_peak_tflops_measured": peak}
            sec["direct"] = bench_direct(dev, lib_mod, peak)
            sec["merger"] = bench_merger(dev, args.drift_steps)
            sec["batch"] = bench_batch(dev)
            sec["adjoint"] = bench_adjoint(dev)
            sec["neighbor_grid"] = bench_grid(dev)
            sec["snapshot"] = bench_snapshot(dev)
            line["secondary"] = sec
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
