"""Benchmark of the sparse level-set engine (one JSON line on rank 0).

Workload (default): the 256^3 three-shell phantom (seeded synthetic stand-in
for the reference's BrainWeb MRI) with four radius-3 seeds, T=0.8, eps=0.1,
alpha=0.85 (data weight), dt=0.5, run until the active count stays under 0.1%
of the initial count for 5 iterations (at most 2000).  The unit of work is
one seeding plus the whole run to convergence, in LSS_MODE_NS.

metric: active-voxel updates per second (sum over iterations of the active
count, from the device counter) over the device time of the steps; one step
= reseed from the device-resident volume + the run to convergence.
e2e: the same metric through the public API with host buffers each step
(volume upload, seeding, run, mask readback), the volume and the mask in
pinned host memory; e2e.pageable_value: the same with a pageable numpy volume
and a newly allocated mask array each step.
roofline: 20 algorithmic bytes per active-voxel update (phi in, I, phi out,
coordinate in/out) over the persistent kernel's CUDA-event time, against the
measured HBM copy bandwidth.
The default line also carries the other workloads, each measured briefly:
config1 (128^3, 300 iterations, GPU and CPU), batch (48 mixed-size volumes,
batched vs sequential plain), adjoint (192^3, K = 64), stress (512x512x768
and the 150 GB mixed batch) and ref_mode (the reference's algorithm at
256^3) and compaction (lss_compact_u32 on 2^28 elements); --workload X runs
one of them alone with the full step count.
--impl reference: the CPU restatement of the path (the FP64 oracle, all host
threads) on the same workload: one whole seeding + run to convergence, timed
as --steps consecutive segments (W warm-up segments first), in a process
that loads the oracle and the input generator only.
Multi-GPU: replicas only (each rank runs the whole workload on its GPU).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

BYTES_PER_UPDATE = 20
# Adjoint: phi 4, I 4, bias 4, lambda in 4 and out 4, bias gradient 8.
ADJOINT_BYTES = 28
FALLBACK_HBM_GBS = 6800.0


def measured_peak():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.samples: list[list[str]] = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = [r for r in self.samples if len(r) == 6 and r[0].isdigit()]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[2 + i] == "Active"})
        return {"sm_mhz": statistics.median(float(r[0]) for r in rows),
                "sm_max_mhz": max(float(r[1]) for r in rows), "reasons": reasons,
                "samples": len(rows)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, value: float) -> float:
    if ws == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(ws, value: float) -> float:
    if ws == 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


# DRAM bytes (read + write) of one launch of the persistent kernel on this
# workload, from an ncu capture of the build whose kernel sources hash to
# the key's first field (profiles/k_ns_persistent_config2_256.md gives the
# capture); a build from other sources reports null rather than a stale
# figure.
DRAM_TRAFFIC = {("f03f39b20e6e", "config2_256", 8, 8, 8, 256): 16179968}
KERNEL_SOURCES = ("ns_kernels.cuh", "ns_engine.cu", "tma.cuh", "common.cuh")
# The same for one adjoint call on config 4 (its two kernels: the forward,
# with the call's set-up and the loss as phases, and the reverse), from
# the capture in profiles/k_adj_config4_192.md.
ADJOINT_TRAFFIC = {("4d7505f8cf68", "config4_192"): 93272576}
ADJOINT_SOURCES = ("ns_adjoint.cu", "ns_kernels.cuh", "common.cuh")


def kernel_source_hash(files=KERNEL_SOURCES) -> str:
    """Hash of the kernel sources with their // comments and blank lines
    left out (a comment edit keeps a capture valid)."""
    import hashlib
    import re
    h = hashlib.sha256()
    csrc = os.path.join(ROOT, "aworkefficientgpualgorithmforlevelsetsegmentation_gb300", "csrc")
    for f in files:
        with open(os.path.join(csrc, f)) as fh:
            for line in fh:
                code = re.sub(r"//.*", "", line).rstrip()
                if code:
                    h.update(code.encode() + b"\n")
    return h.hexdigest()[:12]


def dram_traffic(st, name):
    return DRAM_TRAFFIC.get((kernel_source_hash(), name, st["brick_x"], st["brick_y"], st["brick_z"],
                             st["threads_per_brick"]))


def workload_config(cfg):
    """The workload as both arms name it (identical dicts)."""
    p = cfg["params"]
    nz, ny, nx = cfg["image"].shape
    return {"workload": cfg["name"] + "_three_shell_phantom", "mode": "LSS_MODE_NS",
            "volume_xyz": [nx, ny, nz], "seeds": len(cfg["spheres"]),
            "params": {"T": round(p.target, 6), "eps": round(p.window, 6), "alpha": round(p.curvature, 6),
                       "dt": round(p.time_step, 6), "alpha_weights": "data", "data_term": "normalised"},
            "stopping": "n < 0.1% n0 for 5 iterations, max 2000",
            "unit_of_work": "seeding + the whole run to convergence"}


def oracle_run(cfg, threads, parts=1, warmup_parts=0, max_iters=None):
    """The FP64 oracle on the host cores: seeding (phi and the initial active
    set) + the run to the workload's stopping rule (or max_iters iterations),
    timed as `parts` consecutive segments of about equal iteration counts
    (the last one runs to the stop); `warmup_parts` untimed segments from the
    seeds come first.  Returns (updates, seconds, iterations, per-part ms)."""
    from oracle.oracle import NsOracle
    p = cfg["params"]
    conv = cfg.get("conv")
    o = NsOracle(cfg["image"], brick=(8, 8, 8), threads=threads)
    o.set_params(p.target, p.window, p.curvature, p.time_step, p.phi_min, p.phi_max,
                 p.temporal_threshold, p.spatial_threshold, 26, p.alpha_role)
    expect = max_iters or 450  # iterations of the 256^3 run (434), for the split
    seg = max(1, -(-expect // max(1, parts)))

    def segment(state, m):
        for _ in range(m):
            n = o.n
            o.step(1)
            state["it"] += 1
            if max_iters is not None:
                if state["it"] >= max_iters:
                    return True
                continue
            state["streak"] = state["streak"] + 1 if n < conv["rel"] * o.n0 else 0
            if state["streak"] >= conv["patience"] or n == 0 or state["it"] >= conv["max_iterations"]:
                return True
        return False

    if warmup_parts:
        o.set_phi(cfg["phi0"])
        st = {"it": 0, "streak": 0}
        for _ in range(warmup_parts):
            if segment(st, seg):
                break
    u0 = o.updates
    st = {"it": 0, "streak": 0}
    part_ms, stopped = [], False
    t_all = time.perf_counter()
    for k in range(parts):
        t0 = time.perf_counter()
        if k == 0:
            o.set_phi(cfg["phi0"])
            u0 = o.updates
        stopped = segment(st, seg if k < parts - 1 else 1 << 30)
        part_ms.append(1e3 * (time.perf_counter() - t0))
        if stopped:
            break
    dt = time.perf_counter() - t_all
    return o.updates - u0, dt, st["it"], part_ms


def run_reference(args, ws, rank):
    if rank != 0:
        return
    from aworkefficientgpualgorithmforlevelsetsegmentation_gb300 import phantoms as P
    cfg = P.config2(args.scale)
    threads = os.cpu_count() or 1
    steps = max(1, args.steps)
    upd, sec, its, part_ms = oracle_run(cfg, threads, steps, args.warmup)
    value = upd / sec
    c1 = P.config1(args.scale)
    u1, s1, i1, _ = oracle_run(c1, threads, 1, 0, max_iters=c1["iterations"])
    line = {
        "impl": "reference", "metric": "active_voxel_updates_per_s", "value": value,
        "unit": "voxel_updates/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * sec / max(1, len(part_ms)), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(cfg),
        "cpu_baseline": {"value": value, "unit": "voxel_updates/s", "cores": threads, "kind": "port",
                         "sample": f"one whole run of {cfg['name']} (seeding + {its} iterations to "
                                   f"convergence, {upd} updates) timed as {len(part_ms)} consecutive "
                                   f"segments; FP64 oracle on all host threads",
                         "config1": {"value": u1 / s1, "ms": 1e3 * s1, "iterations": i1,
                                     "voxel_updates": int(u1), "workload": c1["name"]}},
        "e2e": {"value": value, "unit": "voxel_updates/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, ws, rank, local):
    import ctypes
    import torch
    import aworkefficientgpualgorithmforlevelsetsegmentation_gb300 as lss
    from aworkefficientgpualgorithmforlevelsetsegmentation_gb300 import phantoms as P

    torch.cuda.set_device(local)
    cfg = P.config2(args.scale)
    p = cfg["params"]
    conv = cfg["conv"]
    # The plain workload runs the 8x8x8 / 256-thread configuration unless
    # --brick (or --brick 0 0 0 for the autotuner) says otherwise.
    brick = tuple(args.brick) if args.brick else (8, 8, 8)
    threads = args.threads or (256 if not args.brick else 0)
    seg = lss.Segmenter(lss.MODE_NS, device=local, brick=brick, threads_per_brick=threads,
                        brick_workers=args.workers)
    stream = torch.cuda.Stream(device=local)
    seg._chk(seg._lib.lss_set_stream(seg._h, ctypes.c_void_p(stream.cuda_stream)))
    seg.load_volume(cfg["image"])
    seg.set_parameters(p.target, p.window, p.curvature, p.time_step, alpha_role=p.alpha_role)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def one_step():
        seg.clear_current_segmentation()
        seg.set_seed_spheres(cfg["spheres"])
        return seg.step_until_converged(conv["rel"], conv["patience"], conv["max_iterations"])

    for _ in range(args.warmup):
        one_step()
    torch.cuda.synchronize()
    barrier(ws)
    ev_ms, kern_ms, updates, iters = 0.0, 0.0, 0, []
    # Kernel launches of the library inside the timed steps: the counter is
    # read at the start of each stats call, and every stats call itself
    # launches one kernel (the active-count readback) afterwards.
    launches0 = seg.stats()["kernel_launches"]
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.fill_(1)  # L2 flush between timed steps (outside the events)
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            it = one_step()
            e1.record(stream)
            e1.synchronize()
            ev_ms += e0.elapsed_time(e1)
            st = seg.stats()
            kern_ms += st["last_step_ms"]
            updates += st["voxel_updates"]
            iters.append(it)
    launches_steps = st["kernel_launches"] - launches0 - args.steps
    torch.cuda.synchronize()
    barrier(ws)
    t_max = max_over_ranks(ws, ev_ms)
    total_updates = sum_over_ranks(ws, float(updates))
    value = total_updates / (t_max / 1e3)
    st = seg.stats()
    mask = seg.get_saveable_segmentation()

    # e2e through the public API with host buffers: every step uploads the
    # volume, seeds, runs to convergence and reads the mask back.  The main
    # figure stages the volume and the mask in pinned host memory (allocated
    # once, outside the timed steps); the second passes a pageable numpy
    # volume and lets the call allocate a new mask array each step.
    def e2e(img, out):
        ms, upd, m = 0.0, 0, None
        for s in range(args.warmup + args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            seg.load_volume(img)
            seg.set_parameters(p.target, p.window, p.curvature, p.time_step, alpha_role=p.alpha_role)
            seg.set_seed_spheres(cfg["spheres"])
            seg.step_until_converged(conv["rel"], conv["patience"], conv["max_iterations"])
            m = seg.get_saveable_segmentation(out=out)
            t1 = time.perf_counter()
            if s >= args.warmup:
                ms += 1e3 * (t1 - t0)
                upd += seg.stats()["voxel_updates"]
        assert np.array_equal(m, mask)
        return sum_over_ranks(ws, float(upd)) / (max_over_ranks(ws, ms) / 1e3)

    img = np.ascontiguousarray(cfg["image"])
    img_pinned = torch.empty(img.shape, dtype=torch.float32, pin_memory=True).numpy()
    img_pinned[...] = img
    mask_pinned = torch.empty(mask.shape, dtype=torch.uint8, pin_memory=True).numpy()
    e2e_value = e2e(img_pinned, mask_pinned)
    e2e_pageable = e2e(img, None)

    # Dense all-voxel GPU update (same arithmetic, every voxel, no active set)
    # timed over the same number of iterations the sparse run needed.
    seg.clear_current_segmentation()
    seg.set_seed_spheres(cfg["spheres"])
    seg.step_dense(3)
    seg.clear_current_segmentation()
    seg.set_seed_spheres(cfg["spheres"])
    dense_ms_per_it = seg.step_dense(args.dense_iters) / args.dense_iters
    sparse_ms = ev_ms / args.steps
    dense_ms = dense_ms_per_it * statistics.mean(iters)
    del seg
    torch.cuda.synchronize()

    peak, peak_kind = measured_peak()
    achieved = BYTES_PER_UPDATE * updates / (kern_ms / 1e3) / 1e9
    traffic = dram_traffic(st, cfg["name"])
    extra = {}
    if not args.no_extra:
        extra["config1"] = measure_config1(local, args.scale, 10, 3, cpu=rank == 0 and not args.no_cpu)
        extra["batch"] = measure_batch(local, args.scale, 3, 1)
        extra["adjoint"] = measure_adjoint(local, args.scale, 10, 3)
        extra["stress"] = measure_stress(local, args.scale, 2, 1)
        extra["ref_mode"] = measure_ref_mode(local, args.scale, 5, 2)
        extra["compaction"] = measure_compaction(local, 10, 3)
    if rank == 0:
        cpu = None
        if not args.no_cpu:
            cu, ct, cit, _ = oracle_run(cfg, os.cpu_count() or 1)
            cpu = {"value": cu / ct, "unit": "voxel_updates/s", "cores": os.cpu_count(), "kind": "port",
                   "sample": f"one whole run of {cfg['name']} (seeding + {cit} iterations to convergence, "
                             f"{cu} updates); FP64 oracle on all host threads"}
            if "config1" in extra:
                cpu["config1"] = extra["config1"].pop("cpu")
        line = {
            "metric": "active_voxel_updates_per_s", "value": value, "unit": "voxel_updates/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": workload_config(cfg),
            "run": {"iterations_to_converge": iters[-1], "converge_ms": sparse_ms,
                    "brick": [st["brick_x"], st["brick_y"], st["brick_z"]],
                    "threads_per_brick": st["threads_per_brick"], "grid_blocks": st["grid_blocks"],
                    "block_threads": st["block_threads"],
                    "block0_update_ms": st["update_ms"], "block0_barrier_ms": st["barrier_ms"],
                    "l2": "flushed between steps (256 MiB write); volume 192 MiB > L2",
                    "parallelism": "replicas" if ws > 1 else "single"},
            "dense_gpu": {"ms_to_same_iterations": dense_ms, "ms_per_iteration": dense_ms_per_it,
                          "sparse_speedup": dense_ms / sparse_ms},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                         "traffic_source": None if traffic is None else
                         "ncu capture of this kernel build (profiles/k_ns_persistent_config2_256.md)",
                         "kernel_source_hash": kernel_source_hash(),
                         "bytes_per_update": BYTES_PER_UPDATE,
                         "algorithmic_bytes_per_launch": BYTES_PER_UPDATE * updates / args.steps},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "voxel_updates/s",
                    "h2d_bytes_per_step": int(img.nbytes),
                    "d2h_bytes_per_step": int(mask.nbytes),
                    "host_buffers": "pinned (volume staged once; mask read into a reused pinned array)",
                    "pageable_value": e2e_pageable},
            "gpu_launches": int(launches_steps),
            "clocks": clk.summary(),
        }
        line.update(extra)
        print(json.dumps(line), flush=True)


def measure_config1(local, scale, steps, warmup, cpu=True):
    """Config 1: the 128^3 ellipsoid, phi0 = signed distance to a radius-5
    sphere, 300 iterations; GPU device time (set_phi + 300 iterations) and the
    FP64 oracle on all host threads."""
    import torch
    import aworkefficientgpualgorithmforlevelsetsegmentation_gb300 as lss
    from aworkefficientgpualgorithmforlevelsetsegmentation_gb300 import phantoms as P
    c = P.config1(scale)
    p = c["params"]
    s = lss.Segmenter(lss.MODE_NS, device=local, brick=(8, 8, 8), threads_per_brick=256)
    s.load_volume(c["image"])
    s.set_parameters(p.target, p.window, p.curvature, p.time_step, alpha_role=p.alpha_role)
    ms, upd = [], 0
    for k in range(warmup + steps):
        s.set_phi(c["phi0"])
        s.step(c["iterations"])
        st = s.stats()
        if k >= warmup:
            ms.append(st["last_step_ms"])
            upd = st["voxel_updates"]
    out = {"workload": c["name"] + "_ellipsoid", "iterations": c["iterations"],
           "gpu": {"ms": statistics.median(ms), "voxel_updates": int(upd),
                   "value": upd / (statistics.median(ms) / 1e3), "unit": "voxel_updates/s"}}
    del s
    torch.cuda.synchronize()
    if cpu:
        u1, s1, i1, _ = oracle_run(c, os.cpu_count() or 1, max_iters=c["iterations"])
        out["cpu"] = {"value": u1 / s1, "ms": 1e3 * s1, "iterations": i1, "voxel_updates": int(u1),
                      "cores": os.cpu_count(), "kind": "port", "workload": c["name"]}
    return out


def measure_batch(local, scale, steps, warmup, brick=None, threads=0):
    """Batched form: the 48 mixed-size single-ellipsoid volumes in one
    persistent launch (autotuned brick configuration unless `brick` fixes
    it) against the same volumes run one after another through the plain
    engine (8^3 x 256 unless `brick` fixes it)."""
    import torch
    import aworkefficientgpualgorithmforlevelsetsegmentation_gb300 as lss
    from aworkefficientgpualgorithmforlevelsetsegmentation_gb300 import phantoms as P

    cfg = P.config3(48, scale=scale)
    vols, conv = cfg["volumes"], cfg["conv"]
    pbrick = tuple(brick) if brick else (8, 8, 8)
    pthreads = threads or 256
    segs = []
    for v in vols:
        p = v["params"]
        s = lss.Segmenter(lss.MODE_NS, device=local, brick=pbrick, threads_per_brick=pthreads)
        s.load_volume(v["image"])
        s.set_parameters(p.target, p.window, p.curvature, p.time_step, alpha_role=p.alpha_role)
        segs.append(s)

    def plain_all():
        dev_ms, upd, its = 0.0, 0, []
        for s, v in zip(segs, vols):
            s.clear_current_segmentation()
            s.set_seed_spheres(v["spheres"])
            its.append(s.step_until_converged(conv["rel"], conv["patience"], conv["max_iterations"]))
            st = s.stats()
            dev_ms += st["last_step_ms"]
            upd += st["voxel_updates"]
        return dev_ms, upd, its

    bbrick, bthreads = (pbrick, pthreads) if brick else ((0, 0, 0), 0)

    def batched():
        b = lss.Batch(device=local, brick=bbrick, threads_per_brick=bthreads)
        for v in vols:
            b.add_volume(v["image"], v["params"], v["spheres"])
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        it = b.run(conv["rel"], conv["patience"], conv["max_iterations"])
        wall = 1e3 * (time.perf_counter() - t0)
        st = [b.stats(i) for i in range(len(vols))]
        return b, wall, st[0]["last_step_ms"], sum(x["voxel_updates"] for x in st), it

    for _ in range(warmup):
        plain_all()
    seq_wall, seq_dev, seq_upd, its = [], [], 0, []
    for _ in range(steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        d, u, its = plain_all()
        seq_wall.append(1e3 * (time.perf_counter() - t0))
        seq_dev.append(d)
        seq_upd = u
    for _ in range(max(1, warmup)):  # the first run tunes the brick configuration
        batched()
    bat_wall, bat_dev = [], []
    for _ in range(steps):
        b, w, d, bupd, bit = batched()
        bat_wall.append(w)
        bat_dev.append(d)
    same = all(np.array_equal(b.read_mask(i), segs[i].get_saveable_segmentation())
               for i in range(0, len(vols), 7))
    sw, bw = statistics.median(seq_wall), statistics.median(bat_wall)
    out = {"workload": cfg["name"] + "_mixed_size_ellipsoids", "volumes": len(vols),
           "voxels": int(sum(v["image"].size for v in vols)),
           "speedup_wall": sw / bw,
           "speedup_device": statistics.median(seq_dev) / statistics.median(bat_dev),
           "sequential_plain": {"ms_wall": sw, "ms_device": statistics.median(seq_dev),
                                "voxel_updates": int(seq_upd), "iterations_max": int(max(its)),
                                "brick": list(pbrick), "threads_per_brick": pthreads},
           "batched": {"ms_wall": bw, "ms_device": statistics.median(bat_dev), "voxel_updates": int(bupd),
                       "iterations": int(bit), "updates_per_s": bupd / (bw / 1e3),
                       "brick": [b.stats(0)["brick_x"], b.stats(0)["brick_y"], b.stats(0)["brick_z"]],
                       "threads_per_brick": b.stats(0)["threads_per_brick"],
                       "block_threads": b.stats(0)["block_threads"]},
           "masks_identical_to_plain": bool(same), "steps": steps}
    del b, segs
    torch.cuda.synchronize()
    return out


def run_batch(args, ws, rank, local):
    import torch
    torch.cuda.set_device(local)
    r = measure_batch(local, args.scale, args.steps, args.warmup, args.brick, args.threads)
    if rank == 0:
        line = {"metric": "batched_vs_sequential_plain_speedup", "value": r["speedup_wall"], "unit": "x",
                "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "higher_is_better": True,
                "dtype": "f32", "data": "synthetic", "config": {"workload": r["workload"]}, "batch": r}
        print(json.dumps(line), flush=True)


def measure_stress(local, scale, steps, warmup, brick=None, threads=0):
    """Large plain volume (512x512x768 three-shell phantom, 16 radius-4
    seeds) to convergence, and the mixed batch (8 volumes of 384^3 + 64 of
    64^3) in one persistent launch under a 150 GB HBM budget."""
    import torch
    import aworkefficientgpualgorithmforlevelsetsegmentation_gb300 as lss
    from aworkefficientgpualgorithmforlevelsetsegmentation_gb300 import phantoms as P

    t0 = time.perf_counter()
    cfg = P.config5(scale)
    gen_s = time.perf_counter() - t0
    p, conv = cfg["params"], cfg["conv"]
    brick = tuple(brick) if brick else (8, 8, 8)
    threads = threads or 256
    seg = lss.Segmenter(lss.MODE_NS, device=local, brick=brick, threads_per_brick=threads)
    seg.load_volume(cfg["image"])
    seg.set_parameters(p.target, p.window, p.curvature, p.time_step, alpha_role=p.alpha_role)
    runs = []
    for s in range(warmup + steps):
        seg.clear_current_segmentation()
        seg.set_seed_spheres(cfg["spheres"])
        it = seg.step_until_converged(conv["rel"], conv["patience"], conv["max_iterations"])
        st = seg.stats()
        if s >= warmup:
            runs.append((st["last_step_ms"], st["voxel_updates"], it))
    ms = statistics.median(r[0] for r in runs)
    upd = runs[-1][1]
    peak, peak_kind = measured_peak()
    achieved = BYTES_PER_UPDATE * upd / (ms / 1e3) / 1e9
    plain = {"workload": cfg["name"], "ms_to_converge": ms, "iterations": runs[-1][2],
             "voxel_updates": int(upd), "updates_per_s": upd / (ms / 1e3),
             "roofline": {"achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                          "peak_kind": peak_kind, "bytes_per_update": BYTES_PER_UPDATE},
             "device_bytes": int(st["device_bytes"]), "phantom_s": gen_s}
    del seg, cfg
    torch.cuda.synchronize()
    # Mixed batch under a 150 GB budget: 8 three-shell volumes of 384^3 and
    # 64 single-ellipsoid volumes of 64^3.
    big = P.config2(1.5 * scale)
    vols = [(big["image"], big["params"], big["spheres"]) for _ in range(8)]
    rng = np.random.default_rng(9)
    m = max(16, int(round(64 * scale)))
    for i in range(64):
        c = (m - 1) / 2 + rng.uniform(-0.1, 0.1, 3) * m
        axes = rng.uniform(0.2, 0.4, 3) * m
        fg, bg = rng.uniform(0.6, 0.9), rng.uniform(0.1, 0.3)
        img = P.ellipsoid((m, m, m), tuple(c), tuple(axes), fg, bg, 0.05, 2000 + i)
        vols.append((img, P.ns_params(fg, 0.1, 0.9), [(c[0], c[1], c[2], 3.0)]))
    b = lss.Batch(device=local, brick=brick, threads_per_brick=threads, hbm_budget_bytes=150 << 30)
    for img, prm, sp in vols:
        b.add_volume(img, prm, sp)
    t1 = time.perf_counter()
    bit = b.run(conv["rel"], conv["patience"], conv["max_iterations"])
    bwall = 1e3 * (time.perf_counter() - t1)
    bst = [b.stats(i) for i in range(len(vols))]
    bupd = sum(x["voxel_updates"] for x in bst)
    batch = {"volumes": len(vols), "voxels": int(sum(v[0].size for v in vols)), "iterations": int(bit),
             "ms_device": bst[0]["last_step_ms"], "ms_wall": bwall, "voxel_updates": int(bupd),
             "updates_per_s": bupd / (bst[0]["last_step_ms"] / 1e3),
             "device_bytes": int(bst[0]["device_bytes"]), "hbm_budget_bytes": 150 << 30}
    del b
    torch.cuda.synchronize()
    return {"plain": plain, "batch": batch, "brick": list(brick), "threads_per_brick": threads}


def run_stress(args, ws, rank, local):
    import torch
    torch.cuda.set_device(local)
    r = measure_stress(local, args.scale, args.steps, args.warmup, args.brick, args.threads)
    if rank == 0:
        print(json.dumps({"metric": "stress", "dtype": "f32", "data": "synthetic", **r}), flush=True)


def measure_adjoint(local, scale, steps, warmup):
    """Differentiation form: the 192^3 two-shell phantom, K = 64 unrolled
    iterations from the seed, phi checkpointed every 8, soft-Dice loss of
    sigmoid(-phi/0.5) against the inner ellipsoid.  One step = one
    lss_adjoint_run: the forward records the K active sets, the loss, the
    reverse pass recomputes each segment from its checkpoint and scatters the
    transposed stencil Jacobian, giving dloss/dT, deps, dalpha and the bias
    volume's gradient.  The value has target, bias and the bias gradient in
    device memory (used in place); e2e the same calls with pinned host
    buffers (the bias and its gradient cross the host link every call).  The
    metric is active-voxel iterations (the sum over the forward iterations of
    the active voxels updated) per second of the whole call;
    the roofline counts 28 bytes each (phi, I, bias, lambda in and out, the
    bias gradient read and written)."""
    import ctypes
    import torch
    import aworkefficientgpualgorithmforlevelsetsegmentation_gb300 as lss
    from aworkefficientgpualgorithmforlevelsetsegmentation_gb300 import phantoms as P

    cfg = P.config4(scale)
    p = cfg["params"]
    K, every = cfg["K"], cfg["checkpoint_every"]
    seg = lss.Segmenter(lss.MODE_NS, device=local, brick=(8, 8, 8), threads_per_brick=256)
    stream = torch.cuda.Stream(device=local)
    seg._chk(seg._lib.lss_set_stream(seg._h, ctypes.c_void_p(stream.cuda_stream)))
    seg.load_volume(cfg["image"])
    seg.set_parameters(p.target, p.window, p.curvature, p.time_step, alpha_role=p.alpha_role)
    seg.set_phi(cfg["phi0"])
    shape = cfg["image"].shape

    def pinned(dt):
        return torch.empty(shape, dtype=dt, pin_memory=True).numpy()

    def timed(tgt, bias, dbias):
        for _ in range(warmup):
            g = seg.adjoint(K, every, tgt, 0.5, bias=bias, d_bias_out=dbias)
        torch.cuda.synchronize()
        ev_ms, nact = [], 0
        launches0 = seg.stats()["kernel_launches"]
        for _ in range(steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            g = seg.adjoint(K, every, tgt, 0.5, bias=bias, d_bias_out=dbias)
            e1.record(stream)
            e1.synchronize()
            ev_ms.append(e0.elapsed_time(e1))
            nact += g["active_voxel_iterations"]
        return ev_ms, nact, g, (seg.stats()["kernel_launches"] - launches0) // steps

    # Inputs resident in HBM (torch CUDA tensors, used in place): the value.
    tgt_d = torch.from_numpy(np.ascontiguousarray(cfg["target"], np.uint8)).to(f"cuda:{local}")
    bias_d = torch.zeros(shape, dtype=torch.float32, device=f"cuda:{local}")
    dbias_d = torch.empty(shape, dtype=torch.float32, device=f"cuda:{local}")
    ev_ms, nact, g, launches = timed(tgt_d, bias_d, dbias_d)
    # Pinned host buffers, the bias in and its gradient out over the host link: e2e.
    tgt, bias, dbias = pinned(torch.uint8), pinned(torch.float32), pinned(torch.float32)
    tgt[...] = cfg["target"]
    bias[...] = 0.0
    ev_h, nact_h, gh, launches_h = timed(tgt, bias, dbias)
    same = (gh["loss"] == g["loss"] and abs(gh["d_target"] - g["d_target"]) <= 1e-6 * abs(g["d_target"])
            and bool(np.allclose(dbias, dbias_d.cpu().numpy(), rtol=1e-4, atol=1e-9)))
    tot, tot_h = sum(ev_ms), sum(ev_h)
    peak, peak_kind = measured_peak()
    achieved = ADJOINT_BYTES * nact / (tot / 1e3) / 1e9
    n = int(np.prod(shape))
    del seg
    torch.cuda.synchronize()
    return {"workload": cfg["name"] + "_two_shell_adjoint", "K": K, "checkpoint_every": every,
            "ms_per_call": tot / steps, "ms_per_call_median": statistics.median(ev_ms),
            "active_voxel_iterations_per_call": int(g["active_voxel_iterations"]),
            "value": nact / (tot / 1e3), "unit": "active_voxel_iterations/s",
            "loss": g["loss"], "d_target": g["d_target"], "d_window": g["d_window"],
            "d_curvature": g["d_curvature"], "gpu_launches_per_call": int(launches),
            "buffers": "device (target, bias, bias gradient in HBM, used in place)",
            "e2e": {"value": nact_h / (tot_h / 1e3), "unit": "active_voxel_iterations/s",
                    "ms_per_call": tot_h / steps, "ms_per_call_median": statistics.median(ev_h),
                    "buffers": "pinned host (target, bias, bias gradient)",
                    "h2d_bytes_per_step": n + 4 * n, "d2h_bytes_per_step": 4 * n,
                    "gpu_launches_per_call": int(launches_h), "same_result_as_device_buffers": same},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind,
                         "bytes_per_update": ADJOINT_BYTES,
                         "algorithmic_bytes_per_call": ADJOINT_BYTES * int(g["active_voxel_iterations"]),
                         "traffic_per_call": ADJOINT_TRAFFIC.get((kernel_source_hash(ADJOINT_SOURCES), cfg["name"])),
                         "kernel_source_hash": kernel_source_hash(ADJOINT_SOURCES)}, "steps": steps}


def run_adjoint(args, ws, rank, local):
    import torch
    torch.cuda.set_device(local)
    with ClockSampler(local) as clk:
        r = measure_adjoint(local, args.scale, args.steps, args.warmup)
    if rank == 0:
        line = {"metric": "adjoint_active_voxel_iterations_per_s", "value": r["value"], "unit": r["unit"],
                "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_call"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic", "config": {"workload": r["workload"]}, "adjoint": r,
                "e2e": {k: r["e2e"][k] for k in ("value", "unit", "h2d_bytes_per_step", "d2h_bytes_per_step")},
                "gpu_launches": r["gpu_launches_per_call"] * args.steps, "clocks": clk.summary()}
        print(json.dumps(line), flush=True)


def measure_compaction(local, steps, warmup, n=1 << 28, frac=0.5):
    """The kernel-level compaction (lss_compact_u32, the reference's
    CudppCompact; lss_compact_u32_noalloc beside it at its largest size) on
    2^28 elements (1 GiB each of values, flags and output), half of them kept.
    Timed with CUDA events on the call's stream around each call (the call
    takes its scratch from the library's stream-ordered pool, clears it, runs
    the count, scan and scatter passes, reads its error word back and
    synchronises).  Roofline: 8 B an element
    (flag and value) + 4 B a kept one, against the measured HBM peak."""
    import ctypes as C
    import torch
    import aworkefficientgpualgorithmforlevelsetsegmentation_gb300 as lss

    L = lss.load()
    dev = torch.device(f"cuda:{local}")
    g = torch.Generator(device=dev)
    g.manual_seed(5)
    stream = torch.cuda.Stream(device=dev)
    peak, peak_kind = measured_peak()

    def timed(fn, m):
        src = torch.arange(m, dtype=torch.int32, device=dev)
        valid = (torch.rand(m, device=dev, generator=g) < frac).to(torch.int32)
        dst = torch.empty(m, dtype=torch.int32, device=dev)
        cnt = torch.zeros(1, dtype=torch.int64, device=dev)
        args = (C.c_void_p(src.data_ptr()), C.c_void_p(valid.data_ptr()), C.c_void_p(dst.data_ptr()), m,
                C.c_void_p(cnt.data_ptr()), C.c_void_p(stream.cuda_stream))
        torch.cuda.synchronize()
        for _ in range(warmup):
            assert fn(*args) == 0
        ts = []
        for _ in range(steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            assert fn(*args) == 0
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        kept = int(cnt.item())
        same = bool(torch.equal(dst[:kept], src[valid.bool()]))
        ms = statistics.median(ts)
        alg = 8 * m + 4 * kept
        del src, valid, dst
        torch.cuda.empty_cache()
        return {"n": m, "kept": kept, "ms_per_call": ms, "algorithmic_bytes": alg,
                "achieved_gbs": alg / (ms / 1e3) / 1e9, "peak": peak, "peak_kind": peak_kind,
                "frac": alg / (ms / 1e3) / 1e9 / peak, "matches_torch": same}

    return {"lss_compact_u32": timed(L.lss_compact_u32, n),
            "lss_compact_u32_noalloc": timed(L.lss_compact_u32_noalloc, 1 << 26),
            "valid_fraction": frac, "bytes_model": "8 B an element (flag, value) + 4 B a kept element"}


def run_compaction(args, ws, rank, local):
    import torch
    torch.cuda.set_device(local)
    with ClockSampler(local) as clk:
        r = measure_compaction(local, args.steps, args.warmup)
    if rank == 0:
        c = r["lss_compact_u32"]
        line = {"metric": "compaction_algorithmic_bytes_per_s", "value": c["achieved_gbs"], "unit": "GB/s",
                "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": c["ms_per_call"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
                "data": "synthetic", "config": {"workload": "compact_u32_2^28_half_kept",
                                                "l2": "inputs larger than L2 (1 GiB each)"},
                "compaction": r, "gpu_launches": 3 * 2 * args.steps, "clocks": clk.summary()}
        print(json.dumps(line), flush=True)


def measure_ref_mode(local, scale, steps, warmup):
    """LSS_MODE_REF at the headline size: the reference's own solver
    reproduced bit for bit (int8 phi in 16^3 tiles, integer intensities, the
    6-connected output, duplicate-filter and compaction pipeline, one CUDA
    graph an iteration) on the 256^3 three-shell phantom quantised to u8
    (round(255 I)), seeded with the same four spheres; grow level 204 (the
    inner shell's 0.8), window 26 (0.1 in u8 units), curvature weight 0.1,
    dt 0.25; run until the active count stays under 0.1 % of its initial value
    for 5 iterations.  One step = clear + seed + run (the state the fixtures
    of tests/golden/make_golden_ref256.py pin as "rerun").  Metric:
    active-voxel updates per second (device count over the iterations'
    CUDA-event time), the figure the GTX 280 reached at 41.4 M/s with the
    same algorithm on BrainWeb MRI (a different input: a throughput
    comparison only)."""
    import torch
    import aworkefficientgpualgorithmforlevelsetsegmentation_gb300 as lss
    from aworkefficientgpualgorithmforlevelsetsegmentation_gb300 import phantoms as P

    cfg = P.config2(scale)
    u8 = np.clip(np.rint(cfg["image"] * 255.0), 0, 255).astype(np.uint8)
    r = lss.Segmenter(lss.MODE_REF, device=local)
    r.load_volume(u8)
    r.set_parameters(204, 26, 0.1, 0.25)

    def one_step():
        r.clear_current_segmentation()
        for (x, y, z, rad) in cfg["spheres"]:
            r.initialize_seed((x, y, z), rad)
        u0 = r.stats()["voxel_updates"]
        it = r.step_until_converged(1e-3, 5, 2000)
        st = r.stats()
        return it, st["voxel_updates"] - u0, st["last_step_ms"]

    for _ in range(warmup):
        one_step()
    torch.cuda.synchronize()
    ms, upd, its = 0.0, 0, []
    launches0 = r.stats()["kernel_launches"]
    for _ in range(steps):
        it, u, t = one_step()
        ms += t
        upd += u
        its.append(it)
    launches = (r.stats()["kernel_launches"] - launches0) // steps
    mask = r.get_saveable_segmentation()
    del r
    torch.cuda.synchronize()
    return {"workload": cfg["name"] + "_three_shell_phantom_u8", "mode": "LSS_MODE_REF",
            "params": {"grow_level": 204, "grow_window": 26, "curvature": 0.1, "dt": 0.25},
            "stopping": "n < 0.1% n0 for 5 iterations, max 2000",
            "value": upd / (ms / 1e3), "unit": "voxel_updates/s", "ms_per_run": ms / steps,
            "iterations_to_converge": its[-1], "updates_per_run": upd // steps,
            "segmented_voxels": int(mask.sum()), "gpu_launches_per_run": int(launches),
            "gtx280_published_updates_per_s": 41.4e6, "steps": steps}


def run_ref_mode(args, ws, rank, local):
    import torch
    torch.cuda.set_device(local)
    with ClockSampler(local) as clk:
        r = measure_ref_mode(local, args.scale, args.steps, args.warmup)
    if rank == 0:
        line = {"metric": "ref_mode_active_voxel_updates_per_s", "value": r["value"], "unit": r["unit"],
                "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["ms_per_run"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "int8 phi, u8 I", "data": "synthetic", "config": {"workload": r["workload"]},
                "ref_mode": r, "clocks": clk.summary()}
        print(json.dumps(line), flush=True)


def run_tour(args, ws, rank, local):
    """Every kernel of the library once, on small inputs (for a per-kernel
    ncu launch list): the REF engine (u8 volume: seed, steps on the few- and
    many-active paths, read-backs, parameter estimate), the NS engine (seed,
    sparse steps with a block per brick and with four brick workers a block,
    dense steps, read-backs), the batched form (a warp per brick), the
    adjoint and the kernel-level compaction."""
    import ctypes as C
    import torch
    import aworkefficientgpualgorithmforlevelsetsegmentation_gb300 as lss
    from aworkefficientgpualgorithmforlevelsetsegmentation_gb300 import phantoms as P

    torch.cuda.set_device(local)
    cfg = P.config1(0.5)
    u8 = np.clip(cfg["image"] * 200.0, 0, 255).astype(np.uint8)
    r = lss.Segmenter(lss.MODE_REF)
    r.load_volume(u8)
    r.set_parameters(140, 40, 0.2, 0.25)
    r.initialize_seed((32, 32, 32), 6)
    r.request_update_segmentation(20)
    r.get_saveable_segmentation()
    r.read_active_volume()
    r.calculate_segmentation_parameters()
    p = cfg["params"]
    s = lss.Segmenter(lss.MODE_NS, brick=(8, 8, 8), threads_per_brick=256)
    s.load_volume(cfg["image"])
    s.set_parameters(p.target, p.window, p.curvature, p.time_step, alpha_role=p.alpha_role)
    s.set_seed_spheres(cfg["spheres"])
    s.step(20)
    s.active_linear()
    s.read_phi()
    s.freeze_current_segmentation()
    s.get_saveable_segmentation()
    s.step_dense(2)
    w = lss.Segmenter(lss.MODE_NS, brick=(8, 8, 8), threads_per_brick=256, brick_workers=4)
    w.load_volume(cfg["image"])
    w.set_parameters(p.target, p.window, p.curvature, p.time_step, alpha_role=p.alpha_role)
    w.set_seed_spheres(cfg["spheres"])
    w.step(20)
    c4 = P.config4(0.25)
    a = lss.Segmenter(lss.MODE_NS, brick=(8, 8, 8), threads_per_brick=256)
    a.load_volume(c4["image"])
    q = c4["params"]
    a.set_parameters(q.target, q.window, q.curvature, q.time_step, alpha_role=q.alpha_role)
    a.set_phi(c4["phi0"])
    a.adjoint(8, 4, c4["target"])
    b = lss.Batch(brick=(8, 8, 4), threads_per_brick=32)
    for v in P.config3(4, scale=0.25)["volumes"]:
        b.add_volume(v["image"], v["params"], v["spheres"])
    b.run(1e-3, 5, 200)
    n = 1 << 20
    src = torch.arange(n, dtype=torch.int32, device="cuda")
    valid = (torch.arange(n, device="cuda") % 3 == 0).to(torch.int32)
    dst = torch.zeros(n, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int64, device="cuda")
    L = lss.load()
    for f in (L.lss_compact_u32, L.lss_compact_u32_noalloc):
        assert f(C.c_void_p(src.data_ptr()), C.c_void_p(valid.data_ptr()), C.c_void_p(dst.data_ptr()), n,
                 C.c_void_p(cnt.data_ptr()), None) == 0
    torch.cuda.synchronize()
    if rank == 0:
        print(json.dumps({"metric": "tour", "ok": True}), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--scale", type=float, default=1.0)
    ap.add_argument("--brick", type=int, nargs=3, default=None)
    ap.add_argument("--threads", type=int, default=0)
    ap.add_argument("--workers", type=int, default=0,
                    help="brick workers per block (4: one block per SM with four groups of 256 threads)")
    ap.add_argument("--dense-iters", type=int, default=20)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="plain workload only (no config1/batch/adjoint/stress/ref_mode keys)")
    ap.add_argument("--workload", default="plain",
                    choices=["plain", "batch", "stress", "tour", "adjoint", "ref", "compaction"])
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")
    if args.impl == "reference":
        run_reference(args, ws, rank)
    elif args.workload == "batch":
        run_batch(args, ws, rank, local)
    elif args.workload == "stress":
        run_stress(args, ws, rank, local)
    elif args.workload == "tour":
        run_tour(args, ws, rank, local)
    elif args.workload == "adjoint":
        run_adjoint(args, ws, rank, local)
    elif args.workload == "ref":
        run_ref_mode(args, ws, rank, local)
    elif args.workload == "compaction":
        run_compaction(args, ws, rank, local)
    else:
        run_ours(args, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
