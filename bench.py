"""Benchmark of the oibvh collision pipeline on one GB300 (or N replicas).

Default workload ("batched"): 512 mesh pairs (noise-displaced icospheres,
triangle counts log-uniform over 1k..1M, 30-70% overlap, 103 M triangles in
all). One step = one frame = one captured CUDA graph (rigid transforms of
every mesh, one refit launch for all trees, one detect of all pairs); the
line also reports the plain path (the same pairs one at a time) and the ratio.

Workload "deforming": two noise-displaced icospheres at
subdivision 8 (1,310,720 triangles, 655,362 vertices each), B placed by a
seeded rigid transform with ~1% of its surface inside A. One step = one
frame = one collision query: per-vertex Gaussian jitter (sigma 1e-3) on both
meshes, refit both trees, BVTT broad phase (entry level 4, expand 3, the
reference demo's settings), triangle narrow phase, pair count on the host.

  value  queries/s with the frame's positions already in HBM
  e2e    queries/s through the public C ABI with HOST buffers: the pinned
         host positions are copied in, and the colliding pairs copied out,
         inside every timed step

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload deforming|plain]

--impl reference times the reference's CPU path (the oracle port; the
reference's compiled sources cannot be built on the GPU host) on all host
cores, one independent frame per thread.
"""
from __future__ import annotations

import argparse
import gc
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

METRIC = "collision queries/s"
UNIT = "queries/s"
ENTRY_LEVEL, EXPAND_LEVELS = 4, 3  # src/main.cpp:284
# DRAM bytes (read + written) per triangle of one k_refit launch, measured with
# ncu on 64 batched pairs (15,520,000 triangles: 372.7 MB read, 452.3 MB written)
REFIT_DRAM_BYTES_PER_TRIANGLE = (372.71e6 + 452.25e6) / 15520000
# DRAM bytes per vertex of one k_transform_multi launch (ncu, 64 batched pairs:
# 124.3 MB read, 74.0 MB written for 7,760,256 vertices)
TRANSFORM_DRAM_BYTES_PER_VERTEX = (124.32e6 + 73.98e6) / 7760256
# DRAM bytes (read + written) of the traversal kernels (k_init_front, k_top and
# the k_walk rounds) of one frame per BVTT node pair tested, measured with ncu
# on 64 batched pairs (206.9 MB per frame, 15,594,052 pairs tested)
TRAVERSAL_DRAM_BYTES_PER_TESTED = (204.71e6 + 1.54e6 + 0.30e6 + 0.30e6) / 15594052


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: the config's frame count, 60 batched, 100 deforming, else 30)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["batched", "precision", "serving", "deforming", "plain"], default="batched")
    ap.add_argument("--rates", default="1000,3000,10000,30000,60000,100000,150000", help="serving: offered query rates (1/s)")
    ap.add_argument("--pool", type=int, default=2000, help="serving: resident meshes")
    ap.add_argument("--budget-gb", type=float, default=16.0, help="serving: device memory budget for query slots")
    ap.add_argument("--pairs", type=int, default=512, help="mesh pairs of the batched workload")
    ap.add_argument("--cpu-seconds", type=float, default=8.0, help="budget of the CPU-baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-subconfigs", action="store_true",
                    help="batched: leave out the served and precision sub-objects")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = {"batched": 60, "deforming": 100}.get(args.workload, 30)
    return args


REF_NOTE = {
    "reference": "the reference's own CPU path (src/cpu/simpleBVH.cpp, src/utils/utils.cpp), compiled unmodified on "
                 "this host from the sources staged under baseline/_ref",
    "port": "the reference's sources are not staged on this host; the oracle's C restatement of its CPU path runs",
}


def reference_cpu():
    """The reference's own CPU path where it is built on this host
    (oracle/_ref, compiled unmodified from its sources), else the oracle's C
    restatement of it: (class with add_mesh / set_positions / detect, kind)."""
    from oracle.oracle import Port, Reference

    if Reference.available():
        return Reference, "reference"
    return Port, "port"


def max_over_ranks(values, dist, device):
    """The max over ranks of each value (the job's time is its slowest
    replica's); `dist` None means a single process."""
    import torch

    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    if dist is not None:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def replicas_value(units_per_rank, world, ms_max):
    """Whole-job throughput of N independent replicas: every rank processed
    `units_per_rank` units; the job took the slowest rank's time."""
    return units_per_rank * world / (ms_max / 1e3)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def make_workload(name):
    from oibvh_gb300 import workloads as W

    return W.deforming() if name == "deforming" else W.plain()


def workload_config(w, args, extra=None):
    m = w.meshes
    cfg = {
        "workload": w.name,
        "meshes": len(m),
        "triangles_per_mesh": [x.n_triangles for x in m],
        "vertices_per_mesh": [x.n_vertices for x in m],
        "entry_level": ENTRY_LEVEL,
        "expand_levels": EXPAND_LEVELS,
        "l2": "flushed between steps (256 MiB write, outside the timed events)",
        "parallelism": f"replicas{args.gpus}",
    }
    if extra:
        cfg.update(extra)
    return cfg


def jitter_frames(w, n_frames, seed=5):
    """Host float32 positions per frame per mesh: rest + N(0, sigma^2), via torch's CPU generator."""
    import torch

    g = torch.Generator().manual_seed(seed)
    frames = []
    for f in range(n_frames):
        per = []
        for m in w.meshes:
            base = torch.from_numpy(m.xyz)
            if w.jitter_sigma:
                x = base + torch.randn(base.shape, generator=g, dtype=torch.float32) * w.jitter_sigma
            else:
                x = base.clone()
            per.append(x.contiguous())
        frames.append(per)
    return frames


# --------------------------------------------------------------------------- clocks
class ClockSampler:
    """SM clock and clock-event reasons sampled every 5 ms through NVML (read
    only), in a thread, while the timed region runs; nvidia-smi (200 ms) when
    the NVML library cannot be loaded."""

    # nvmlClocksEventReasons bits (nvml.h)
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, cuda_index):
        self.index = self._nvml_index(cuda_index)
        self.rows = []
        self.proc = None
        self.thread = None
        self.stop_flag = threading.Event()
        self.nvml = None
        self.source = None

    @staticmethod
    def _nvml_index(cuda_index):
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
        ids = [v.strip() for v in vis.split(",") if v.strip()]
        if ids and cuda_index < len(ids) and ids[cuda_index].isdigit():
            return int(ids[cuda_index])
        return cuda_index

    def _open_nvml(self):
        import ctypes as C

        try:
            lib = C.CDLL("libnvidia-ml.so.1")
            if lib.nvmlInit_v2() != 0:
                return None
            h = C.c_void_p()
            if lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(self.index), C.byref(h)) != 0:
                return None
            reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                lib.nvmlDeviceGetCurrentClocksThrottleReasons
            mx = C.c_uint()
            lib.nvmlDeviceGetMaxClockInfo(h, 1, C.byref(mx))  # NVML_CLOCK_SM
            return lib, h, reasons, mx.value
        except (OSError, AttributeError):
            return None

    def start(self):
        self.nvml = self._open_nvml()
        if self.nvml is not None:
            self.source = "nvml 5 ms"
            self.thread = threading.Thread(target=self._poll_nvml, daemon=True)
            self.thread.start()
            return
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.source = "nvidia-smi 200 ms"
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _poll_nvml(self):
        import ctypes as C

        lib, h, reasons, mx = self.nvml
        clk, r = C.c_uint(), C.c_ulonglong()
        while not self.stop_flag.is_set():
            if lib.nvmlDeviceGetClockInfo(h, 1, C.byref(clk)) == 0 and reasons(h, C.byref(r)) == 0:
                self.rows.append((float(clk.value), float(mx), int(r.value)))
            time.sleep(0.005)

    def _read(self):
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        bits = {v: k for k, v in self.REASONS.items()}
        for line in self.proc.stdout:
            r = [x.strip() for x in line.split(",")]
            try:
                mask = 0
                for k, n in enumerate(names):
                    if len(r) > 4 + k and r[4 + k].lower().startswith("active"):
                        mask |= bits[n]
                self.rows.append((float(r[0]), float(r[1]), mask))
            except (ValueError, IndexError):
                continue

    def stop(self):
        if self.source is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["clock sampling unavailable"]}
        self.stop_flag.set()
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        if self.nvml is not None:
            try:
                self.nvml[0].nvmlShutdown()
            except Exception:
                pass
        rows = list(self.rows)
        sm = [r[0] for r in rows]
        reasons = sorted({n for r in rows for b, n in self.REASONS.items() if r[2] & b})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(r[1] for r in rows) if rows else None,
                "sm_min_mhz": min(sm) if sm else None, "reasons": reasons, "samples": len(sm), "source": self.source}


# --------------------------------------------------------------------------- our arm
def run_ours(args, rank, world, local):
    import torch

    from oibvh_gb300 import DeviceType, OibvhTree, Scene, _native

    torch.cuda.set_device(local)
    dev = local
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    w = make_workload(args.workload)
    n_frames = args.warmup + args.steps
    host_frames = jitter_frames(w, n_frames, seed=5 + rank)
    pinned = [[x.pin_memory() for x in fr] for fr in host_frames]
    # device-resident frames in the library's vertex layout: (x, y, z, 0), 16 B per vertex
    dev_frames = [[torch.nn.functional.pad(x, (0, 1)).contiguous().to(f"cuda:{dev}") for x in fr]
                  for fr in host_frames]
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream

    trees = [OibvhTree(m, device=dev) for m in w.meshes]
    for t in trees:
        t.build(stream=sh)
    sc = Scene(dev)
    for t in trees:
        sc.addOibvhTree(t)
    L = _native.lib()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{dev}")
    for t, x in zip(trees, dev_frames[0]):
        t.set_positions4_device(x.data_ptr())
    sc.refit(stream=sh)
    tuning = sc.autotune(ENTRY_LEVEL, 3)  # the library's autotuner, on the first frame

    def step_calls(f):
        # one call per stage: positions, refit, detect (the reference's sequence)
        for t, x in zip(trees, dev_frames[f]):
            t.set_positions4_device(x.data_ptr())
        sc.refit(stream=sh)
        sc.detectCollision(DeviceType(dev), ENTRY_LEVEL, EXPAND_LEVELS, stream=sh)

    # the same frame as a captured graph: the trees read fixed position buffers
    # that each frame's positions are copied into, then refit + detect replay
    fixed = [torch.empty_like(x) for x in dev_frames[0]]
    for t, x, y in zip(trees, fixed, dev_frames[0]):
        x.copy_(y)
        t.set_positions4_device(x.data_ptr())
    sc.capture_frame(ENTRY_LEVEL, EXPAND_LEVELS, True, stream=sh)

    def step_device(f):
        for x, y in zip(fixed, dev_frames[f]):
            x.copy_(y, non_blocking=True)
        sc.launch_frame(stream=sh)
        sc.finish_frame(stream=sh)

    hit_buf = torch.empty((1 << 22, 4), dtype=torch.int32).pin_memory()
    hit_bytes = [0]
    import ctypes as C

    def step_e2e(f):
        # the public C ABI with host buffers: pinned xyz in (staged into each
        # tree's own buffer, which the captured frame reads), the frame graph,
        # pair records out
        for t, x in zip(trees, pinned[f]):
            _native.check(L.oibvh_tree_set_positions(t.handle, C.cast(C.c_void_p(x.data_ptr()), _native._f32p),
                                                     C.c_void_p(sh)), "oibvh_tree_set_positions")
        _native.check(L.oibvh_scene_launch_frame(sc.handle, C.c_void_p(sh)), "oibvh_scene_launch_frame")
        _native.check(L.oibvh_scene_finish_frame(sc.handle, C.c_void_p(sh)), "oibvh_scene_finish_frame")
        n = L.oibvh_scene_get_int_tri_pair_count(sc.handle)
        got = C.c_uint64()
        cap = min(n, hit_buf.shape[0])
        _native.check(L.oibvh_scene_get_int_tri_pairs(sc.handle, C.cast(C.c_void_p(hit_buf.data_ptr()), _native._u32p),
                                                      cap, C.byref(got)), "oibvh_scene_get_int_tri_pairs")
        hit_bytes[0] += 16 * cap

    def timed(step_fn):
        for f in range(args.warmup):
            step_fn(f)
        barrier()
        flush.fill_(1)
        barrier()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        launches0 = L.oibvh_get_launch_count()
        wall0 = time.perf_counter()
        for k in range(args.steps):
            flush.fill_(k & 255)  # evict L2 between steps, outside the events
            starts[k].record(stream)
            step_fn(args.warmup + k)
            ends[k].record(stream)
        barrier()
        wall = time.perf_counter() - wall0
        launches = L.oibvh_get_launch_count() - launches0
        ms = sum(s.elapsed_time(e) for s, e in zip(starts, ends))
        return ms, wall, launches

    sampler = ClockSampler(dev) if rank == 0 else None
    if sampler:
        sampler.start()
    ms_dev, wall_dev, launches = timed(step_device)
    stats = sc.stats()
    hits = sc.getIntTriPairCount()
    cands = sc.candidate_count()
    ms_calls, _, _ = timed(step_calls)
    hit_bytes[0] = 0
    # the trees read their own position buffers from here on: capture for them
    for t, x in zip(trees, pinned[0]):
        _native.check(L.oibvh_tree_set_positions(t.handle, C.cast(C.c_void_p(x.data_ptr()), _native._f32p),
                                                 C.c_void_p(sh)), "oibvh_tree_set_positions")
    sc.capture_frame(ENTRY_LEVEL, EXPAND_LEVELS, True, stream=sh)
    ms_e2e, wall_e2e, _ = timed(step_e2e)
    clocks = sampler.stop() if sampler else None

    # dominant HBM kernel (the one-launch refit of both trees) timed alone on the same stream:
    # positions converted into the trees' own buffers first, so each refit is the one kernel
    xyz0 = [x[:, :3].contiguous() for x in dev_frames[0]]
    for t, x in zip(trees, xyz0):
        t.set_positions_device(x.data_ptr(), stream=sh)
    rf_s = [torch.cuda.Event(enable_timing=True) for _ in range(20)]
    rf_e = [torch.cuda.Event(enable_timing=True) for _ in range(20)]
    for k in range(20):
        flush.fill_(k & 255)
        rf_s[k].record(stream)
        sc.refit(stream=sh)
        rf_e[k].record(stream)
    torch.cuda.synchronize()
    refit_ms = statistics.mean(s.elapsed_time(e) for s, e in zip(rf_s, rf_e))

    # max over ranks
    ms_dev, ms_e2e = max_over_ranks([ms_dev, ms_e2e], dist, f"cuda:{dev}")
    if dist is not None:
        dist.destroy_process_group()
    if rank != 0:
        return None

    K = args.steps
    queries = K * world
    value = replicas_value(K, world, ms_dev)
    e2e = queries / (ms_e2e / 1e3)
    tri_total = sum(m.n_triangles for m in w.meshes)
    V = sum(m.n_vertices for m in w.meshes)
    # refit algorithmic bytes per launch (both trees): per tree 12 B per vertex
    # read, 12 B per face read, 24 B per node written (compulsory bytes of the
    # reference layout: xyz vertices, uint32x3 faces, 6-float boxes)
    def tree_size(T):
        p = 1 << (T - 1).bit_length()
        return 2 * T + bin(p - T).count("1") - 1
    refit_bytes = sum(12 * m.n_vertices + 12 * m.n_triangles + 24 * tree_size(m.n_triangles) for m in w.meshes)
    peaks = load_peaks()
    achieved = refit_bytes / (refit_ms / 1e3) / 1e9
    line = {
        "metric": METRIC,
        "value": round(value, 3),
        "unit": UNIT,
        "n_gpus": world,
        "steps": K,
        "warmup": args.warmup,
        "ms_per_step": round(ms_dev / K, 5),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded noise icospheres, per-frame Gaussian jitter)",
        "config": workload_config(w, args, {"tuning": tuning, "frame": "positions copied into the trees' "
                                            "buffers, then refit + detect as one captured CUDA graph"}),
        "one_call_per_stage": {"ms_per_step": round(ms_calls / args.steps, 5),
                               "queries_per_s": round(args.steps * world / (ms_calls / 1e3), 3)},
        "tri_pairs_per_s": round(cands * queries / (ms_dev / 1e3), 1),
        "triangles_per_s": round(tri_total * queries / (ms_dev / 1e3), 1),
        "hits_last_frame": hits,
        "candidates_last_frame": cands,
        "bvtt_nodes_last_frame": stats["nodes_tested"],
        "e2e": {"value": round(e2e, 3), "unit": UNIT, "h2d_bytes_per_step": 12 * V,
                "d2h_bytes_per_step": int(hit_bytes[0] / max(1, K)), "ms_per_step": round(ms_e2e / K, 5)},
        "roofline": {"kernel": "k_refit (one launch: both trees, leaf boxes + every level)", "bound": "hbm",
                     "achieved": round(achieved, 1), "peak": peaks[0], "unit": "GB/s",
                     "frac": round(achieved / peaks[0], 4), "peak_source": peaks[1],
                     "algorithmic_bytes_per_launch": refit_bytes, "launch_ms": round(refit_ms, 5),
                     "traffic": None},
        "gpu_launches": int(launches),
        "clocks": clocks,
        "wall_s": round(wall_dev, 3),
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_sample(w, args.cpu_seconds)
    return line


def ctypes_f32(t):
    import ctypes

    return ctypes.cast(ctypes.c_void_p(t.data_ptr()), ctypes.POINTER(ctypes.c_float))


def ctypes_stream(h):
    import ctypes

    return ctypes.c_void_p(h)


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (of measured)"
    except Exception:
        return 6800.0, "fallback 6.8 TB/s (of fallback)"


# --------------------------------------------------------------------------- CPU
def cpu_baseline_sample(w, seconds, threads=1):
    """The oracle port (C restatement of the reference CPU path) on this host:
    one frame = refit both SimpleBVHs to the frame's positions + detect."""
    Ref, ref_kind = reference_cpu()

    frames = jitter_frames(w, 64, seed=99)

    def worker(out, idx0, stride, deadline):
        p = Ref()
        for m in w.meshes:
            p.add_mesh(m.xyz, m.tri)
        n = 0
        f = idx0
        while time.perf_counter() < deadline or n == 0:
            fr = frames[f % len(frames)]
            for i, x in enumerate(fr):
                p.set_positions(i, x.numpy())
            p.detect()
            n += 1
            f += stride
        out.append(n)

    out = []
    # build (not timed) happens inside the workers; give it a head start
    t0 = time.perf_counter()
    deadline = t0 + seconds
    ths = [threading.Thread(target=worker, args=(out, k, threads, deadline)) for k in range(threads)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()
    el = time.perf_counter() - t0
    n = sum(out)
    return {"value": round(n / el, 3), "unit": UNIT, "cores": threads, "kind": ref_kind,
            "sample": f"{n} frames of the workload (refit both + detect) in {el:.1f} s, build included"}


def run_reference(args, rank, world):
    """The reference arm: the reference CPU path (oracle port) on all host cores."""
    if rank != 0:
        return None
    w = make_workload(args.workload)
    threads = os.cpu_count() or 1
    Ref, ref_kind = reference_cpu()

    frames = jitter_frames(w, max(8, threads), seed=5)
    scenes = [None] * threads

    def setup(k):
        p = Ref()
        for m in w.meshes:
            p.add_mesh(m.xyz, m.tri)
        scenes[k] = p

    ths = [threading.Thread(target=setup, args=(k,)) for k in range(threads)]
    for t in ths:
        t.start()
    for t in ths:
        t.join()

    def one_step(step):
        def work(k):
            fr = frames[(step * threads + k) % len(frames)]
            for i, x in enumerate(fr):
                scenes[k].set_positions(i, x.numpy())
            scenes[k].detect()

        ts = [threading.Thread(target=work, args=(k,)) for k in range(threads)]
        for t in ts:
            t.start()
        for t in ts:
            t.join()

    for s in range(args.warmup):
        one_step(s)
    t0 = time.perf_counter()
    for s in range(args.steps):
        one_step(args.warmup + s)
    el = time.perf_counter() - t0
    q = args.steps * threads
    value = q / el
    return {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 * el / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded noise icospheres, per-frame Gaussian jitter)",
        "config": workload_config(w, args, {"parallelism": f"{threads} host threads, one frame each per step"}),
        "impl": "reference",
        "cpu_baseline": {"value": round(value, 3), "unit": UNIT, "cores": threads, "kind": ref_kind,
                         "sample": f"{q} frames (refit both + detect), {threads} per step"},
        "e2e": {"value": round(value, 3), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": REF_NOTE[ref_kind],
    }


# --------------------------------------------------------------------------- batched workload
def batched_workload(args):
    from oibvh_gb300 import workloads as W

    return W.batched(args.pairs)


def run_ours_batched(args, rank, world, local):
    """512 mesh pairs (T log-uniform 1k..1M), every frame a captured CUDA graph:
    device rigid transforms of all meshes, one refit launch for all trees, one
    detect of all pairs. Compared with the plain path: the same pairs one at a
    time (per pair: transform, refit, detect), same device-resident inputs."""
    import ctypes as C

    import torch

    from oibvh_gb300 import DeviceType, OibvhTree, Scene, _native

    torch.cuda.set_device(local)
    dev = local
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    t_setup = time.perf_counter()
    w = batched_workload(args)
    n_frames = args.warmup + args.steps
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    L = _native.lib()
    trees = [OibvhTree(m, device=dev) for m in w.rest]
    sc = Scene(dev)
    for t in trees:
        sc.addOibvhTree(t)
    sc.set_pairs(w.pairs)
    rest = torch.from_numpy(w.packed_rest_xyzw()).to(f"cuda:{dev}")
    mats_all = torch.from_numpy(np.stack([w.matrices(f) for f in range(n_frames)])).to(f"cuda:{dev}")
    mats_pinned = torch.from_numpy(np.stack([w.matrices(f) for f in range(n_frames)])).pin_memory()
    mats = mats_all[0].clone()
    torch.cuda.synchronize()
    tb = time.perf_counter()
    sc.build(stream=sh)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - tb
    sc.transform(rest.data_ptr(), mats.data_ptr(), stream=sh)
    sc.refit(stream=sh)
    tuning = sc.autotune(ENTRY_LEVEL, 3)
    sc.capture_frame(ENTRY_LEVEL, EXPAND_LEVELS, True, rest.data_ptr(), mats.data_ptr(), stream=sh)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{dev}")
    setup_s = time.perf_counter() - t_setup

    def step_device(f):
        mats.copy_(mats_all[f], non_blocking=True)
        sc.launch_frame(stream=sh)
        sc.finish_frame(stream=sh)

    hit_buf = torch.empty((1 << 24, 4), dtype=torch.int32).pin_memory()
    d2h = [0]

    def step_e2e(f):
        mats.copy_(mats_pinned[f], non_blocking=True)  # this frame's transforms from pinned host memory
        sc.launch_frame(stream=sh)
        sc.finish_frame(stream=sh)
        n = sc.getIntTriPairCount()
        got = C.c_uint64()
        cap = min(n, hit_buf.shape[0])
        _native.check(L.oibvh_scene_get_int_tri_pairs(sc.handle, C.cast(C.c_void_p(hit_buf.data_ptr()), _native._u32p),
                                                      cap, C.byref(got)), "oibvh_scene_get_int_tri_pairs")
        d2h[0] += 16 * cap

    def timed(step_fn, steps):
        for f in range(args.warmup):
            step_fn(f)
        barrier()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        l0 = L.oibvh_get_launch_count()
        for k in range(steps):
            flush.fill_(k & 255)  # evict L2 between steps, outside the events
            starts[k].record(stream)
            step_fn(args.warmup + k)
            ends[k].record(stream)
        barrier()
        return sum(s_.elapsed_time(e) for s_, e in zip(starts, ends)), L.oibvh_get_launch_count() - l0

    sampler = ClockSampler(dev) if rank == 0 else None
    if sampler:
        sampler.start()
    redos0 = sc.stats()["frame_redos"]
    ms_dev, launches = timed(step_device, args.steps)
    stats = sc.stats()
    redos = stats["frame_redos"] - redos0
    hits = sc.getIntTriPairCount()
    cands = sc.candidate_count()
    ms_e2e, _ = timed(step_e2e, args.steps)
    clocks = sampler.stop() if sampler else None

    # the plain single-pair path over the same pairs and inputs (one frame)
    plain = []
    for p, (a, b) in enumerate(w.pairs):
        ps = Scene(dev)
        ps.addOibvhTree(trees[a])
        ps.addOibvhTree(trees[b])
        plain.append(ps)
    offs = np.concatenate([[0], np.cumsum([m.n_vertices for m in w.rest])])
    mats.copy_(mats_all[0])

    def plain_frame():
        for p, (a, b) in enumerate(w.pairs):
            plain[p].transform(rest.data_ptr() + 16 * int(offs[a]), mats.data_ptr() + 48 * a, stream=sh)
            plain[p].refit(stream=sh)
            plain[p].detectCollision(DeviceType(dev), ENTRY_LEVEL, EXPAND_LEVELS, stream=sh)

    plain_frame()
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    plain_frames = 2
    ev0.record(stream)
    for _ in range(plain_frames):
        plain_frame()
    ev1.record(stream)
    torch.cuda.synchronize()
    plain_ms = ev0.elapsed_time(ev1) / plain_frames
    plain_hits = sum(ps.getIntTriPairCount() for ps in plain)

    # every stage of the frame timed on its own: the same kernels, enqueued
    # stage by stage with CUDA events between the stages (L2 flushed before each)
    profs = []
    for k in range(10):
        flush.fill_(k & 255)
        mats.copy_(mats_all[k % n_frames])
        torch.cuda.nvtx.range_push("profile_frame")  # selects these launches for an ncu capture
        profs.append(sc.profile_frame(stream=sh))
        torch.cuda.nvtx.range_pop()
    prof = {key: statistics.median(p_[key] for p_ in profs)
            for key in ("transform_ms", "refit_ms", "start_ms", "walk_ms", "narrow_ms")}
    prof_hits, prof_cands = sc.getIntTriPairCount(), sc.candidate_count()
    prof_tested = sc.stats()["nodes_tested"]

    # the one-launch refit of all 1024 trees, also timed alone
    rf = []
    for k in range(10):
        flush.fill_(k & 255)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        sc.refit(stream=sh)
        e1.record(stream)
        torch.cuda.synchronize()
        rf.append(e0.elapsed_time(e1))
    refit_ms = statistics.median(rf)

    ms_dev, ms_e2e = max_over_ranks([ms_dev, ms_e2e], dist, f"cuda:{dev}")
    if dist is not None:
        dist.destroy_process_group()
    if rank != 0:
        return None

    K = args.steps
    n_pairs = len(w.pairs)
    queries = K * n_pairs * world
    value = replicas_value(K * n_pairs, world, ms_dev)

    def tree_size(T):
        p2 = 1 << (T - 1).bit_length()
        return 2 * T + bin(p2 - T).count("1") - 1

    refit_bytes = sum(12 * m.n_vertices + 12 * m.n_triangles + 24 * tree_size(m.n_triangles) for m in w.rest)
    peaks = load_peaks()
    achieved = refit_bytes / (refit_ms / 1e3) / 1e9
    rooflines = frame_rooflines(w, prof, prof_cands, prof_hits, prof_tested, peaks, refit_ms, refit_bytes, ms_dev / K)
    line = {
        "metric": "collision queries/s (mesh pairs through refit + broad + narrow)",
        "value": round(value, 1),
        "unit": "queries/s",
        "n_gpus": world,
        "steps": K,
        "warmup": args.warmup,
        "ms_per_step": round(ms_dev / K, 4),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded noise icospheres, per-frame rigid motion)",
        "config": {"workload": w.name, **w.info, "entry_level": ENTRY_LEVEL, "expand_levels": EXPAND_LEVELS,
                   "frame": "one captured CUDA graph: transform all meshes + refit all trees + detect all pairs",
                   "tuning": tuning, "l2": "flushed between steps (256 MiB write, outside the timed events)",
                   "parallelism": f"replicas{world}"},
        "plain_single_pair": {"queries_per_s": round(n_pairs / (plain_ms / 1e3), 1), "ms_per_frame": round(plain_ms, 3),
                              "how": "same pairs and inputs, one pair per call: transform + refit + detect",
                              "hits_per_frame": plain_hits},
        "batched_over_plain": round(value / (n_pairs / (plain_ms / 1e3)), 2),
        "tri_pairs_per_s": round(cands * K * world / (ms_dev / 1e3), 1),
        "triangles_per_s": round(w.info["triangles_total"] * K * world / (ms_dev / 1e3), 1),
        "hits_last_frame": hits,
        "candidates_last_frame": cands,
        "bvtt_pairs_tested_last_frame": stats["nodes_tested"],
        "walk_rounds_captured": stats["steps"],
        "frames_redone": redos,
        "e2e": {"value": round(queries / (ms_e2e / 1e3), 1), "unit": "queries/s",
                "h2d_bytes_per_step": 48 * len(w.rest), "d2h_bytes_per_step": int(d2h[0] / max(1, K)),
                "ms_per_step": round(ms_e2e / K, 4)},
        "roofline": rooflines,
        "gpu_launches": int(launches),
        "clocks": clocks,
        "setup_s": round(setup_s, 2),
        "scene_build_s": round(build_s, 3),
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_batched(w, args.cpu_seconds)
    return line


def _tree_size(T):
    """Real nodes of an oibvh tree of T leaves (include/cuda/oibvh.cuh:56-59)."""
    p2 = 1 << (T - 1).bit_length()
    return 2 * T + bin(p2 - T).count("1") - 1


def frame_rooflines(w, prof, cands, hits, tested, peaks, refit_alone_ms, refit_bytes, ms_step):
    """HBM roofline of every stage of one batched frame, each timed inside
    the frame (CUDA events between the stages). Algorithmic bytes follow the
    compulsory-traffic rule of the reference layout: refit 12 B per vertex +
    12 B per face read and 24 B per tree node written; traversal 24 B per
    node of both trees of every pair (broad phase in), 8 B per candidate out,
    104 B per candidate in (narrow phase: the candidate, two faces, six
    vertices) and 8 B per hit out; transform 16 B in + 16 B out per vertex.
    `traffic` is the DRAM bytes ncu measured for the stage on a smaller case,
    scaled by the units it processes; `frac_dram` = traffic / time / peak."""
    peak, src = peaks
    tri_total = w.info["triangles_total"]
    broad = sum(24 * (_tree_size(w.rest[a].n_triangles) + _tree_size(w.rest[b].n_triangles)) for a, b in w.pairs)
    stages = {
        "transform": ("k_transform_multi (one launch: every vertex of every mesh)",
                      sum(32 * m.n_vertices + 48 for m in w.rest), prof["transform_ms"],
                      TRANSFORM_DRAM_BYTES_PER_VERTEX * w.info["vertices_total"],
                      "16 B in + 16 B out per vertex, 48 B of matrix per mesh"),
        "refit": ("k_refit (one launch: all trees, leaf boxes + every level)", refit_bytes, prof["refit_ms"],
                  REFIT_DRAM_BYTES_PER_TRIANGLE * tri_total,
                  "12 B per vertex + 12 B per face read, 24 B per tree node written (the reference layout; this "
                  "layout stores internal nodes only, 32 B each, and reads 16 B per face and per vertex)"),
        "traversal": ("k_init_front + k_top + k_walk rounds (broad phase, fused 17-axis narrow phase)",
                      broad + 112 * cands + 8 * hits, prof["start_ms"] + prof["walk_ms"],
                      TRAVERSAL_DRAM_BYTES_PER_TESTED * tested if TRAVERSAL_DRAM_BYTES_PER_TESTED else None,
                      "24 B per node of both trees of every pair + 112 B per candidate + 8 B per hit"),
    }
    out = {}
    for name, (kern, b, ms, traffic, rule) in stages.items():
        ach = b / (ms / 1e3) / 1e9
        e = {"kernel": kern, "bound": "hbm", "achieved": round(ach, 1), "peak": peak, "unit": "GB/s",
             "frac": round(ach / peak, 4), "traffic": int(traffic) if traffic else None,
             "algorithmic_bytes_per_launch": int(b), "launch_ms": round(ms, 4),
             "share_of_step": round(ms / ms_step, 4), "bytes_rule": rule}
        if traffic:
            e["frac_dram"] = round(traffic / (ms / 1e3) / 1e9 / peak, 4)
        out[name] = e
    out["refit"]["frac_effective"] = out["refit"]["frac"]
    out["refit"]["alone_ms"] = round(refit_alone_ms, 4)
    dominant = max(("transform", "refit", "traversal"), key=lambda k: out[k]["launch_ms"])
    top = dict(out[dominant])
    top.update({"stage": dominant, "peak_source": src, "stages": out,
                "stages_ms_sum": round(sum(prof[k] for k in ("transform_ms", "refit_ms", "start_ms", "walk_ms")), 4),
                "stages_cover_of_step": round(sum(out[k]["launch_ms"] for k in out) / ms_step, 4),
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum per stage on 64 batched pairs "
                                  "(profiles/), scaled by the units the stage processes",
                "bvtt_pairs_tested": tested, "candidates": cands, "hits": hits})
    return top


def _sample_pairs(w, n):
    step = max(1, len(w.pairs) // n)
    return list(range(0, len(w.pairs), step))[:n]


def _sample_positions(w, sample, frames):
    """{frame: {mesh: xyz}} for the meshes of the sampled pairs only."""
    need = sorted({m for p in sample for m in w.pairs[p]})
    return {f: dict(zip(need, w.positions(f, need))) for f in frames}


def cpu_baseline_batched(w, seconds, threads=1, frames=(1, 2, 3, 4)):
    """The oracle port on this host: for a fixed sample of the pairs, refit both
    SimpleBVHs to the frame's transformed positions and detect, pair by pair."""
    Ref, ref_kind = reference_cpu()

    sample = _sample_pairs(w, 32)
    pos = _sample_positions(w, sample, frames)
    scenes = []
    for p in sample:
        a, b = w.pairs[p]
        ps = Ref()
        ps.add_mesh(pos[frames[0]][a], w.rest[a].tri)
        ps.add_mesh(pos[frames[0]][b], w.rest[b].tri)
        scenes.append((ps, a, b))
    t0 = time.perf_counter()
    n = 0
    k = 0
    while time.perf_counter() - t0 < seconds or n == 0:
        f = frames[k % len(frames)]
        ps, a, b = scenes[n % len(scenes)]
        ps.set_positions(0, pos[f][a])
        ps.set_positions(1, pos[f][b])
        ps.detect()
        n += 1
        if n % len(scenes) == 0:
            k += 1
    el = time.perf_counter() - t0
    return {"value": round(n / el, 3), "unit": "queries/s", "cores": threads, "kind": ref_kind,
            "sample": f"{n} pair queries (refit both + detect) over a fixed sample of {len(sample)} pairs, {el:.1f} s"}


def run_reference_batched(args, rank, world):
    """The reference CPU path (oracle port) on every host core: each step runs a
    bounded sample of the workload, 8 pair queries per thread."""
    if rank != 0:
        return None
    Ref, ref_kind = reference_cpu()

    w = batched_workload(args)
    threads = os.cpu_count() or 1
    sample = _sample_pairs(w, 8 * threads)
    frames = list(range(1, 5))
    pos = _sample_positions(w, sample, frames)
    per = [[] for _ in range(threads)]
    for i, p in enumerate(sample):
        per[i % threads].append(p)
    scenes = [None] * threads

    def setup(k):
        lst = []
        for p in per[k]:
            a, b = w.pairs[p]
            ps = Ref()
            ps.add_mesh(pos[1][a], w.rest[a].tri)
            ps.add_mesh(pos[1][b], w.rest[b].tri)
            lst.append((ps, a, b))
        scenes[k] = lst

    ts = [threading.Thread(target=setup, args=(k,)) for k in range(threads)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()

    def one_step(step):
        f = frames[step % len(frames)]

        def work(k):
            for ps, a, b in scenes[k]:
                ps.set_positions(0, pos[f][a])
                ps.set_positions(1, pos[f][b])
                ps.detect()

        tt = [threading.Thread(target=work, args=(k,)) for k in range(threads)]
        for t in tt:
            t.start()
        for t in tt:
            t.join()

    for s_ in range(args.warmup):
        one_step(s_)
    t0 = time.perf_counter()
    for s_ in range(args.steps):
        one_step(args.warmup + s_)
    el = time.perf_counter() - t0
    q = args.steps * len(sample)
    value = q / el
    return {
        "metric": "collision queries/s (mesh pairs through refit + broad + narrow)", "value": round(value, 3),
        "unit": "queries/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * el / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded noise icospheres, per-frame rigid motion)",
        "config": {"workload": w.name, **w.info,
                   "parallelism": f"{threads} host threads; each step: {len(sample)} sampled pairs, 8 per thread"},
        "impl": "reference",
        "cpu_baseline": {"value": round(value, 3), "unit": "queries/s", "cores": threads, "kind": ref_kind,
                         "sample": f"{q} pair queries over a fixed sample of {len(sample)} of the {len(w.pairs)} pairs"},
        "e2e": {"value": round(value, 3), "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": REF_NOTE[ref_kind],
    }


# --------------------------------------------------------------------------- precision workload
def _pctl(xs, q):
    xs = sorted(xs)
    if not xs:
        return None
    k = min(len(xs) - 1, max(0, int(round(q / 100.0 * (len(xs) - 1)))))
    return xs[k]


def run_ours_precision(args, rank, world, local):
    """64 pairs of 256x256-quad sine sheets, 10% of B's triangles coplanar
    with A's or within 1e-7: every frame (identity rigid transforms uploaded,
    transform + refit + detect as one captured CUDA graph) runs the
    FP64-filtered triangle test. Reported beside it: the same frame with the
    reference's float test, the float/FP64 disagreement count, frame latency
    percentiles, and the plain path (one pair per call) with its per-query
    latency percentiles."""
    import ctypes as C

    import torch

    from oibvh_gb300 import DeviceType, OibvhTree, Scene, _native
    from oibvh_gb300 import workloads as W

    torch.cuda.set_device(local)
    dev = local
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    w = W.sheets(args.pairs if args.pairs != 512 else 64, 256)
    n_pairs = len(w.pairs)
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream
    L = _native.lib()
    trees = [OibvhTree(m, device=dev) for m in w.meshes]
    sc = Scene(dev)
    for t in trees:
        sc.addOibvhTree(t)
    sc.set_pairs(w.pairs)
    rest = torch.from_numpy(np.concatenate([np.pad(m.xyz, ((0, 0), (0, 1))) for m in w.meshes], 0)).to(f"cuda:{dev}")
    ident = np.tile(np.array([1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0], dtype=np.float32), (len(w.meshes), 1))
    mats = torch.from_numpy(ident).to(f"cuda:{dev}")
    mats_pinned = torch.from_numpy(ident).pin_memory()
    sc.build(stream=sh)
    sc.transform(rest.data_ptr(), mats.data_ptr(), stream=sh)
    sc.refit(stream=sh)
    sc.set_precision(_native.PRECISION_FP64_FILTERED)
    tuning = sc.autotune(ENTRY_LEVEL, 3)  # the library's autotuner, on the first frame (FP64-filtered)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{dev}")
    hit_buf = torch.empty((1 << 24, 4), dtype=torch.int32).pin_memory()

    def measure(mode, steps, e2e=False):
        sc.set_precision(mode)
        sc.capture_frame(ENTRY_LEVEL, EXPAND_LEVELS, True, rest.data_ptr(), mats.data_ptr(), stream=sh)
        d2h = 0
        for _ in range(args.warmup):
            sc.launch_frame(stream=sh)
            sc.finish_frame(stream=sh)
        barrier()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
        lat = []
        l0 = L.oibvh_get_launch_count()
        for k in range(steps):
            flush.fill_(k & 255)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            starts[k].record(stream)
            if e2e:
                mats.copy_(mats_pinned, non_blocking=True)
            sc.launch_frame(stream=sh)
            sc.finish_frame(stream=sh)
            if e2e:
                n = sc.getIntTriPairCount()
                got = C.c_uint64()
                cap = min(n, hit_buf.shape[0])
                _native.check(L.oibvh_scene_get_int_tri_pairs(
                    sc.handle, C.cast(C.c_void_p(hit_buf.data_ptr()), _native._u32p), cap, C.byref(got)),
                    "oibvh_scene_get_int_tri_pairs")
                d2h += 16 * cap
            ends[k].record(stream)
            lat.append(1e3 * (time.perf_counter() - t0))
        barrier()
        ms = sum(a.elapsed_time(b) for a, b in zip(starts, ends))
        return ms, lat, L.oibvh_get_launch_count() - l0, sc.stats(), d2h

    sampler = ClockSampler(dev) if rank == 0 else None
    if sampler:
        sampler.start()
    ms_f, lat_f, launches, st_f, _ = measure(_native.PRECISION_FP64_FILTERED, args.steps)
    hits = sc.getIntTriPairCount()
    ms_e2e, lat_e2e, _, _, d2h = measure(_native.PRECISION_FP64_FILTERED, args.steps, e2e=True)
    clocks = sampler.stop() if sampler else None
    got_f = sc.int_tri_pairs() if not args.no_cpu_baseline else None
    got_f_all = sc.int_tri_pairs() if got_f is None else got_f
    ms_32, lat_32, _, st_32, _ = measure(_native.PRECISION_FP32, max(3, args.steps // 2))
    hits32 = sc.getIntTriPairCount()
    got_32 = sc.int_tri_pairs()
    # float vs FP64 disagreements per pair: symmetric difference of the two pair sets
    def keyed(recs, a_, b_):
        r = recs[(recs[:, 0] == a_) & (recs[:, 1] == b_)]
        return (r[:, 2].astype(np.int64) << 32) | r[:, 3].astype(np.int64)

    per_pair = [int(np.setxor1d(keyed(got_f_all, a_, b_), keyed(got_32, a_, b_)).size) for a_, b_ in w.pairs]

    # the plain path: one pair per call (refit both trees + detect), each query alone
    plain = []
    for a, b in w.pairs:
        ps = Scene(dev)
        ps.addOibvhTree(trees[a])
        ps.addOibvhTree(trees[b])
        ps.set_precision(_native.PRECISION_FP64_FILTERED)
        plain.append(ps)
    for ps in plain:
        ps.refit(stream=sh)
        ps.detectCollision(DeviceType(dev), ENTRY_LEVEL, EXPAND_LEVELS, stream=sh)
    barrier()
    q_lat = []
    tp0 = time.perf_counter()
    for rep in range(3):
        for ps in plain:
            t0 = time.perf_counter()
            ps.refit(stream=sh)
            ps.detectCollision(DeviceType(dev), ENTRY_LEVEL, EXPAND_LEVELS, stream=sh)
            ps.getIntTriPairCount()
            q_lat.append(1e3 * (time.perf_counter() - t0))
    plain_s = (time.perf_counter() - tp0) / 3
    plain_hits = sum(ps.getIntTriPairCount() for ps in plain)
    # the float arithmetic (the reference's), one pair per call, on the sample
    # of pairs the reference's GPU kernels are timed on (REF_GPU_SAMPLE)
    q_lat32 = []
    for p in _sample_pairs(w, REF_GPU_SAMPLE):
        ps = plain[p]
        ps.set_precision(_native.PRECISION_FP32)
        for rep_ in range(4):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ps.refit(stream=sh)
            ps.detectCollision(DeviceType(dev), ENTRY_LEVEL, EXPAND_LEVELS, stream=sh)
            ps.getIntTriPairCount()
            if rep_:
                q_lat32.append(1e3 * (time.perf_counter() - t0))
        ps.set_precision(_native.PRECISION_FP64_FILTERED)

    ms_f, ms_e2e = max_over_ranks([ms_f, ms_e2e], dist, f"cuda:{dev}")
    if dist is not None:
        dist.destroy_process_group()
    if rank != 0:
        return None
    K = args.steps
    value = replicas_value(K * n_pairs, world, ms_f)
    line = {
        "metric": "collision queries/s (mesh pairs through refit + broad + narrow), FP64-filtered triangle test",
        "value": round(value, 1), "unit": "queries/s", "n_gpus": world, "steps": K, "warmup": args.warmup,
        "ms_per_step": round(ms_f / K, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 + f64 (filtered)", "data": "synthetic (seeded sine sheets)",
        "config": {"workload": w.name, **w.info, "entry_level": ENTRY_LEVEL, "expand_levels": EXPAND_LEVELS,
                   "frame": "one captured CUDA graph: identity transforms + refit all sheets + detect all pairs",
                   "tuning": tuning,
                   "l2": "flushed between steps (256 MiB write, outside the timed events)",
                   "parallelism": f"replicas{world}"},
        "frame_latency_ms": {"p50": round(_pctl(lat_f, 50), 4), "p99": round(_pctl(lat_f, 99), 4),
                             "max": round(max(lat_f), 4), "how": "host wall clock, launch to results on the host; "
                             "every query of a frame completes with it"},
        "fp64_filter": {"candidates": st_f["candidates"], "fp64_candidates": st_f["fp64_candidates"],
                        "fp64_axes": st_f["fp64_axes"], "fp32_disagreements": st_f["fp32_disagreements"],
                        "hits_fp64": hits, "hits_fp32": hits32,
                        "fp32_vs_fp64_disagreements_per_pair": per_pair,
                        "pairs_with_disagreements": sum(1 for x in per_pair if x)},
        "fp32_frame": {"queries_per_s": round(max(3, K // 2) * n_pairs / (ms_32 / 1e3), 1),
                       "ms_per_frame": round(ms_32 / max(3, K // 2), 4),
                       "latency_p99_ms": round(_pctl(lat_32, 99), 4)},
        "plain_single_pair": {"queries_per_s": round(n_pairs / plain_s, 1),
                              "latency_ms": {"p50": round(_pctl(q_lat, 50), 4), "p99": round(_pctl(q_lat, 99), 4)},
                              "how": "each pair its own scene: refit both trees + detect, synchronous, FP64-filtered",
                              "hits": plain_hits},
        "batched_over_plain": round(value / (n_pairs / plain_s), 2),
        "plain_single_pair_fp32": {"ms_per_query": {"p50": round(_pctl(q_lat32, 50), 4),
                                                    "p99": round(_pctl(q_lat32, 99), 4)},
                                   "how": f"float test, one pair per call (refit both + detect), "
                                          f"{REF_GPU_SAMPLE} sampled pairs x 3"},
        "e2e": {"value": round(K * n_pairs * world / (ms_e2e / 1e3), 1), "unit": "queries/s",
                "h2d_bytes_per_step": int(mats_pinned.numel() * 4), "d2h_bytes_per_step": int(d2h / max(1, K)),
                "latency_ms": {"p50": round(_pctl(lat_e2e, 50), 4), "p99": round(_pctl(lat_e2e, 99), 4)}},
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_precision(w, got_f, args.cpu_seconds)
        line["fp64_oracle"] = fp64_oracle_all_pairs(w, got_f, min(16, os.cpu_count() or 1))
    return line


def fp64_oracle_all_pairs(w, got, threads):
    """The all-FP64 oracle over EVERY pair of the workload on `threads` host
    threads (outside any timed region): pair-set mismatches against the
    GPU's FP64-filtered result, summed over the pairs."""
    from oracle.oracle import Port

    mism = [0] * len(w.pairs)

    def work(k):
        for p in range(k, len(w.pairs), threads):
            a, b = w.pairs[p]
            port = Port()
            port.add_mesh(w.meshes[a].xyz, w.meshes[a].tri)
            port.add_mesh(w.meshes[b].xyz, w.meshes[b].tri)
            h64, _ = port.detect(fp64=True)
            mine = got[(got[:, 0] == a) & (got[:, 1] == b)][:, 2:]
            mism[p] = len({tuple(r) for r in h64[:, 2:].tolist()} ^ {tuple(r) for r in mine.tolist()})

    t0 = time.perf_counter()
    ts = [threading.Thread(target=work, args=(k,)) for k in range(threads)]
    for t in ts:
        t.start()
    for t in ts:
        t.join()
    return {"fp64_oracle_mismatches": int(sum(mism)), "pairs_checked": len(w.pairs),
            "pairs_with_mismatches": sum(1 for x in mism if x), "threads": threads,
            "seconds": round(time.perf_counter() - t0, 1)}


def cpu_baseline_precision(w, got, seconds):
    """The FP64 oracle on this host (1 core) over a sample of the pairs, each
    pair set compared with the GPU's filtered result for that pair."""
    from oracle.oracle import Port

    t0 = time.perf_counter()
    n = 0
    mismatches = 0
    checked = []
    for p in _sample_pairs(w, len(w.pairs)):
        a, b = w.pairs[p]
        port = Port()
        port.add_mesh(w.meshes[a].xyz, w.meshes[a].tri)
        port.add_mesh(w.meshes[b].xyz, w.meshes[b].tri)
        h64, _ = port.detect(fp64=True)
        n += 1
        mine = got[(got[:, 0] == a) & (got[:, 1] == b)][:, 2:]
        want = {tuple(r) for r in h64[:, 2:].tolist()}
        have = {tuple(r) for r in mine.tolist()}
        mismatches += len(want ^ have)
        checked.append(p)
        if time.perf_counter() - t0 > seconds:
            break
    el = time.perf_counter() - t0
    return {"value": round(n / el, 3), "unit": "queries/s", "cores": 1, "kind": "port",
            "sample": f"{n} pair queries (build both + FP64 detect) of the {len(w.pairs)} pairs, {el:.1f} s",
            "fp64_oracle_mismatches": mismatches, "pairs_checked": len(checked)}


def run_reference_precision(args, rank, world):
    """The reference CPU path over the sheets (oracle port; FP32 test, the
    reference's arithmetic) on every host core, 1 pair per thread per step."""
    if rank != 0:
        return None
    Ref, ref_kind = reference_cpu()
    from oibvh_gb300 import workloads as W

    w = W.sheets(64, 256)
    threads = os.cpu_count() or 1
    sample = _sample_pairs(w, min(len(w.pairs), threads))
    ports = []
    for p in sample:
        a, b = w.pairs[p]
        port = Ref()
        port.add_mesh(w.meshes[a].xyz, w.meshes[a].tri)
        port.add_mesh(w.meshes[b].xyz, w.meshes[b].tri)
        ports.append((port, a, b))

    def one_step():
        def work(k):
            port, a, b = ports[k]
            port.set_positions(0, w.meshes[a].xyz)
            port.set_positions(1, w.meshes[b].xyz)
            port.detect()

        tt = [threading.Thread(target=work, args=(k,)) for k in range(len(ports))]
        for t in tt:
            t.start()
        for t in tt:
            t.join()

    for _ in range(args.warmup):
        one_step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        one_step()
    el = time.perf_counter() - t0
    q = args.steps * len(ports)
    value = q / el
    return {"metric": "collision queries/s (mesh pairs through refit + broad + narrow), FP64-filtered triangle test",
            "value": round(value, 3), "unit": "queries/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1e3 * el / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded sine sheets)",
            "config": {"workload": w.name, **w.info, "parallelism": f"{len(ports)} host threads, 1 pair each"},
            "impl": "reference",
            "cpu_baseline": {"value": round(value, 3), "unit": "queries/s", "cores": len(ports), "kind": ref_kind,
                             "sample": f"{q} pair queries (refit both + detect, float test) over {len(ports)} pairs"},
            "e2e": {"value": round(value, 3), "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# --------------------------------------------------------------------------- serving workload
def run_ours_serving(args, rank, world, local):
    """A pool of resident meshes (2,000 noise icospheres, T log-uniform
    500..2M) behind the continuous-batching server; Poisson query streams at
    each offered rate; per-query latency = (submit - scheduled arrival) +
    queue + service (launch to results on the host). The plain path is the
    same queries one at a time (each alone on the GPU)."""
    import ctypes as C

    import torch

    from oibvh_gb300 import OibvhTree, Scene, Server, _native
    from oibvh_gb300 import workloads as W

    torch.cuda.set_device(local)
    dev = local
    t0 = time.perf_counter()
    w = W.serving(args.pool)
    trees = [OibvhTree(m, device=dev) for m in w.meshes]
    sc = Scene(dev)
    for t in trees:
        sc.addOibvhTree(t)
    sc.build()  # one launch per build stage for the whole pool
    torch.cuda.synchronize()
    setup_s = time.perf_counter() - t0
    srv = Server(dev, int(args.budget_gb * (1 << 30)), 4096, 4)
    for t in trees:
        srv.add_mesh(t)
    srv.start()
    L = _native.lib()
    rates = [float(r) for r in args.rates.split(",") if r]
    sampler = ClockSampler(dev) if rank == 0 else None
    if sampler:
        sampler.start()

    def run_stream(rate, n, seed):
        # the load generator is Python: a cyclic-GC pass over the process's
        # objects would stall submission and count as latency, so it stays
        # off while a stream runs
        gc.collect()
        gc.disable()
        try:
            return _run_stream(rate, n, seed)
        finally:
            gc.enable()

    def _run_stream(rate, n, seed):
        ab, mats = w.queries(n, seed=seed)
        rng = np.random.Generator(np.random.PCG64(seed + 7))
        arrivals = np.cumsum(rng.exponential(1.0 / rate, size=n))
        mp = mats.ctypes.data
        tickets = np.empty(n, dtype=np.uint64)
        lag = np.empty(n, dtype=np.float64)
        tk = C.c_uint64()
        submit = L.oibvh_server_submit
        start = time.perf_counter() + 0.002
        for k in range(n):
            target = start + arrivals[k]
            now = time.perf_counter()
            while now < target:
                now = time.perf_counter()
            st = submit(srv._h, int(ab[k, 0]), int(ab[k, 1]), C.cast(C.c_void_p(mp + 48 * k), _native._f32p),
                        C.byref(tk))
            if st:
                raise RuntimeError(L.oibvh_last_error().decode())
            tickets[k] = tk.value
            lag[k] = now - target
        lat = np.empty(n)
        queue = np.empty(n)
        service = np.empty(n)
        sizes = np.empty(n)
        pairs = 0
        r = _native.QueryResult()
        t_last = 0.0
        for k in range(n):
            _native.check(L.oibvh_server_wait(srv._h, int(tickets[k]), 600000, C.byref(r)), "oibvh_server_wait")
            lat[k] = 1e3 * lag[k] + (r.queue_us + r.service_us) / 1e3
            queue[k] = r.queue_us / 1e3
            service[k] = r.service_us / 1e3
            sizes[k] = r.batch_size
            pairs += r.n_pairs
            t_last = max(t_last, arrivals[k] + lag[k] + (r.queue_us + r.service_us) / 1e6)
            L.oibvh_server_release(srv._h, int(tickets[k]))
        return {"offered_per_s": rate, "queries": n, "throughput_per_s": round(n / t_last, 1),
                "latency_ms": {"p50": round(float(np.percentile(lat, 50)), 4),
                               "p99": round(float(np.percentile(lat, 99)), 4),
                               "max": round(float(lat.max()), 4)},
                "submit_lag_ms": {"p99": round(1e3 * float(np.percentile(lag, 99)), 4),
                                  "max": round(1e3 * float(lag.max()), 4)},
                "queue_ms": {"p99": round(float(np.percentile(queue, 99)), 4), "max": round(float(queue.max()), 4)},
                "service_ms": {"p99": round(float(np.percentile(service, 99)), 4),
                               "max": round(float(service.max()), 4)},
                "mean_batch": round(float(sizes.mean()), 2), "pairs": int(pairs)}

    # warm-up stream (lane buffers grow to their working sizes)
    run_stream(30000.0, 6000, seed=99)
    sweep = []
    launches0 = L.oibvh_get_launch_count()
    for i, rate in enumerate(rates):
        n = int(min(max(2000, rate * 0.4), 40000))
        sweep.append(run_stream(rate, n, seed=1000 + i))
    sweep_launches = L.oibvh_get_launch_count() - launches0
    sweep_queries = sum(r["queries"] for r in sweep)
    sweep_pairs = sum(r["pairs"] for r in sweep)
    clocks = sampler.stop() if sampler else None

    # plain: the same kind of queries one at a time, each alone on the GPU
    n_plain = 400
    ab, mats = w.queries(n_plain, seed=4242)
    plain_lat = []
    tp0 = time.perf_counter()
    r = _native.QueryResult()
    tk = C.c_uint64()
    for k in range(n_plain):
        q0 = time.perf_counter()
        _native.check(L.oibvh_server_submit(srv._h, int(ab[k, 0]), int(ab[k, 1]),
                                            C.cast(C.c_void_p(mats.ctypes.data + 48 * k), _native._f32p),
                                            C.byref(tk)), "oibvh_server_submit")
        _native.check(L.oibvh_server_wait(srv._h, tk.value, 600000, C.byref(r)), "oibvh_server_wait")
        L.oibvh_server_release(srv._h, tk.value)
        plain_lat.append(1e3 * (time.perf_counter() - q0))
    plain_qps = n_plain / (time.perf_counter() - tp0)
    st = srv.stats()
    srv.close()
    top = max(sweep, key=lambda x: x["throughput_per_s"])
    line = {
        "metric": "served collision queries/s (Poisson arrivals, continuous batching) with p50/p99 latency",
        "value": top["throughput_per_s"], "unit": "queries/s", "n_gpus": world, "steps": len(rates),
        "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded noise icospheres, seeded query stream)",
        "config": {"workload": w.name, **w.info, "memory_budget_gb": args.budget_gb, "lanes": 4,
                   "max_batch": 4096, "entry_level": 4, "parallelism": f"replicas{world}",
                   "l2": "inputs far larger than L2 (pool of " + str(w.info["triangles_total"]) + " triangles)"},
        "sweep": sweep,
        "plain_one_at_a_time": {"queries_per_s": round(plain_qps, 1),
                                "latency_ms": {"p50": round(float(np.percentile(plain_lat, 50)), 4),
                                               "p99": round(float(np.percentile(plain_lat, 99)), 4)}},
        "served_over_plain": round(top["throughput_per_s"] / plain_qps, 2),
        "server_stats": st,
        "e2e": {"value": top["throughput_per_s"], "unit": "queries/s", "h2d_bytes_per_step": 48,
                "d2h_bytes_per_step": round(8 * sweep_pairs / max(1, sweep_queries) + 4, 1),
                "note": "every served query is end to end: host submit -> host pairs; a step is one query "
                        "(48 B of transform in; its pairs out, 8 B each, and a 4 B offset)"},
        "gpu_launches": int(sweep_launches),
        "gpu_launches_note": f"this library's kernels over the {sweep_queries} queries of the sweep",
        "clocks": clocks,
        "setup_s": round(setup_s, 2),
    }
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_serving(w, args.cpu_seconds)
    return line


def cpu_baseline_serving(w, seconds):
    """The reference CPU path per query on 1 core: B's SimpleBVH refit to the
    transformed positions, then detect against A (both meshes resident)."""
    Ref, ref_kind = reference_cpu()
    from oibvh_gb300 import workloads as W

    ab, mats = w.queries(64, seed=777)
    t0 = time.perf_counter()
    n = 0
    ports = {}
    t_run = 0.0
    for k in range(64):
        a, b = int(ab[k, 0]), int(ab[k, 1])
        if (a, b) not in ports:
            p = Ref()
            p.add_mesh(w.meshes[a].xyz, w.meshes[a].tri)
            p.add_mesh(w.meshes[b].xyz, w.meshes[b].tri)
            ports[(a, b)] = p
        p = ports[(a, b)]
        xb = W.rigid_apply(w.meshes[b].xyz, mats[k])
        q0 = time.perf_counter()
        p.set_positions(1, xb)
        p.detect()
        t_run += time.perf_counter() - q0
        n += 1
        del ports[(a, b)]
        if time.perf_counter() - t0 > seconds:
            break
    return {"value": round(n / t_run, 3), "unit": "queries/s", "cores": 1, "kind": ref_kind,
            "sample": f"{n} queries of the stream (refit B + detect; BVH build and the transform untimed), "
                      f"{t_run:.1f} s"}


def run_reference_serving(args, rank, world):
    """The reference CPU path on every host core: queries of the stream run
    independently, one per thread, refit + detect each."""
    if rank != 0:
        return None
    Ref, ref_kind = reference_cpu()
    from oibvh_gb300 import workloads as W

    w = W.serving(args.pool)
    threads = os.cpu_count() or 1
    ab, mats = w.queries(threads, seed=777)
    ports = []
    for k in range(threads):
        a, b = int(ab[k, 0]), int(ab[k, 1])
        p = Ref()
        p.add_mesh(w.meshes[a].xyz, w.meshes[a].tri)
        p.add_mesh(w.meshes[b].xyz, w.meshes[b].tri)
        ports.append((p, W.rigid_apply(w.meshes[b].xyz, mats[k])))

    def one_step():
        def work(k):
            p, xb = ports[k]
            p.set_positions(1, xb)
            p.detect()

        tt = [threading.Thread(target=work, args=(k,)) for k in range(threads)]
        for t in tt:
            t.start()
        for t in tt:
            t.join()

    for _ in range(args.warmup):
        one_step()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        one_step()
    el = time.perf_counter() - t0
    value = args.steps * threads / el
    return {"metric": "served collision queries/s (Poisson arrivals, continuous batching) with p50/p99 latency",
            "value": round(value, 3), "unit": "queries/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1e3 * el / args.steps, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded noise icospheres, seeded query stream)",
            "config": {"workload": w.name, **w.info, "parallelism": f"{threads} host threads, 1 query each"},
            "impl": "reference",
            "cpu_baseline": {"value": round(value, 3), "unit": "queries/s", "cores": threads, "kind": ref_kind,
                             "sample": f"{args.steps * threads} queries (refit B + detect), {threads} per step"},
            "e2e": {"value": round(value, 3), "unit": "queries/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# --------------------------------------------------------------------------- sub-configs of the default line
def _sub_args(args, **kw):
    sub = argparse.Namespace(**vars(args))
    for k, v in kw.items():
        setattr(sub, k, v)
    return sub


def _free_device_memory():
    import gc

    gc.collect()
    try:
        import torch

        if torch.cuda.is_available():
            torch.cuda.synchronize()
            torch.cuda.empty_cache()
    except Exception:
        pass


SERVED_RATES = "10000,30000,60000,100000,150000"


def subconfigs_ours(args, local):
    """The serving config (2,000-mesh pool, Poisson sweep) and the precision
    config (64 sheet pairs, FP64-filtered test) as compact sub-objects of the
    default line: served queries/s with p50/p99 and served vs plain; frame and
    per-query p50/p99, the FP64 oracle's mismatch count over all 64 pairs
    and the float/FP64 disagreements. Run on this rank's GPU alone."""
    out = {}
    _free_device_memory()
    sv = run_ours_serving(_sub_args(args, rates=SERVED_RATES, pool=2000, budget_gb=16.0,
                                    cpu_seconds=min(args.cpu_seconds, 4.0)), 0, 1, local)
    out["served"] = {
        "workload": sv["config"]["workload"], "pool_triangles": sv["config"]["triangles_total"],
        "memory_budget_gb": sv["config"]["memory_budget_gb"],
        "queries_per_s": sv["value"],
        "sweep": [{"offered_per_s": r["offered_per_s"], "queries": r["queries"],
                   "throughput_per_s": r["throughput_per_s"], "p50_ms": r["latency_ms"]["p50"],
                   "p99_ms": r["latency_ms"]["p99"], "max_ms": r["latency_ms"]["max"],
                   "submit_lag_max_ms": r["submit_lag_ms"]["max"], "queue_p99_ms": r["queue_ms"]["p99"],
                   "service_p99_ms": r["service_ms"]["p99"],
                   "mean_batch": r["mean_batch"]} for r in sv["sweep"]],
        "server_redos": sv["server_stats"]["redos"], "max_batch_seen": sv["server_stats"]["max_batch_seen"],
        "plain_one_at_a_time": sv["plain_one_at_a_time"], "served_over_plain": sv["served_over_plain"],
        "latency_how": ("per query: (submit - scheduled Poisson arrival) + queue + service, host clock; "
                        "the Python load generator runs with its cyclic GC off during a stream"),
        "gpu_launches": sv["gpu_launches"], "clocks": sv["clocks"],
    }
    if "cpu_baseline" in sv:
        out["served"]["cpu_baseline"] = sv["cpu_baseline"]
    _free_device_memory()
    pr = run_ours_precision(_sub_args(args, pairs=64, steps=100, warmup=5,
                                      cpu_seconds=min(args.cpu_seconds, 4.0)), 0, 1, local)
    f = pr["fp64_filter"]
    out["precision"] = {
        "workload": pr["config"]["workload"], "queries_per_s": pr["value"], "frame_ms": pr["ms_per_step"],
        "frames": pr["steps"], "frame_latency_ms": pr["frame_latency_ms"],
        "plain_single_pair": pr["plain_single_pair"], "batched_over_plain": pr["batched_over_plain"],
        "plain_single_pair_fp32": pr["plain_single_pair_fp32"],
        "fp64_oracle_mismatches": pr.get("fp64_oracle", {}).get("fp64_oracle_mismatches"),
        "fp64_oracle": pr.get("fp64_oracle"),
        "fp32_vs_fp64_disagreements": int(sum(f["fp32_vs_fp64_disagreements_per_pair"])),
        "pairs_with_disagreements": f["pairs_with_disagreements"],
        "candidates": f["candidates"], "fp64_candidates": f["fp64_candidates"], "fp64_axes": f["fp64_axes"],
        "fp32_frame": pr["fp32_frame"], "e2e": pr["e2e"], "gpu_launches": pr["gpu_launches"],
        "clocks": pr["clocks"], "tuning": pr["config"]["tuning"],
    }
    if "cpu_baseline" in pr:
        out["precision"]["cpu_baseline"] = pr["cpu_baseline"]
    out["targets"] = {
        "batched_and_served_over_plain_min": 5.0,
        "p99_ms_max": 2.0,
        "p99_ms_precision_frame": pr["frame_latency_ms"]["p99"],
        "p99_ms_precision_per_query": pr["plain_single_pair"]["latency_ms"]["p99"],
        "p99_ms_served": {str(int(r["offered_per_s"])): r["latency_ms"]["p99"] for r in sv["sweep"]},
        "fp64_oracle_mismatches": out["precision"]["fp64_oracle_mismatches"],
        "reading": "config numbering is ambiguous (1-based: batching + precision; 0-based: precision + serving); "
                   "both are reported",
    }
    return out


def subconfigs_reference(args):
    """The reference CPU path on the same sub-configs, on every host core, and
    the reference's own GPU kernels where its construction can run safely."""
    sub = _sub_args(args, steps=3, warmup=1)
    sv = run_reference_serving(sub, 0, 1)
    pr = run_reference_precision(sub, 0, 1)
    pick = ("value", "unit", "cpu_baseline", "config", "ms_per_step")
    return {"served": {k: sv[k] for k in pick}, "precision": {k: pr[k] for k in pick},
            "reference_gpu": reference_gpu_sheets()}


REF_GPU_SAMPLE = 16  # sheet pairs of config 4 timed through the reference's GPU kernels


def reference_gpu_sheets():
    """The reference's own GPU kernels (src/cuda/oibvh.cu, src/cuda/collide.cu,
    compiled unmodified for sm_103a, driven by oracle/ref_gpu_harness.cu's
    restatement of OibvhTree::refit and Scene::detectCollisionOnGPU, entry 4,
    expand 3) per query on a sample of config 4's sheet pairs: refit both
    trees, then detect, as the reference's frame does (positions and faces go
    to the device and the trees back to the host on every refit). The other
    configs' icosphere meshes have triangle counts 20 x 4^s, never powers of
    two, so the construction kernels' schedules have partial blocks (threads
    that return before __syncthreads); the harness refuses them."""
    try:
        import torch

        from oracle.oracle import RefGPU
        from oibvh_gb300 import workloads as W
    except Exception as e:  # noqa: BLE001
        return {"unavailable": f"reference GPU kernels not importable: {e}"}
    if not RefGPU.available() or not torch.cuda.is_available():
        return {"unavailable": "reference GPU kernels not built here (oracle/build_ref.sh) or no GPU"}
    w = W.sheets(64, 256)
    sample = _sample_pairs(w, REF_GPU_SAMPLE)
    wall, kern, cands, hits, refused = [], [], 0, 0, 0
    for p in sample:
        a, b = w.pairs[p]
        ta, tb = RefGPU.Tree(w.meshes[a].xyz, w.meshes[a].tri), RefGPU.Tree(w.meshes[b].xyz, w.meshes[b].tri)
        if ta.build()[0] != RefGPU.OK or tb.build()[0] != RefGPU.OK:
            refused += 1
            continue
        for rep_ in range(4):  # one warm-up query, three timed
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            sa, ma = ta.refit(w.meshes[a].xyz)
            sb, mb = tb.refit(w.meshes[b].xyz)
            n, _, nc, md = RefGPU.detect([ta, tb], 4, 3)
            torch.cuda.synchronize()
            el = 1e3 * (time.perf_counter() - t0)
            if n < 0 or sa or sb:
                refused += 1
                break
            if rep_:
                wall.append(el)
                kern.append(float(ma[1] + mb[1] + md[1] + md[2]))
        cands += nc
        hits += max(n, 0)
    if not wall:
        return {"unavailable": f"every sampled pair was refused by the harness's safety checks ({refused})"}
    return {"what": "the reference's own GPU kernels, compiled unmodified for sm_103a, headless host sequence "
                    "(refit both trees + detect, entry 4, expand 3)",
            "config": f"precision sheets: {len(wall) // 3} of {len(w.pairs)} pairs, 131,072 triangles per sheet",
            "ms_per_query": {"p50": round(_pctl(wall, 50), 3), "p99": round(_pctl(wall, 99), 3)},
            "queries_per_s": round(1e3 / statistics.median(wall), 2),
            "kernels_ms_per_query": round(statistics.median(kern), 3),
            "candidates_per_query": cands // max(1, len(wall) // 3), "hits_per_query": hits // max(1, len(wall) // 3),
            "refused_pairs": refused,
            "not_run": "configs 1, 2, 3 and 5: icosphere triangle counts are never powers of two, so the reference's "
                       "construction kernels would run partial blocks whose threads return before __syncthreads "
                       "(src/cuda/oibvh.cu:87-88, :122); the harness refuses them before launching"}


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        line = {"batched": run_reference_batched, "precision": run_reference_precision,
                "serving": run_reference_serving}.get(
            args.workload, run_reference)(args, rank, world)
    else:
        line = {"batched": run_ours_batched, "precision": run_ours_precision,
                "serving": run_ours_serving}.get(
            args.workload, run_ours)(args, rank, world, local)
    if line is not None and args.workload == "batched" and not args.no_subconfigs:
        line.update(subconfigs_reference(args) if args.impl == "reference" else subconfigs_ours(args, local))
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
