#!/usr/bin/env python
"""Benchmark of the GPU-driven fill pipeline on one GB300 (or N replicas).

Workloads (``--config``, the configurations the benchmark is quoted on; seeded synthetic scenes):

  1  one scene of 240 closed cubic paths (8-24 segments each), 1024 x 1024, seed 0
  2  20,000 paths (60% cubic / 40% quadratic, 4-64 segments, log-uniform boxes 8-2048 px,
     alternating fill rules, 30% translucent), 4096 x 4096, seed 0
  3  150,000 glyph-like quadratic outlines (1-3 contours, holes reversed, 12-48 px on a
     jittered grid), black on white, 2048 x 2048, seed 0
  4  (default) 512 independent scenes of the config-1 generator, paths per scene log-uniform
     16-4096, canvas side in {256, 512, 1024, 2048}, seeds 1000+i, rendered in one frame
  5  the held-out mixed scene of the learned sizer: 8,192 paths of the three families at
     4096 x 4096, seed 7 (learned frame against the exact one)

One step = one frame over the configuration's scenes.  The JSON line (rank 0) holds:
  value        scenes/s of the frame the library runs by default (pf_render_auto: the learned
               one-pass frame where it measured faster, else the exact one), inputs resident;
  exact/learned the two frames timed on their own;
  plain        (config 4) scenes/s of the single-scene pipeline, one frame per scene;
  e2e          the same metric through the C-ABI from pinned host buffers: upload, frame and
               every image delivered to pinned host memory inside the timed region (the fastest
               of three timed blocks of --steps steps);
  roofline     the dominant stages (flatten + bin) against the measured HBM peak, with the
               algorithmic bytes of the hot-path scope table (8 B per point and per segment
               read, 12 B per fill and 4 B per visible tile written); roofline_composite the
               fused coverage + composite kernel (12 B per composited fill, 16 B per composite
               entry, 4 B per framebuffer tile, 4 B per pixel written);
  cpu_baseline the oracle port (restated d3d9 tiler + FP64 coverage and src-over composite) on
               the host cores: 1 thread, 4 threads and all cores;
  parity       the frame's tiles and pixels against the oracle on a stratified sample of scenes.

``--impl reference`` times that CPU implementation alone (the reference arm).
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import gc
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "pathfinder-cpp_gb300")
sys.path.insert(0, PKG)

METRIC = "frame ms & scenes/s: batched+learned vs plain CUDA pipeline, 1 GB300, exact tiles"
UNIT = "scenes/s"
# DRAM bytes of the hot kernels per algorithmic byte, from an ncu capture of each workload
# (written next to the capture's summary; absent: traffic is reported as null)
TRAFFIC_FILE = os.path.join(ROOT, "profiles", "dram_traffic.json")
# pf_render_auto calls that always suffice for it to decide (two timed frames of each kind)
AUTO_SETTLE = 7
# end-to-end blocks timed (the fastest is reported)
E2E_BLOCKS = 3
L2_FLUSH_BYTES = 256 << 20  # written between timed steps of the single-scene configurations

CONFIG_DESC = {
    1: "config 1: one scene of 240 closed cubic paths (8-24 segments, control points uniform), nonzero, "
       "opaque colours, 1024x1024, seed 0",
    2: "config 2: one scene of 20,000 paths, 60% cubic / 40% quadratic, 4-64 segments, log-uniform boxes "
       "8-2048 px, alternating fill rules, 30% translucent, 4096x4096, seed 0",
    3: "config 3: one scene of 150,000 glyph-like quadratic outlines (10-40 segments, 1-3 contours, holes "
       "reversed), 12-48 px on a jittered grid, black on white, 2048x2048, seed 0",
    4: "batched: %d scenes, paths/scene log-uniform 16-4096 (cubic 8-24 seg, control points uniform over "
       "the canvas), canvas side in {256,512,1024,2048}, seeds 1000+i",
    5: "config 5: held-out mixed scene, 8,192 paths of the three families at 4096x4096, seed 7",
}


class no_gc:
    """Python's garbage collector off for a timed region (as timeit does)."""

    def __enter__(self):
        self.was = gc.isenabled()
        gc.disable()

    def __exit__(self, *exc):
        if self.was:
            gc.enable()


def replica_first_seed(rank: int) -> int:
    """First scene seed of a rank's batch: replicas render disjoint batches (no collective)."""
    return 1000 + 100000 * rank


def max_over_ranks(ms: float, dist, device: str) -> float:
    """The slowest rank's time (the whole job's step time); dist None for one process."""
    if dist is None:
        return ms
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", type=int, choices=[1, 2, 3, 4, 5], default=4)
    ap.add_argument("--scenes", type=int, default=512, help="scenes of the batched configuration")
    ap.add_argument("--cpu-sample", type=int, default=64,
                    help="batched configuration: scenes of the stratified CPU-baseline sample (all cores; "
                         "a quarter of it at 1 and 4 threads)")
    ap.add_argument("--ref-sample", type=int, default=16,
                    help="batched configuration: scenes per step of the reference arm")
    ap.add_argument("--parity-sample", type=int, default=8,
                    help="scenes of the stratified sample checked against the oracle (0: none)")
    ap.add_argument("--strokes", action="store_true",
                    help="the batched scenes as stroked paths (scenes.batched_stroked: 30%% dashed); the upload "
                         "strokes them on the GPU, and the line reports that stage too")
    ap.add_argument("--gradients", action="store_true",
                    help="the batched scenes with half of the paths painted with gradients "
                         "(scenes.batched_gradients: linear and radial, clamped and repeated)")
    ap.add_argument("--clips", type=int, default=0,
                    help="clip paths per scene (0: none): the batched scenes with that many clip shapes "
                         "each, 60%% of the draw paths clipped")
    ap.add_argument("--svg", action="store_true",
                    help="SVG documents: the batch is N seeded documents (svg_docs.random_document, shapes per "
                         "document log-uniform 16-1024) parsed on the host by pf_svg_parse; the line adds an "
                         "svg_stage whose end-to-end step parses the documents' text too")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--tuning", default=None,
                    help="launch parameters to set over the built-in or tuned ones, as JSON (pf_tuning fields, "
                         "e.g. '{\"bin_concurrent\": 1}')")
    ap.add_argument("--counters", action="store_true",
                    help="frame counters on in every frame (composite entries and fills, alpha and visible "
                         "tiles), for --profile-frames captures that need them")
    ap.add_argument("--profile-frames", action="store_true",
                    help="only the exact, learned and default frames (warm-up + steps each), a short summary "
                         "line instead of the benchmark line: the command the committed launch lists profile")
    args = ap.parse_args(argv)
    if args.config != 4 and (args.strokes or args.gradients or args.clips or args.svg):
        ap.error("--strokes/--gradients/--clips/--svg vary the batched configuration (--config 4)")
    return args


def variant(args) -> str:
    """Key of the workload in the traffic file: config<N>, with the batched variant appended."""
    for name in ("strokes", "gradients", "svg"):
        if getattr(args, name):
            return f"config{args.config}_{name}"
    return f"config{args.config}_clips" if args.clips else f"config{args.config}"


def svg_texts(n, first_seed):
    """n seeded SVG documents with 16-1024 shapes each (log-uniform)."""
    import numpy as np
    import svg_docs
    rng = np.random.default_rng(first_seed)
    sizes = np.exp(rng.uniform(np.log(16), np.log(1024), n)).astype(int)
    return [svg_docs.random_document(first_seed + i, n_shapes=int(sizes[i])) for i in range(n)]


def make_scenes(args, first_seed):
    import scenes as S
    rank_seed = first_seed - 1000  # 0 on rank 0: the configurations' own seeds
    if args.config == 1:
        return [S.plain_small(seed=rank_seed)]
    if args.config == 2:
        return [S.large_single(seed=rank_seed)]
    if args.config == 3:
        return [S.glyphs(seed=rank_seed)]
    if args.config == 5:
        return [S.mixed(seed=7 + rank_seed, n_paths=8192, side=4096)]
    if args.svg:
        import pfcuda
        return [pfcuda.parse_svg(t) for t in svg_texts(args.scenes, first_seed)]
    if args.strokes:
        return S.batched_stroked(n_scenes=args.scenes, first_seed=first_seed)
    if args.gradients:
        return S.batched_gradients(n_scenes=args.scenes, first_seed=first_seed)
    if args.clips > 0:
        return S.batched_clipped(n_scenes=args.scenes, first_seed=first_seed, n_clips=args.clips)
    return S.batched(n_scenes=args.scenes, first_seed=first_seed)


def workload_config(args, scenes_list):
    import numpy as np
    n_scenes = len(scenes_list)
    desc = CONFIG_DESC[args.config] % n_scenes if args.config == 4 else CONFIG_DESC[args.config]
    if args.strokes:
        desc = ("batched stroked: %d scenes, paths/scene log-uniform 16-4096, canvas side in "
                "{256,512,1024,2048}, seeds 1000+i; every path stroked (1-3 contours of 1-12 line/quad/cubic "
                "segments in a log-uniform box, 40%% closed, width 0.5-24 px, caps/joins uniform), 30%% "
                "dashed" % n_scenes)
    if args.svg:
        desc = ("svg: %d seeded SVG documents (svg_docs.random_document, seeds 1000+i, 16-1024 shapes each: "
                "rect/circle/ellipse/line/poly/path with all path commands, nested transforms, fills, strokes "
                "with caps/joins/dashes, linear and radial gradients), parsed by pf_svg_parse" % n_scenes)
    if args.gradients:
        desc += "; half of the paths painted with gradients (linear and radial, 2-5 stops, 30%% repeating)"
    if args.clips:
        desc += "; %d clip paths per scene (cubic 3-8 seg, a quarter to a whole canvas wide), 60%% of the " \
                "draw paths clipped" % args.clips
    return {
        "workload": desc,
        "scenes": n_scenes,
        "paths": int(sum(s.n_paths for s in scenes_list)),
        "points": int(sum(s.n_points for s in scenes_list)),
        "pixels": int(sum(int(np.ceil(s.width)) * int(np.ceil(s.height)) for s in scenes_list)),
        "tile": 16,
        "l2": ("inputs and working set larger than L2 (129 MB) every step" if args.config == 4 else
               "L2 flushed between timed steps (a 256 MB write); each step timed on its own"),
    }


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def wait_first(self, timeout: float = 10.0):
        """Block until nvidia-smi has printed its first sample (its start-up stays out of the
        timed regions)."""
        t0 = time.time()
        while self.proc and not self.lines and time.time() - t0 < timeout:
            time.sleep(0.05)

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def pack_pinned(scenes_list):
    """All scenes' arrays packed contiguously (per array) in pinned host memory."""
    import numpy as np
    import torch
    import pfcuda
    import scenes as S
    keys = [("points", np.float32), ("flags", np.uint8), ("contour_start", np.uint32),
            ("path_start", np.uint32), ("fill_rule", np.uint8), ("color", np.uint32)]
    has = lambda k: any(getattr(s, k, None) is not None for s in scenes_list)  # noqa: E731
    if has("path_clip"):
        keys += [("path_clip", np.uint32), ("path_is_clip", np.uint8)]
    if has("path_stroke"):
        keys += [("path_stroke", S.STROKE_DTYPE), ("contour_closed", np.uint8), ("dashes", np.float32)]
    if has("path_paint"):
        keys += [("path_paint", S.PAINT_DTYPE), ("stops", S.STOP_DTYPE)]

    def field(s, k):
        a = getattr(s, k)
        if a is None:  # a scene without clips or strokes in a batch with some
            defaults = {"path_clip": np.full(s.n_paths, 0xFFFFFFFF, np.uint32),
                        "path_stroke": np.zeros(s.n_paths, S.STROKE_DTYPE),
                        "contour_closed": np.zeros(s.n_contours, np.uint8), "dashes": np.zeros(0, np.float32),
                        "path_paint": np.zeros(s.n_paths, S.PAINT_DTYPE), "stops": np.zeros(0, S.STOP_DTYPE)}
            a = defaults.get(k, np.zeros(s.n_paths, np.uint8))
        return a

    bufs = {}
    for k, dt in keys:
        total = sum(field(s, k).nbytes for s in scenes_list)
        bufs[k] = torch.empty(max(total, 16), dtype=torch.uint8, pin_memory=True)
    offs = {k: 0 for k, _ in keys}
    views = []
    for s in scenes_list:
        ptrs = {}
        for k, dt in keys:
            a = np.ascontiguousarray(field(s, k), dt)
            dst = bufs[k].numpy()[offs[k]:offs[k] + a.nbytes]
            dst[:] = a.view(np.uint8).reshape(-1)
            ptrs[k] = bufs[k].data_ptr() + offs[k]
            offs[k] += a.nbytes
        v = pfcuda.SceneView(*(ptrs[k] for k, _ in keys[:6]), s.n_points, s.n_contours, s.n_paths,
                             s.width, s.height, s.clear)
        if "path_clip" in ptrs:
            v.path_clip, v.path_is_clip = ptrs["path_clip"], ptrs["path_is_clip"]
        if "path_stroke" in ptrs:
            v.path_stroke, v.contour_closed, v.dashes = ptrs["path_stroke"], ptrs["contour_closed"], ptrs["dashes"]
            v.n_dashes = len(field(s, "dashes"))
        if "path_paint" in ptrs:
            v.path_paint, v.stops, v.n_stops = ptrs["path_paint"], ptrs["stops"], len(field(s, "stops"))
        views.append(v)
    h2d = sum(offs.values())
    return bufs, views, h2d


# ---------------------------------------------------------------------------------------------
# CPU side: the oracle port (test infrastructure; here only the timed CPU baseline and the
# checker of the parity sample)

def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    if not os.path.exists(oracle.LIB_ORACLE):
        oracle.build()
    return oracle


def stratified(scenes_list, n):
    """n scenes spread evenly over the batch ordered by a work estimate (paths x canvas side),
    so the sample holds the small and the large scenes in proportion."""
    if n >= len(scenes_list):
        return list(range(len(scenes_list)))
    order = sorted(range(len(scenes_list)), key=lambda i: (scenes_list[i].n_paths * scenes_list[i].width, i))
    step = len(order) / n
    return sorted(order[int(step * k + step / 2)] for k in range(n))


def cpu_time(scenes_list, idx, threads: int) -> float:
    """Seconds for the oracle port to tile and composite scenes idx.  One scene: threads inside the
    scene (paths, then framebuffer tiles); several: a pool of `threads` over the scenes."""
    oracle = _oracle()
    t0 = time.perf_counter()
    if len(idx) == 1:
        oracle.render(scenes_list[idx[0]], threads=threads)
    elif threads == 1:
        for i in idx:
            oracle.render(scenes_list[i], threads=1)
    else:
        with cf.ThreadPoolExecutor(threads) as ex:
            list(ex.map(lambda i: oracle.render(scenes_list[i], threads=1), idx))
    return time.perf_counter() - t0


CPU_RUNS = 5  # timed runs of the CPU sample after one warm-up; their median is reported


def cpu_baseline(args, scenes_list):
    """scenes/s of the oracle port at 1 thread, 4 threads and all host threads: the median of
    CPU_RUNS timed runs after one warm-up run.  The batched configuration times stratified
    samples (all threads: --cpu-sample scenes; 1 and 4 threads: a quarter of that); a single scene
    runs whole, a run repeating it to at least 0.2 s when one pass is shorter."""
    n = len(scenes_list)
    cores = os.cpu_count() or 1
    out = {}
    for label, threads in (("1", 1), ("4", min(4, cores)), ("all", cores)):
        k = args.cpu_sample if label == "all" else max(4, args.cpu_sample // 4)
        idx = stratified(scenes_list, k) if n > 1 else [0]
        warm = cpu_time(scenes_list, idx, threads)
        reps = 1 if warm >= 0.2 else min(50, int(math.ceil(0.2 / max(warm, 1e-6))))
        runs = sorted(sum(cpu_time(scenes_list, idx, threads) for _ in range(reps)) / reps for _ in range(CPU_RUNS))
        dt = runs[len(runs) // 2]
        out[label] = {"value": len(idx) / dt, "threads": threads, "scenes": len(idx), "seconds": dt, "repeats": reps,
                      "runs_seconds": runs}
    v = out["all"]
    sample = (f"{v['scenes']} of {n} scenes (stratified by paths x canvas side), a pool of {cores} threads over "
              f"the scenes" if n > 1 else f"the whole scene, {cores} threads over paths and framebuffer tiles")
    paths_per_scene = sum(s.n_paths for s in scenes_list) / n
    return {"value": v["value"], "unit": UNIT, "cores": cores, "kind": "port",
            "sample": sample + "; restated d3d9 tiler + FP64 coverage and src-over composite",
            "by_threads": {k: {"value": o["value"], "paths_per_s": o["value"] * paths_per_scene,
                               "threads": o["threads"], "scenes": o["scenes"], "seconds": o["seconds"],
                               "repeats": o["repeats"], "runs_seconds": o["runs_seconds"]}
                           for k, o in out.items()},
            "method": f"median of {CPU_RUNS} timed runs after one warm-up run, per thread count",
            "paths_per_s": v["value"] * paths_per_scene}


def run_reference(args, scenes_list):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    n = len(scenes_list)
    idx = stratified(scenes_list, args.ref_sample) if n > 1 else [0]
    for _ in range(max(args.warmup, 0)):
        cpu_time(scenes_list, idx, cores)
    times = [cpu_time(scenes_list, idx, cores) for _ in range(args.steps)]
    per_step = sum(times) / len(times)
    value = len(idx) / per_step
    sample = (f"{len(idx)} of {n} scenes per step (stratified by paths x canvas side), a pool of {cores} threads"
              if n > 1 else f"the whole scene per step, {cores} threads") + \
        "; restated d3d9 tiler + FP64 coverage and src-over composite"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "runs_on": f"host CPU only, {cores} threads; no GPU is used (n_gpus is the launch's N)",
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_step * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 tiling, f64 coverage",
        "data": "synthetic", "config": workload_config(args, scenes_list),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


CANON_KEYS = ["path_rect", "path_tile_first", "path_column_first", "tile_alpha", "tile_backdrop", "tile_fill_count",
              "fills", "column_backdrop", "fb_tiles", "z", "fb_list_first", "fb_list", "tile_mask", "tile_clip",
              "tile_dest_backdrop"]


def parity_sample(args, r, scenes_list):
    """The last frame's tiles and pixels against the oracle on a stratified sample of scenes."""
    import numpy as np
    if args.parity_sample <= 0:
        return None
    oracle = _oracle()
    idx = stratified(scenes_list, args.parity_sample) if len(scenes_list) > 1 else [0]
    cores = os.cpu_count() or 1

    def want(i):
        tiled = {}
        img, _ = oracle.render(scenes_list[i], threads=1 if len(idx) > 1 else cores, tiled=tiled)
        return tiled, img

    bad, mx, tot, cnt, fills = [], 0, 0, 0, 0
    with cf.ThreadPoolExecutor(min(cores, len(idx))) as ex:
        futs = {i: ex.submit(want, i) for i in idx}
        for i in idx:
            got, img = r.canon(i), r.image(i)
            w, wimg = futs.pop(i).result()
            bad += [f"{i}:{k}" for k in CANON_KEYS if got[k].shape != w[k].shape or not np.array_equal(got[k], w[k])]
            d = np.abs(img.astype(np.int16) - wimg.astype(np.int16))
            mx = max(mx, int(d.max()))
            tot += int(d.sum(dtype=np.int64))
            cnt += d.size
            fills += len(got["fills"])
    return {"scenes_checked": len(idx), "fills_checked": fills, "tiles_bit_exact": not bad, "differing": bad[:8],
            "rgba8_max_err": mx, "rgba8_mean_err": tot / max(cnt, 1),
            "full_size": "every scene of configs 2-5 is checked by tests/test_gpu_full_size.py"}


def load_traffic():
    try:
        with open(TRAFFIC_FILE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def main():
    args = parse_args()
    import numpy as np

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        run_reference(args, make_scenes(args, 1000))
        return

    import torch
    import pfcuda
    import build as pf_build
    if not os.path.exists(pfcuda.LIB_PATH):
        pf_build.build()

    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local_rank)

    def barrier():
        if dist is not None:
            dist.barrier()

    # replicas: every rank renders its own scenes (seeds offset by rank); no data-path collective
    scenes_list = make_scenes(args, replica_first_seed(rank))
    n_scenes = len(scenes_list)
    n_paths = sum(s.n_paths for s in scenes_list)
    bufs, views, h2d_bytes = pack_pinned(scenes_list)
    stream = torch.cuda.Stream()
    r = pfcuda.Renderer(device=local_rank, stream=stream.cuda_stream, stage_timing=True, counters=args.counters)
    r.upload_views(views)
    img_bytes = r.image_bytes()
    img_host = torch.empty(img_bytes, dtype=torch.uint8, pin_memory=True)
    single = args.config != 4
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.int32, device="cuda") if single else None

    def timed(fn, steps):
        """Mean ms per step on the device.  Batched: the steps back to back between two events
        (the working set is far larger than L2).  Single scenes: each step between its own
        events, with an L2 flush before each step outside them.  Python's garbage collector is
        off inside (a collection would land in a step's host time)."""
        barrier()
        torch.cuda.synchronize()
        out = []
        with no_gc():
            ms = timed_steps(fn, steps, out)
        barrier()
        return max_over_ranks(ms, dist, "cuda"), out

    def timed_steps(fn, steps, out):
        if flush is None:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            out.extend(fn() for _ in range(steps))
            e1.record(stream)
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) / steps
        ms = 0.0
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            out.append(fn())
            e1.record(stream)
            torch.cuda.synchronize()
            ms += e0.elapsed_time(e1)
        return ms / steps

    learned = os.path.exists(pfcuda.DEFAULT_WEIGHTS)
    if learned:
        r.sizer_load(pfcuda.DEFAULT_WEIGHTS)
    # the launch parameters the autotuner (tune.py) found for the batched configuration on this
    # GPU; the built-in ones are timed beside them (an A/B in this run)
    tuning = None
    if args.config == 4 and os.path.exists(pfcuda.DEFAULT_RENDER_CONFIG):
        builtin = r.tuning()
        frame0 = r.render_auto if learned else r.render
        for _ in range(max(args.warmup, AUTO_SETTLE)):
            frame0()
        ms_builtin, _ = timed(frame0, args.steps)
        cfg = r.load_render_config()
        tuning = {"source": "weights/render_config.json (tune.py: pf_autotune on this configuration)",
                  "params": r.tuning(), "builtin_params": builtin, "frame_ms_builtin": ms_builtin,
                  "tuned_on": cfg.get("gpu"), "tune_frame_ms": cfg.get("frame_ms"),
                  "tune_start_frame_ms": cfg.get("start_frame_ms")}
    if args.tuning:
        r.set_tuning({**r.tuning(), **json.loads(args.tuning)})
        tuning = dict(tuning or {}, params=r.tuning(), override=json.loads(args.tuning))

    # 1. the exact two-pass frame, inputs resident
    for _ in range(args.warmup):
        r.render()
    ms_exact, stats_e = timed(lambda: r.render(), args.steps)

    clocks = ClockSampler(local_rank)
    clocks.start()
    clocks.wait_first()
    # 2. the learned one-pass frame, inputs resident
    ms_learned, stats_l = None, None
    if learned:
        for _ in range(args.warmup):
            r.render_learned()
        ms_learned, stats_l = timed(lambda: r.render_learned(), args.steps)
    # 3. the library's default frame (pf_render_auto), the headline: its first calls over a
    #    workload time the exact and the learned frame (at most seven decide), so it takes at
    #    least that many warm-up frames
    frame = r.render_auto if learned else r.render
    for _ in range(max(args.warmup, AUTO_SETTLE)):
        frame()
    ms_frame, stats_f = timed(frame, args.steps)
    st = stats_f[-1]
    sizer = None
    if learned:
        over, pool = r.sizer_last_frame()
        sizer = {"frames_redone_exactly": int(sum(s["overflow"] for s in stats_l)), "paths_over_budget": over,
                 "spill_pool_slots_used": pool, "learned_host_syncs": stats_l[-1]["host_syncs"],
                 "exact_host_syncs": stats_e[-1]["host_syncs"], "learned_launches": stats_l[-1]["kernel_launches"],
                 "exact_launches": stats_e[-1]["kernel_launches"], "auto": r.last_auto_choice()}

    if args.profile_frames:
        clocks.stop()
        if rank == 0:
            print(json.dumps({"profile_frames": True, "exact_ms": ms_exact, "learned_ms": ms_learned,
                              "frame_ms": ms_frame, "exact_stats": stats_e[-1], "frame_stats": st,
                              "sizer": sizer, "tuning": tuning}), flush=True)
        r.close()
        return

    # 4. parity of this frame against the oracle on a stratified sample (untimed)
    parity = parity_sample(args, r, scenes_list) if rank == 0 else None

    # 5. (batched) the plain single-scene pipeline: one exact frame per scene, inputs resident
    plain = None
    if not single:
        def plain_pass():
            launches = 0
            for i in range(n_scenes):
                launches += r.render(i, 1)["kernel_launches"]
            return launches
        plain_pass()
        ms_plain, launches_plain = timed(plain_pass, max(1, min(args.steps, 3)))
        plain = {"value": world * n_scenes / (ms_plain * 1e-3), "unit": UNIT, "ms_per_step": ms_plain,
                 "gpu_launches_per_step": launches_plain[-1]}

    # 6. end to end through the C-ABI: pinned H2D upload, frame, every image delivered to pinned
    #    host memory.  pf_read_images_async snapshots the images on the device and copies them to
    #    the host on the library's copy stream, so step i's images cross the link while step i+1
    #    uploads and renders; the timed region ends after the last step's images have arrived.
    #    The default frame keeps its choice across uploads of scenes of the same size.
    def e2e_block(steps):
        for _ in range(steps):
            r.upload_views(views)
            frame()
            r.read_images_async(img_host.data_ptr(), img_bytes)
        r.images_wait()

    def timed_block(block, steps):
        barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with no_gc():
            e0.record(stream)
            block(steps)
            e1.record(stream)
            torch.cuda.synchronize()
        barrier()
        return max_over_ranks(e0.elapsed_time(e1) / steps, dist, "cuda")
    # E2E_BLOCKS blocks of `steps` steps each, the fastest reported (every block is timed whole,
    # its last images included): the host link is shared with the machine's other GPUs, and the
    # same build measured 39.5 to 63 ms a step over runs
    e2e_block(max(2, args.warmup // 2))
    e2e_blocks = [timed_block(e2e_block, args.steps) for _ in range(E2E_BLOCKS)]
    ms_e2e = min(e2e_blocks)

    # the same with the composite writing the images straight into the host buffer over
    # NVLink-C2C (pf_set_host_image): the pixels cross while the composite runs
    r.set_host_image(img_host.data_ptr(), img_bytes)

    def e2e_host_block(steps):
        for _ in range(steps):
            r.upload_views(views)
            frame()
            r.read_images(img_host.data_ptr(), img_bytes)
    e2e_host_block(max(1, args.warmup // 2))
    e2e_host_blocks = [timed_block(e2e_host_block, args.steps) for _ in range(E2E_BLOCKS)]
    ms_e2e_host = min(e2e_host_blocks)
    r.set_host_image(None)
    clk = clocks.stop()

    # SVG documents end to end (--svg): every step parses the documents' text on the host
    # (pf_svg_parse on a thread pool; ctypes releases the interpreter lock), uploads straight
    # from the parser's arrays, renders and delivers the images to pinned host memory
    svg_stage = None
    if args.svg:
        texts = [t.encode() for t in svg_texts(args.scenes, replica_first_seed(rank))]
        n_threads = min(16, os.cpu_count() or 1)
        pool = cf.ThreadPoolExecutor(n_threads)
        parse_ms = []

        def svg_block(steps):
            for _ in range(steps):
                t0 = time.perf_counter()
                docs = list(pool.map(pfcuda.SvgDocument, texts))
                parse_ms.append((time.perf_counter() - t0) * 1e3)
                r.upload_views([d.view for d in docs])
                frame()
                r.read_images_async(img_host.data_ptr(), img_bytes)
                for d in docs:
                    d.close()
            r.images_wait()
        svg_block(max(1, args.warmup // 2))
        parse_ms.clear()
        ms_svg = timed_block(svg_block, args.steps)
        t0 = time.perf_counter()
        for t in texts[:64]:
            pfcuda.SvgDocument(t).close()
        one_thread_ms = (time.perf_counter() - t0) * 1e3 * len(texts) / 64
        mb = sum(len(t) for t in texts) / 1e6
        svg_stage = {
            "e2e": {"value": world * n_scenes / (ms_svg * 1e-3), "unit": UNIT, "ms_per_step": ms_svg,
                    "h2d_bytes_per_step": h2d_bytes, "d2h_bytes_per_step": img_bytes,
                    "includes": "host parse of the text + pageable H2D upload + frame + images to host"},
            "parse_ms": sum(parse_ms) / len(parse_ms), "parse_threads": n_threads,
            "parse_ms_one_thread_est": one_thread_ms, "text_mb": mb,
            "parse_mb_per_s": mb / (sum(parse_ms) / len(parse_ms) * 1e-3),
        }
        r.upload_views(views)

    # one more (untimed) frame with the frame counters on: composite entries and fills, alpha
    # and visible tiles, for the rooflines' bytes
    r.set_flags(stage_timing=True, counters=True)
    st_c = frame()
    r.set_flags(stage_timing=True, counters=False)
    st = dict(st)
    for k in ("composite_entries", "composited_fills", "alpha_tiles", "visible_tiles"):
        st[k] = st_c[k]
    st["walk_chunks"] = int(r.debug_counters()[15])  # 32-candidate chunks the composite's z-walks read

    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback 6.8 TB/s"
    if os.path.exists(peaks_path):
        with open(peaks_path) as f:
            peak = float(json.load(f)["hbm_gbs"])
        peak_src = "measured (MEASURED_PEAKS.json hbm_gbs)"
    traffic = load_traffic().get(variant(args), {})

    # the stroke pass of the upload (--strokes): uploads from pinned host memory, timed on the
    # host clock (H2D copies, dashing, stroking and the pass's three synchronisations), and
    # the dash / stroke kernels' device time from the library's events
    stroke_stage = None
    if args.strokes:
        ups, ust = [], []
        for _ in range(args.warmup):
            r.upload_views(views)
        for _ in range(args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r.upload_views(views)
            ups.append((time.perf_counter() - t0) * 1e3)
            ust.append(r.upload_stats())
        us = ust[-1]
        ms_dash = sum(x["ms_dash"] for x in ust) / len(ust)
        ms_stroke = sum(x["ms_stroke"] for x in ust) / len(ust)
        stroked_in = 0
        for sc in scenes_list:
            w = sc.path_stroke["line_width"] > 0
            plain_st = w & (sc.path_stroke["dash_count"] == 0)
            pts_per_path = np.diff(sc.contour_start.astype(np.int64)[sc.path_start.astype(np.int64)])
            stroked_in += int(pts_per_path[plain_st].sum())
        stroked_in += us["dash_points"]
        # each pass (count, write) reads every stroked input point twice (forward and backward
        # offsets; 8 B + 1 B flag) and the write pass stores every outline point (9 B)
        s_bytes = 2 * 2 * 9 * stroked_in + 9 * us["n_points"]
        s_ach = s_bytes / (ms_stroke * 1e-3) / 1e9 if ms_stroke > 0 else None
        stroke_stage = {
            "upload_ms": sum(ups) / len(ups), "ms_dash": ms_dash, "ms_stroke": ms_stroke,
            "stroked_paths": us["stroked_paths"], "dashed_paths": us["dashed_paths"],
            "dash_points": us["dash_points"], "stroke_input_points": stroked_in,
            "outline_points": us["n_points"], "outline_contours": us["n_contours"],
            "roofline": {"kernel": "k_stroke (count + write passes)", "bound": "hbm", "achieved": s_ach,
                         "peak": peak, "unit": "GB/s", "frac": s_ach / peak if s_ach else None, "traffic": None,
                         "algorithmic_bytes": s_bytes,
                         "note": "compute bound: exact-IEEE offset curves (divisions, square roots, "
                                 "tolerance samples) per leaf; bytes are the points read and written"},
        }
        if rank == 0 and not args.no_cpu_baseline:
            oracle = _oracle()
            sample = stratified(scenes_list, 16)
            t0 = time.perf_counter()
            for i in sample:
                oracle.stroke_scene(scenes_list[i])
            dt = time.perf_counter() - t0
            stroke_stage["cpu_baseline"] = {
                "value": len(sample) / dt, "unit": "scenes/s (stroke pass only)", "cores": 1, "kind": "port",
                "sample": f"16 stratified scenes ({dt:.2f} s): restated OutlineDash + OutlineStrokeToFill, one thread"}
            stroke_stage["gpu_scenes_per_s"] = n_scenes / ((ms_dash + ms_stroke) * 1e-3)

    # roofline of the dominant stages, flatten + bin, with the hot-path scope table's bytes:
    # points and segments read (8 B each), fills written (12 B, the reference's Fill record) and
    # a 4-byte word per visible tile, over the two stages' CUDA-event time on the frame's stream
    fb_ms = sum(x["ms_flatten"] + x["ms_bin"] for x in stats_f) / len(stats_f)
    bin_ms = sum(x["ms_bin"] for x in stats_f) / len(stats_f)
    fb_bytes = 8 * st["points"] + 8 * st["segments"] + 12 * st["fills"] + 4 * st["visible_tiles"]
    fb_ach = fb_bytes / (fb_ms * 1e-3) / 1e9 if fb_ms > 0 else None
    # the bytes this implementation's layout moves in the same two stages: 16 B per leaf line
    # written by the flatten and read by binning, 8 B per fill, 6 B per tile (state and end
    # offset), 36 B per path
    own_bytes = 32 * st["microlines"] + 8 * st["fills"] + 6 * st["tiles"] + 36 * st["paths"]
    # ncu DRAM bytes per algorithmic byte of these stages' kernels in the capture, applied here
    fb_ratio = traffic.get("flatten_bin_dram_per_algorithmic_byte")
    fb_traffic = fb_ratio * fb_bytes / 1e9 if fb_ratio else None

    # roofline of the fused coverage + composite kernel (the units it processes: the composited
    # fills and entries after the z-cull, every framebuffer tile and pixel)
    pixels = sum(int(np.ceil(s.width)) * int(np.ceil(s.height)) for s in scenes_list)
    comp_bytes = (12 * st["composited_fills"] + 16 * st["composite_entries"]
                  + 4 * st["framebuffer_tiles"] + 4 * pixels)
    comp_ms = sum(x["ms_composite"] for x in stats_f) / len(stats_f)
    comp_ach = comp_bytes / (comp_ms * 1e-3) / 1e9 if comp_ms > 0 else None
    comp_ratio = traffic.get("composite_dram_per_algorithmic_byte")

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args, scenes_list)

    if rank == 0:
        value = world * n_scenes / (ms_frame * 1e-3)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_frame, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (exact-IEEE tiling), int32 fixed-point coverage", "data": "synthetic",
            "config": workload_config(args, scenes_list),
            "frame": ("pf_render_auto (the learned one-pass frame where it measured faster than the exact "
                      "two-pass frame, else the exact one)" if learned else "exact two-pass (no sizer weights)"),
            "paths_per_s": world * n_paths / (ms_frame * 1e-3),
            "exact": {"value": world * n_scenes / (ms_exact * 1e-3), "unit": UNIT, "ms_per_step": ms_exact,
                      "host_syncs": stats_e[-1]["host_syncs"], "gpu_launches": stats_e[-1]["kernel_launches"]},
            "learned": ({"value": world * n_scenes / (ms_learned * 1e-3), "unit": UNIT, "ms_per_step": ms_learned,
                         "host_syncs": stats_l[-1]["host_syncs"], "gpu_launches": stats_l[-1]["kernel_launches"]}
                        if learned else None),
            **({"plain": plain, "speedup_vs_plain": plain["ms_per_step"] / ms_frame} if plain else {}),
            "sizer": sizer,
            "tuning": dict(tuning, frame_ms_tuned=ms_frame) if tuning else None,
            **({"stroke_stage": stroke_stage} if stroke_stage else {}),
            **({"svg_stage": svg_stage} if svg_stage else {}),
            "e2e": {"value": world * n_scenes / (ms_e2e * 1e-3), "unit": UNIT, "ms_per_step": ms_e2e,
                    "paths_per_s": world * n_paths / (ms_e2e * 1e-3),
                    "h2d_bytes_per_step": h2d_bytes, "d2h_bytes_per_step": img_bytes,
                    "blocks_ms_per_step": e2e_blocks,
                    "blocks": f"fastest of {E2E_BLOCKS} timed blocks of {args.steps} steps, each whole with its last "
                              f"images",
                    "images": "pf_read_images_async into pinned host memory each step (copied while the "
                              "next step runs; the last step's copy inside the timed region)"},
            "e2e_host_image": {"value": world * n_scenes / (ms_e2e_host * 1e-3), "unit": UNIT,
                               "ms_per_step": ms_e2e_host, "blocks_ms_per_step": e2e_host_blocks,
                               "images": "composited straight into pinned host memory (pf_set_host_image)"},
            "stages_ms": {k: st[k] for k in ("ms_setup", "ms_flatten", "ms_bin", "ms_propagate", "ms_lists",
                                             "ms_composite", "ms_total")},
            "counts": {k: st[k] for k in ("paths", "points", "segments", "microlines", "tiles", "fills",
                                          "alpha_tiles", "visible_tiles", "composite_entries",
                                          "composited_fills", "framebuffer_tiles", "walk_chunks", "host_syncs")},
            "roofline": {"kernel": "flatten + bin (k_flatten_pool or k_flatten, then k_bin_fused)", "bound": "hbm",
                         "achieved": fb_ach, "peak": peak, "unit": "GB/s",
                         "frac": (fb_ach / peak) if fb_ach else None, "traffic": fb_traffic,
                         "traffic_unit": "GB per frame: ncu dram__bytes_read.sum + dram__bytes_write.sum of the "
                                         "stages' kernels per algorithmic byte (the capture summarised in "
                                         "profiles/) times this frame's algorithmic bytes",
                         "algorithmic_bytes": fb_bytes,
                         "bytes_formula": "8 B x points + 8 B x segments + 12 B x fills + 4 B x visible tiles",
                         "ms": fb_ms, "peak_source": peak_src,
                         "own_layout": {"algorithmic_bytes": own_bytes,
                                        "achieved": own_bytes / (fb_ms * 1e-3) / 1e9 if fb_ms > 0 else None,
                                        "formula": "32 B x leaf lines (written, read) + 8 B x fills + 6 B x tiles "
                                                   "+ 36 B x paths"},
                         "bin_ms": bin_ms,
                         "note": "instruction bound: the exact-IEEE tile walk per leaf line"},
            "roofline_composite": {"kernel": "k_composite (fused coverage + src-over)", "bound": "hbm",
                                   "achieved": comp_ach, "peak": peak, "unit": "GB/s",
                                   "frac": (comp_ach / peak) if comp_ach else None,
                                   "traffic": comp_ratio * comp_bytes / 1e9 if comp_ratio else None,
                                   "algorithmic_bytes": comp_bytes, "ms": comp_ms,
                                   "bytes_formula": "12 B x composited fills + 16 B x composite entries + 4 B x "
                                                    "framebuffer tiles + 4 B x pixels"},
            "cpu_baseline": cpu,
            "parity": parity,
            "clocks": clk,
            "gpu_launches": int(st["kernel_launches"]) * args.steps,
        }
        print(json.dumps(line), flush=True)
    r.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
