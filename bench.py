#!/usr/bin/env python
"""Benchmark of the GPU-driven fill pipeline on one GB300 (or N replicas).

Workload (default): the batched configuration - 512 independent scenes, path
count per scene log-uniform in [16, 4096] from the 240-path cubic generator,
canvas side drawn from {256, 512, 1024, 2048} (scenes.batched()).  One step =
one pass of the pipeline over the whole batch.

Arms printed in one JSON line (rank 0):
  value        scenes/s of the batched frame (all 512 scenes in one frame),
               inputs resident in HBM when the timed region starts;
  plain        scenes/s of the plain single-scene pipeline (one frame per scene);
  e2e          scenes/s through the C-ABI from pinned host buffers: upload,
               frame and read-back of every image inside the timed region;
  roofline     the composite kernel (fused coverage + src-over), achieved bytes/s
               from its algorithmic bytes and its CUDA-event time;
  cpu_baseline the oracle port (restated d3d9 tiler + FP64 coverage/composite)
               on the host cores over a bounded sample of the batch.

--impl reference times that CPU implementation alone (the reference arm).
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
PKG = os.path.join(ROOT, "pathfinder-cpp_gb300")
sys.path.insert(0, PKG)

METRIC = "frame ms & scenes/s: batched+learned vs plain CUDA pipeline, 1 GB300, exact tiles"
# From profiles/kernels_full_batched32.md: DRAM bytes of k_bin_fused<0..2> / their algorithmic bytes.
BIN_TRAFFIC_PER_ALGORITHMIC_BYTE = 1.16
UNIT = "scenes/s"


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


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--scenes", type=int, default=512)
    ap.add_argument("--cpu-sample-every", type=int, default=32)
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
    ap.add_argument("--profile-frames", action="store_true",
                    help="only the batched exact and learned frames (warm-up + steps each), a short summary "
                         "line instead of the benchmark line: the command the committed launch lists profile")
    return ap.parse_args()


def svg_texts(n, first_seed):
    """n seeded SVG documents with 16-1024 shapes each (log-uniform)."""
    import numpy as np
    import svg_docs
    rng = np.random.default_rng(first_seed)
    sizes = np.exp(rng.uniform(np.log(16), np.log(1024), n)).astype(int)
    return [svg_docs.random_document(first_seed + i, n_shapes=int(sizes[i])) for i in range(n)]


def make_scenes(args, first_seed):
    import scenes as S
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


def workload_config(n_scenes, scenes_list, clips=0, strokes=False, gradients=False, svg=False):
    import numpy as np
    desc = ("batched: %d scenes, paths/scene log-uniform 16-4096 (cubic 8-24 seg, control points "
            "uniform over the canvas), canvas side in {256,512,1024,2048}, seeds 1000+i" % n_scenes)
    if strokes:
        desc = ("batched stroked: %d scenes, paths/scene log-uniform 16-4096, canvas side in "
                "{256,512,1024,2048}, seeds 1000+i; every path stroked (1-3 contours of 1-12 line/quad/cubic "
                "segments in a log-uniform box, 40%% closed, width 0.5-24 px, caps/joins uniform), 30%% "
                "dashed" % n_scenes)
    if svg:
        desc = ("svg: %d seeded SVG documents (svg_docs.random_document, seeds 1000+i, 16-1024 shapes each: "
                "rect/circle/ellipse/line/poly/path with all path commands, nested transforms, fills, strokes "
                "with caps/joins/dashes, linear and radial gradients), parsed by pf_svg_parse" % n_scenes)
    if gradients:
        desc += "; half of the paths painted with gradients (linear and radial, 2-5 stops, 30%% repeating)"
    if clips:
        desc += "; %d clip paths per scene (cubic 3-8 seg, a quarter to a whole canvas wide), 60%% of the " \
                "draw paths clipped" % clips
    return {
        "workload": desc,
        "scenes": n_scenes,
        "paths": int(sum(s.n_paths for s in scenes_list)),
        "points": int(sum(s.n_points for s in scenes_list)),
        "pixels": int(sum(int(np.ceil(s.width)) * int(np.ceil(s.height)) for s in scenes_list)),
        "tile": 16,
        "l2": "inputs and working set larger than L2 (129 MB) every step",
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


def cpu_baseline(scenes_list, every: int, threads: int):
    """The oracle port over every `every`-th scene: tiling + FP64 coverage/composite."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    if not os.path.exists(oracle.LIB_ORACLE):
        oracle.build()
    sample = scenes_list[::every]
    t0 = time.perf_counter()
    for s in sample:
        oracle.render(s, threads=threads)
    dt = time.perf_counter() - t0
    return len(sample) / dt, len(sample), dt


def run_reference(args, scenes_list):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    # warm-up, then K timed steps; each step renders the bounded sample
    for _ in range(max(args.warmup, 0)):
        cpu_baseline(scenes_list, args.cpu_sample_every, threads)
    times, n = [], 0
    for _ in range(args.steps):
        v, n, dt = cpu_baseline(scenes_list, args.cpu_sample_every, threads)
        times.append(dt)
    per_step = sum(times) / len(times)
    value = n / per_step
    sample = f"every {args.cpu_sample_every}th scene of the batch ({n} scenes), restated d3d9 tiler + FP64 " \
             f"coverage and src-over composite"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "runs_on": f"host CPU only, {threads} threads; no GPU is used (n_gpus is the launch's N)",
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_step * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 tiling, f64 coverage",
        "data": "synthetic", "config": workload_config(len(scenes_list), scenes_list, args.clips, args.strokes, args.gradients, args.svg),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    import numpy as np
    import scenes as S

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        scenes_list = make_scenes(args, 1000)
        run_reference(args, scenes_list)
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

    # replicas: every rank renders its own batch (seeds offset by rank); no data-path collective
    scenes_list = make_scenes(args, replica_first_seed(rank))
    bufs, views, h2d_bytes = pack_pinned(scenes_list)
    stream = torch.cuda.Stream()
    r = pfcuda.Renderer(device=local_rank, stream=stream.cuda_stream, stage_timing=True)
    r.upload_views(views)
    img_bytes = r.image_bytes()
    img_host = torch.empty(img_bytes, dtype=torch.uint8, pin_memory=True)
    n_scenes = len(scenes_list)

    def timed(fn, steps):
        barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = [fn() for _ in range(steps)]
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        ms = e0.elapsed_time(e1) / steps
        return max_over_ranks(ms, dist, "cuda"), out

    learned = os.path.exists(pfcuda.DEFAULT_WEIGHTS)
    if learned:
        r.sizer_load(pfcuda.DEFAULT_WEIGHTS)

    # 1. batched exact two-pass frame, inputs resident
    for _ in range(args.warmup):
        r.render()
    ms_exact, stats_e = timed(lambda: r.render(), args.steps)

    # 2. batched learned one-pass frame (the headline), inputs resident.  Clocks are sampled
    #    from here through the end-to-end runs.
    frame = r.render_learned if learned else r.render
    clocks = ClockSampler(local_rank)
    clocks.start()
    clocks.wait_first()
    for _ in range(args.warmup):
        frame()
    ms_batched, stats_b = timed(frame, args.steps)
    st = stats_b[-1]
    sizer = None
    if learned:
        over, pool = r.sizer_last_frame()
        sizer = {"frames_redone_exactly": int(sum(s["overflow"] for s in stats_b)), "paths_over_budget": over,
                 "spill_pool_slots_used": pool, "host_syncs": st["host_syncs"],
                 "exact_host_syncs": stats_e[-1]["host_syncs"]}

    if args.profile_frames:
        clocks.stop()
        if rank == 0:
            print(json.dumps({"profile_frames": True, "exact_ms": ms_exact, "learned_ms": ms_batched,
                              "exact_stats": stats_e[-1], "learned_stats": st}), flush=True)
        r.close()
        return

    # 3. plain single-scene pipeline (one exact frame per scene), inputs resident
    def plain_pass():
        last = None
        launches = 0
        for i in range(n_scenes):
            last = r.render(i, 1)
            launches += last["kernel_launches"]
        return launches
    plain_pass()
    ms_plain, launches_plain = timed(plain_pass, max(1, min(args.steps, 3)))

    # 4. end to end through the C-ABI: pinned H2D upload, frame, every image delivered to
    #    pinned host memory.  pf_read_images_async snapshots the images on the device and
    #    copies them to the host on the library's copy stream, so step i's images cross the
    #    link (about 190 GB/s device-to-host here) while step i+1 uploads and renders; the
    #    timed region ends after the last step's images have arrived (pf_images_wait).
    def e2e_block(steps):
        for _ in range(steps):
            r.upload_views(views)
            frame()
            r.read_images_async(img_host.data_ptr(), img_bytes)
        r.images_wait()
        return 0

    def timed_block(block, steps):
        barrier()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        block(steps)
        e1.record(stream)
        torch.cuda.synchronize()
        barrier()
        return max_over_ranks(e0.elapsed_time(e1) / steps, dist, "cuda")
    e2e_block(max(1, args.warmup // 2))
    ms_e2e = timed_block(e2e_block, args.steps)

    # the same with the composite writing the images straight into the host buffer over
    # NVLink-C2C (pf_set_host_image): the pixels cross while the composite runs
    r.set_host_image(img_host.data_ptr(), img_bytes)

    def e2e_step_host():
        r.upload_views(views)
        s = frame()
        r.read_images(img_host.data_ptr(), img_bytes)
        return s
    for _ in range(max(1, args.warmup // 2)):
        e2e_step_host()
    ms_e2e_host, _ = timed(e2e_step_host, args.steps)
    r.set_host_image(None)
    clk = clocks.stop()

    # SVG documents end to end (--svg): every step parses the documents' text on the host
    # (pf_svg_parse on a thread pool; ctypes releases the interpreter lock), uploads straight
    # from the parser's arrays, renders and delivers the images to pinned host memory
    svg_stage = None
    if args.svg:
        import concurrent.futures as cf
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
            return 0
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
    r.set_host_image(None)

    # one more (untimed) frame with the composite's work counters on, for the roofline's bytes
    r.set_flags(stage_timing=True, counters=True)
    st_c = frame()
    r.set_flags(stage_timing=True, counters=False)
    st = dict(st)
    st["composite_entries"] = st_c["composite_entries"]
    st["composited_fills"] = st_c["composited_fills"]
    st["walk_chunks"] = int(r.debug_counters()[15])  # 32-candidate chunks the composite's z-walks read

    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    peak, peak_src = 6800.0, "fallback 6.8 TB/s"
    if os.path.exists(peaks_path):
        with open(peaks_path) as f:
            peak = float(json.load(f)["hbm_gbs"])
        peak_src = "measured (MEASURED_PEAKS.json hbm_gbs)"

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
            plain = w & (sc.path_stroke["dash_count"] == 0)
            pts_per_path = np.diff(sc.contour_start.astype(np.int64)[sc.path_start.astype(np.int64)])
            stroked_in += int(pts_per_path[plain].sum())
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
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import oracle
            sample = scenes_list[::args.cpu_sample_every]
            t0 = time.perf_counter()
            for sc in sample:
                oracle.stroke_scene(sc)
            dt = time.perf_counter() - t0
            stroke_stage["cpu_baseline"] = {
                "value": len(sample) / dt, "unit": "scenes/s (stroke pass only)", "cores": 1, "kind": "port",
                "sample": f"every {args.cpu_sample_every}th scene ({len(sample)} scenes, {dt:.2f} s): restated "
                          f"OutlineDash + OutlineStrokeToFill, one thread"}
            stroke_stage["gpu_scenes_per_s"] = n_scenes / ((ms_dash + ms_stroke) * 1e-3)

    # roofline of the dominant kernel: binning (k_bin_fused, the three CTA classes, with the
    # classification and the class-3 passes that run empty here), timed by the library's
    # stage events on the frame's stream over the timed steps.  Algorithmic bytes: every leaf
    # line read once (16 B), every fill written (8 B), every tile's state and end offset
    # written (2 + 4 B), every path record read and its fill block written (32 + 4 B).
    bin_ms = sum(x["ms_bin"] for x in stats_b) / len(stats_b)
    bin_bytes = 16 * st["microlines"] + 8 * st["fills"] + 6 * st["tiles"] + 36 * st["paths"]
    bin_achieved = bin_bytes / (bin_ms * 1e-3) / 1e9 if bin_ms > 0 else None
    # DRAM bytes per algorithmic byte of the binning kernels in the ncu capture of the
    # 32-scene batch (dram__bytes_read.sum + dram__bytes_write.sum over k_bin_fused<0..2>)
    bin_traffic_ratio = BIN_TRAFFIC_PER_ALGORITHMIC_BYTE

    # roofline of the composite kernel (fused coverage + src-over)
    pixels = sum(int(np.ceil(s.width)) * int(np.ceil(s.height)) for s in scenes_list)
    comp_bytes = (8 * st["composited_fills"] + 13 * st["composite_entries"]
                  + 8 * (st["framebuffer_tiles"] + 1) + 4 * pixels)
    comp_ms = sum(x["ms_composite"] for x in stats_b) / len(stats_b)
    achieved = comp_bytes / (comp_ms * 1e-3) / 1e9 if comp_ms > 0 else None

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        v, n, dt = cpu_baseline(scenes_list, args.cpu_sample_every, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"every {args.cpu_sample_every}th scene ({n} scenes, {dt:.1f} s): restated d3d9 tiler "
                         f"+ FP64 coverage/composite"}

    if rank == 0:
        value = world * n_scenes / (ms_batched * 1e-3)
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_batched, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32 (exact-IEEE tiling), int32 fixed-point coverage", "data": "synthetic",
            "config": workload_config(n_scenes, scenes_list, args.clips, args.strokes, args.gradients, args.svg) | {"parallelism": f"replicas x{world}"},
            "frame": "batched learned one-pass" if learned else "batched exact two-pass",
            "batched_exact": {"value": world * n_scenes / (ms_exact * 1e-3), "unit": UNIT, "ms_per_step": ms_exact},
            "plain": {"value": world * n_scenes / (ms_plain * 1e-3), "unit": UNIT, "ms_per_step": ms_plain,
                      "gpu_launches_per_step": launches_plain[-1]},
            "speedup_vs_plain": ms_plain / ms_batched,
            "sizer": sizer,
            **({"stroke_stage": stroke_stage} if stroke_stage else {}),
            **({"svg_stage": svg_stage} if svg_stage else {}),
            "e2e": {"value": world * n_scenes / (ms_e2e * 1e-3), "unit": UNIT, "ms_per_step": ms_e2e,
                    "h2d_bytes_per_step": h2d_bytes, "d2h_bytes_per_step": img_bytes,
                    "images": "pf_read_images_async into pinned host memory each step (copied while the "
                              "next step runs; the last step's copy inside the timed region)"},
            "e2e_host_image": {"value": world * n_scenes / (ms_e2e_host * 1e-3), "unit": UNIT,
                               "ms_per_step": ms_e2e_host,
                               "images": "composited straight into pinned host memory (pf_set_host_image)"},
            "stages_ms": {k: st[k] for k in ("ms_setup", "ms_flatten", "ms_bin", "ms_propagate", "ms_lists",
                                             "ms_composite", "ms_total")},
            "counts": {k: st[k] for k in ("paths", "segments", "microlines", "tiles", "fills", "composite_entries",
                                          "composited_fills", "framebuffer_tiles", "walk_chunks",
                                          "host_syncs")},
            "roofline": {"kernel": "k_bin_fused (binning stage)", "bound": "hbm", "achieved": bin_achieved,
                         "peak": peak, "unit": "GB/s", "frac": (bin_achieved / peak) if bin_achieved else None,
                         "traffic": bin_traffic_ratio * bin_bytes / 1e9, "traffic_unit": "GB per launch",
                         "algorithmic_bytes": bin_bytes, "ms": bin_ms, "peak_source": peak_src,
                         "note": "latency/compute bound: the exact-IEEE tile walk per line; DRAM traffic is "
                                 "the algorithmic minimum"},
            "roofline_composite": {"kernel": "k_composite", "bound": "hbm", "achieved": achieved, "peak": peak,
                                   "unit": "GB/s", "frac": (achieved / peak) if achieved else None,
                                   "traffic": None, "algorithmic_bytes": comp_bytes, "ms": comp_ms},
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": int(st["kernel_launches"]) * args.steps,
        }
        print(json.dumps(line), flush=True)
    r.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
