"""Python front end of libpfcuda.so (the C-ABI in include/pfcuda.h).

This mirrors the reference's per-frame flow, ``Canvas::draw``
(pathfinder/core/canvas.cpp:557-567): a scene is handed to the renderer
(``Renderer`` = :class:`Renderer` here, one CUDA context), drawn, and the
destination image read back.  The CUDA library is required: there is no CPU
fallback, and constructing a :class:`Renderer` without the built library or
without a GPU raises.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from typing import Dict, List, Optional, Sequence

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# PFCUDA_LIB: another build of the library to load (the in-tree build by default)
LIB_PATH = os.environ.get("PFCUDA_LIB") or os.path.join(HERE, "_build", "libpfcuda.so")

PF_OK = 0
PF_CONFIG_STAGE_TIMING = 0x1
PF_CONFIG_FRAME_COUNTERS = 0x2

EXPORTS = [
    "pf_abi_version", "pf_device_count", "pf_ctx_create", "pf_ctx_destroy", "pf_last_error",
    "pf_scene_upload", "pf_scene_upload_batch", "pf_render", "pf_render_scenes", "pf_read_image", "pf_read_image_scene",
    "pf_image_device_ptr", "pf_read_canon", "pf_read_canon_scene", "pf_read_coverage", "pf_draw",
    "pf_image_bytes", "pf_image_offset", "pf_read_images", "pf_render_learned", "pf_sizer_param_count",
    "pf_sizer_init", "pf_sizer_set_params", "pf_sizer_get_params", "pf_sizer_set_margin", "pf_sizer_predict",
    "pf_sizer_gradient", "pf_sizer_train", "pf_sizer_save", "pf_sizer_load", "pf_path_features", "pf_path_counts",
    "pf_sizer_last_frame", "pf_debug_counters", "pf_ctx_set_flags", "pf_sizer_predict_noalloc",
    "pf_set_host_image", "pf_read_outline", "pf_upload_stats_get", "pf_svg_parse", "pf_svg_scene", "pf_svg_free",
    "pf_read_images_async", "pf_images_wait", "pf_write_image", "pf_render_auto", "pf_auto_choice",
    "pf_tuning_get", "pf_tuning_set", "pf_autotune",
]

N_FEATURES = 12
N_OUTPUTS = 2
DEFAULT_WEIGHTS = os.path.join(HERE, "weights", "sizer.bin")
# launch parameters found by the autotuner (tune.py) for the batched configuration
DEFAULT_RENDER_CONFIG = os.path.join(HERE, "weights", "render_config.json")


class Tuning(C.Structure):
    """pf_tuning: the launch parameters of the frame's kernels."""
    _fields_ = [("bin_ctas_per_sm", C.c_uint32 * 3), ("long_line", C.c_float), ("bin_concurrent", C.c_uint32),
                ("seg_sorted", C.c_uint32), ("composite_ticket", C.c_uint32), ("reserved", C.c_uint32 * 8)]

    KEYS = ("bin_ctas_per_sm", "long_line", "bin_concurrent", "seg_sorted", "composite_ticket")

    def to_dict(self) -> Dict[str, object]:
        return {"bin_ctas_per_sm": list(self.bin_ctas_per_sm), "long_line": float(self.long_line),
                "bin_concurrent": int(self.bin_concurrent), "seg_sorted": int(self.seg_sorted),
                "composite_ticket": int(self.composite_ticket)}

    @classmethod
    def from_dict(cls, d: Dict[str, object]) -> "Tuning":
        t = cls()
        t.bin_ctas_per_sm[:] = [int(v) for v in d["bin_ctas_per_sm"]]
        t.long_line = float(d["long_line"])
        t.bin_concurrent = int(d["bin_concurrent"])
        t.seg_sorted = int(d["seg_sorted"])
        t.composite_ticket = int(d.get("composite_ticket", 0))
        return t


class Stroke(C.Structure):
    """pf_stroke (the numpy layout is scenes.STROKE_DTYPE)."""
    _fields_ = [("line_width", C.c_float), ("miter_limit", C.c_float), ("line_cap", C.c_uint8),
                ("line_join", C.c_uint8), ("reserved", C.c_uint16), ("dash_first", C.c_uint32),
                ("dash_count", C.c_uint32), ("dash_offset", C.c_float)]


class SceneView(C.Structure):
    _fields_ = [
        ("points", C.c_void_p), ("point_flags", C.c_void_p), ("contour_start", C.c_void_p),
        ("path_start", C.c_void_p), ("fill_rule", C.c_void_p), ("color", C.c_void_p),
        ("n_points", C.c_uint32), ("n_contours", C.c_uint32), ("n_paths", C.c_uint32),
        ("width", C.c_float), ("height", C.c_float), ("clear_color", C.c_uint32),
        ("path_clip", C.c_void_p), ("path_is_clip", C.c_void_p),
        ("path_stroke", C.c_void_p), ("contour_closed", C.c_void_p), ("dashes", C.c_void_p),
        ("n_dashes", C.c_uint32), ("path_paint", C.c_void_p), ("stops", C.c_void_p), ("n_stops", C.c_uint32),
        ("view_box", C.c_void_p), ("load_action", C.c_uint32),
    ]


class Config(C.Structure):
    _fields_ = [("device", C.c_int), ("stream", C.c_void_p), ("flags", C.c_uint32),
                ("reserved", C.c_uint32 * 8)]


class FrameStats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in (
        "paths", "contours", "points", "segments", "microlines", "tiles", "fills", "alpha_tiles",
        "visible_tiles", "composite_entries", "framebuffer_tiles")] + [
        ("overflow", C.c_uint32), ("kernel_error", C.c_uint32)] + [
        (n, C.c_float) for n in ("ms_setup", "ms_flatten", "ms_bin", "ms_propagate", "ms_lists",
                                 "ms_composite", "ms_total")] + [
        ("composited_fills", C.c_uint64), ("kernel_launches", C.c_uint32), ("host_syncs", C.c_uint32)]

    def to_dict(self) -> Dict[str, float]:
        return {n: getattr(self, n) for n, _ in self._fields_}


class Canon(C.Structure):
    _fields_ = [
        ("n_paths", C.c_uint32), ("path_rect", C.c_void_p), ("path_tile_first", C.c_void_p),
        ("path_column_first", C.c_void_p), ("n_tiles", C.c_uint64), ("tile_alpha", C.c_void_p),
        ("tile_backdrop", C.c_void_p), ("tile_fill_count", C.c_void_p), ("n_fills", C.c_uint64),
        ("fills", C.c_void_p), ("n_columns", C.c_uint64), ("column_backdrop", C.c_void_p),
        ("fb_tiles_x", C.c_uint32), ("fb_tiles_y", C.c_uint32), ("z", C.c_void_p),
        ("fb_list_first", C.c_void_p), ("n_list", C.c_uint64), ("fb_list", C.c_void_p),
        ("tile_mask", C.c_void_p), ("tile_clip", C.c_void_p), ("tile_dest_backdrop", C.c_void_p),
    ]


class OutlineOut(C.Structure):
    _fields_ = [
        ("n_points", C.c_uint32), ("n_contours", C.c_uint32), ("n_paths", C.c_uint32),
        ("points", C.c_void_p), ("point_flags", C.c_void_p), ("contour_start", C.c_void_p),
        ("path_start", C.c_void_p), ("fill_rule", C.c_void_p),
    ]


class UploadStats(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in ("n_points", "n_contours", "stroked_paths", "dashed_paths",
                                          "stroke_contours", "dash_points")] + \
               [("ms_dash", C.c_float), ("ms_stroke", C.c_float)]


class PfError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"pfcuda status {status}: {msg}")
        self.status = status


_lib: Optional[C.CDLL] = None


def load(path: str = LIB_PATH) -> C.CDLL:
    """Load libpfcuda.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} is not built; run pathfinder-cpp_gb300/build.py")
        lib = C.CDLL(path)
        lib.pf_last_error.restype = C.c_char_p
        lib.pf_last_error.argtypes = [C.c_void_p]
        for name in EXPORTS:
            if name == "pf_last_error":
                continue
            if not hasattr(lib, name):
                if path == os.path.join(HERE, "_build", "libpfcuda.so"):
                    raise AttributeError(f"{path} does not export {name}")
                continue  # another build (PFCUDA_LIB) of an older ABI: its entry points only
            getattr(lib, name).restype = C.c_int
        lib.pf_svg_parse.argtypes = [C.c_char_p, C.c_size_t, C.c_float, C.POINTER(C.c_void_p)]
        lib.pf_svg_scene.argtypes = [C.c_void_p, C.c_void_p]
        lib.pf_svg_free.argtypes, lib.pf_svg_free.restype = [C.c_void_p], None
        _lib = lib
    return _lib


def scene_view(scene) -> "tuple[SceneView, list]":
    """pf_scene_view over a scenes.Scene (numpy arrays); returns (view, keepalive)."""
    arrs = [np.ascontiguousarray(scene.points, np.float32), np.ascontiguousarray(scene.flags, np.uint8),
            np.ascontiguousarray(scene.contour_start, np.uint32),
            np.ascontiguousarray(scene.path_start, np.uint32),
            np.ascontiguousarray(scene.fill_rule, np.uint8), np.ascontiguousarray(scene.color, np.uint32)]
    v = SceneView(*(a.ctypes.data for a in arrs), scene.n_points, scene.n_contours, scene.n_paths,
                  scene.width, scene.height, scene.clear)
    # the clip arrays go in as given (the library checks that they come together)
    if getattr(scene, "path_clip", None) is not None:
        clip = np.ascontiguousarray(scene.path_clip, np.uint32)
        v.path_clip = clip.ctypes.data
        arrs.append(clip)
    if getattr(scene, "path_is_clip", None) is not None:
        is_clip = np.ascontiguousarray(scene.path_is_clip, np.uint8)
        v.path_is_clip = is_clip.ctypes.data
        arrs.append(is_clip)
    if getattr(scene, "path_stroke", None) is not None:
        st = np.ascontiguousarray(scene.path_stroke)
        if st.dtype.itemsize != C.sizeof(Stroke):
            raise ValueError("path_stroke must use scenes.STROKE_DTYPE (pf_stroke)")
        v.path_stroke = st.ctypes.data
        arrs.append(st)
    if getattr(scene, "contour_closed", None) is not None:
        cc = np.ascontiguousarray(scene.contour_closed, np.uint8)
        v.contour_closed = cc.ctypes.data
        arrs.append(cc)
    if getattr(scene, "dashes", None) is not None:
        d = np.ascontiguousarray(scene.dashes, np.float32)
        v.dashes, v.n_dashes = d.ctypes.data, len(d)
        arrs.append(d)
    if getattr(scene, "path_paint", None) is not None:
        pp = np.ascontiguousarray(scene.path_paint)
        if pp.dtype.itemsize != 64:
            raise ValueError("path_paint must use scenes.PAINT_DTYPE (pf_paint)")
        st_ = np.ascontiguousarray(scene.stops)
        v.path_paint, v.stops, v.n_stops = pp.ctypes.data, st_.ctypes.data, len(st_)
        arrs += [pp, st_]
    if getattr(scene, "view_box", None) is not None:
        vb = np.ascontiguousarray(scene.view_box, np.float32)
        if vb.shape != (4,):
            raise ValueError("view_box is (left, top, right, bottom)")
        v.view_box = vb.ctypes.data
        arrs.append(vb)
    v.load_action = int(getattr(scene, "load_action", 0))
    return v, arrs


def _arr(ptr, n, dtype):
    if n == 0 or not ptr:
        return np.zeros(0, dtype)
    buf = (C.c_char * (int(n) * np.dtype(dtype).itemsize)).from_address(ptr)
    return np.frombuffer(buf, dtype=dtype).copy()


class SvgDocument:
    """A parsed SVG document (pf_svg): its scene view points into the parser's own arrays, so
    ``Renderer.upload_views([doc.view])`` hands the document to the GPU without a copy.

    The reference's SvgScene (pathfinder/core/svg.cpp:135-205): nanosvg's parse replayed through
    the canvas, one fill path and one stroke path per shape where their paints are visible.
    Strokes stay strokes (path_stroke); the upload converts them on the GPU.  Host code: no GPU
    is needed to parse."""

    def __init__(self, text, dpi: float = 96.0):
        self.lib = load()
        data = text.encode() if isinstance(text, str) else bytes(text)
        self.handle = C.c_void_p()
        st = self.lib.pf_svg_parse(data, len(data), dpi, C.byref(self.handle))
        if st != PF_OK:
            raise PfError(st, "pf_svg_parse failed")
        self.view = SceneView()
        self.lib.pf_svg_scene(self.handle, C.byref(self.view))

    def close(self) -> None:
        if self.handle:
            self.lib.pf_svg_free(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def scene(self):
        """The document as a scenes.Scene (numpy copies of the view's arrays)."""
        import scenes as S
        v = self.view
        n_p, n_c, n_n = v.n_points, v.n_contours, v.n_paths
        sc = S.Scene(points=_arr(v.points, 2 * n_p, np.float32).reshape(-1, 2),
                     flags=_arr(v.point_flags, n_p, np.uint8),
                     contour_start=_arr(v.contour_start, n_c + 1, np.uint32),
                     path_start=_arr(v.path_start, n_n + 1, np.uint32),
                     fill_rule=_arr(v.fill_rule, n_n, np.uint8), color=_arr(v.color, n_n, np.uint32),
                     width=float(v.width), height=float(v.height))
        sc.path_stroke = _arr(v.path_stroke, n_n, S.STROKE_DTYPE)
        sc.contour_closed = _arr(v.contour_closed, n_c, np.uint8)
        sc.dashes = _arr(v.dashes, v.n_dashes, np.float32)
        sc.path_paint = _arr(v.path_paint, n_n, S.PAINT_DTYPE)
        sc.stops = _arr(v.stops, v.n_stops, S.STOP_DTYPE)
        return sc


def parse_svg(text, dpi: float = 96.0):
    """An SVG document as a scenes.Scene (see :class:`SvgDocument`)."""
    with SvgDocument(text, dpi) as doc:
        return doc.scene()


class Renderer:
    """One CUDA context: upload scenes, draw them, read images and tile data back."""

    def __init__(self, device: int = 0, stream: int = 0, stage_timing: bool = False, counters: bool = False):
        self.lib = load()
        flags = (PF_CONFIG_STAGE_TIMING if stage_timing else 0) | (PF_CONFIG_FRAME_COUNTERS if counters else 0)
        cfg = Config(device, C.c_void_p(stream or None), flags)
        h = C.c_void_p()
        self._check(self.lib.pf_ctx_create(C.byref(cfg), C.byref(h)), None)
        self.ctx = h
        self._sizes: List[tuple] = []

    def _check(self, st: int, ctx) -> None:
        if st != PF_OK:
            msg = self.lib.pf_last_error(ctx)
            raise PfError(st, msg.decode() if msg else "")

    def close(self) -> None:
        if getattr(self, "ctx", None):
            self.lib.pf_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # -- frame ---------------------------------------------------------------
    def upload(self, scenes) -> None:
        if not isinstance(scenes, (list, tuple)):
            scenes = [scenes]
        views, keep = [], []
        for s in scenes:
            v, k = scene_view(s)
            views.append(v)
            keep.append(k)
        arr = (SceneView * len(views))(*views)
        self._check(self.lib.pf_scene_upload_batch(self.ctx, arr, len(views)), self.ctx)
        self._sizes = [(math.ceil(s.width), math.ceil(s.height)) for s in scenes]

    def render(self, first: int = 0, count: Optional[int] = None) -> Dict[str, float]:
        """Exact two-pass frame over uploaded scenes [first, first + count) (default: all)."""
        st = FrameStats()
        if count is None:
            count = len(self._sizes) - first
        self._check(self.lib.pf_render_scenes(self.ctx, first, count, C.byref(st)), self.ctx)
        return st.to_dict()

    def image(self, scene: int = 0) -> np.ndarray:
        w, h = self._sizes[scene]
        out = np.empty((h, w, 4), np.uint8)
        self._check(self.lib.pf_read_image_scene(self.ctx, scene, C.c_void_p(out.ctypes.data), out.nbytes),
                    self.ctx)
        return out

    def write_image(self, scene: int, rgba: np.ndarray) -> None:
        """Put pixels into a scene's destination image, for a frame with load_action 1 (LOAD)."""
        w, h = self._sizes[scene]
        rgba = np.ascontiguousarray(rgba, np.uint8)
        if rgba.size != w * h * 4:
            raise ValueError(f"scene {scene} needs a {h}x{w}x4 image")
        self._check(self.lib.pf_write_image(self.ctx, scene, C.c_void_p(rgba.ctypes.data), C.c_size_t(rgba.nbytes)),
                    self.ctx)

    def upload_stats(self) -> Dict[str, float]:
        """The last upload's stroke pass: outline sizes, stroked/dashed paths, device times."""
        r = UploadStats()
        self._check(self.lib.pf_upload_stats_get(self.ctx, C.byref(r)), self.ctx)
        return {n: getattr(r, n) for n, _ in r._fields_}

    def outline(self, scene: int = 0) -> Dict[str, np.ndarray]:
        """The scene's fill outline as the frames tile it (strokes converted)."""
        r = OutlineOut()
        self._check(self.lib.pf_read_outline(self.ctx, scene, C.byref(r)), self.ctx)
        return {
            "points": _arr(r.points, 2 * r.n_points, np.float32).reshape(-1, 2),
            "flags": _arr(r.point_flags, r.n_points, np.uint8),
            "contour_start": _arr(r.contour_start, r.n_contours + 1, np.uint32),
            "path_start": _arr(r.path_start, r.n_paths + 1, np.uint32),
            "fill_rule": _arr(r.fill_rule, r.n_paths, np.uint8),
        }

    def canon(self, scene: int = 0) -> Dict[str, np.ndarray]:
        r = Canon()
        self._check(self.lib.pf_read_canon_scene(self.ctx, scene, C.byref(r)), self.ctx)
        nfb = r.fb_tiles_x * r.fb_tiles_y
        return {
            "path_rect": _arr(r.path_rect, 4 * r.n_paths, np.int32).reshape(-1, 4),
            "path_tile_first": _arr(r.path_tile_first, r.n_paths + 1, np.uint64),
            "path_column_first": _arr(r.path_column_first, r.n_paths + 1, np.uint64),
            "tile_alpha": _arr(r.tile_alpha, r.n_tiles, np.uint8),
            "tile_backdrop": _arr(r.tile_backdrop, r.n_tiles, np.int8),
            "tile_fill_count": _arr(r.tile_fill_count, r.n_tiles, np.uint32),
            "fills": _arr(r.fills, 4 * r.n_fills, np.uint16).reshape(-1, 4),
            "column_backdrop": _arr(r.column_backdrop, r.n_columns, np.int32),
            "fb_tiles": np.array([r.fb_tiles_x, r.fb_tiles_y], np.uint32),
            "z": _arr(r.z, nfb, np.int32),
            "fb_list_first": _arr(r.fb_list_first, nfb + 1, np.uint64),
            "fb_list": _arr(r.fb_list, r.n_list, np.uint32),
            "tile_mask": _arr(r.tile_mask, r.n_tiles, np.uint8),
            "tile_clip": _arr(r.tile_clip, r.n_tiles, np.uint64),
            "tile_dest_backdrop": _arr(r.tile_dest_backdrop, r.n_tiles, np.int8),
        }

    def set_flags(self, stage_timing: bool = False, counters: bool = False) -> None:
        flags = (PF_CONFIG_STAGE_TIMING if stage_timing else 0) | (PF_CONFIG_FRAME_COUNTERS if counters else 0)
        self._check(self.lib.pf_ctx_set_flags(self.ctx, C.c_uint32(flags)), self.ctx)

    def debug_counters(self) -> np.ndarray:
        out = np.zeros(16, np.uint32)
        self._check(self.lib.pf_debug_counters(self.ctx, C.c_void_p(out.ctypes.data), C.c_size_t(16)), self.ctx)
        return out

    def image_bytes(self) -> int:
        n = C.c_uint64()
        self._check(self.lib.pf_image_bytes(self.ctx, C.byref(n)), self.ctx)
        return n.value

    def image_offset(self, scene: int) -> int:
        n = C.c_uint64()
        self._check(self.lib.pf_image_offset(self.ctx, scene, C.byref(n)), self.ctx)
        return n.value

    def read_images(self, dst_ptr: int, capacity: int) -> None:
        """Copy every image of the batch into host memory at dst_ptr (one transfer)."""
        self._check(self.lib.pf_read_images(self.ctx, C.c_void_p(dst_ptr), C.c_size_t(capacity)), self.ctx)

    def read_images_async(self, dst_ptr: int, capacity: int) -> None:
        """Start delivering the last frame's images to dst (pinned host memory); returns at once.
        Call images_wait() before reading dst."""
        self._check(self.lib.pf_read_images_async(self.ctx, C.c_void_p(dst_ptr), C.c_size_t(capacity)), self.ctx)

    def images_wait(self) -> None:
        self._check(self.lib.pf_images_wait(self.ctx), self.ctx)

    def set_host_image(self, host_ptr: Optional[int], capacity: int = 0) -> None:
        """Composite later frames straight into host memory at host_ptr (None: device images)."""
        self._check(self.lib.pf_set_host_image(self.ctx, C.c_void_p(host_ptr or 0), C.c_size_t(capacity)),
                    self.ctx)

    def upload_views(self, views) -> None:
        """Upload a batch described by ready-made SceneView structs (host pointers)."""
        arr = (SceneView * len(views))(*views)
        self._check(self.lib.pf_scene_upload_batch(self.ctx, arr, len(views)), self.ctx)
        self._sizes = [(math.ceil(v.width), math.ceil(v.height)) for v in views]

    # -- learned frame and sizer -------------------------------------------------
    def render_learned(self, first: int = 0, count: Optional[int] = None) -> Dict[str, float]:
        """One-pass frame with sizer-predicted buffers (falls back to the exact frame on overflow)."""
        st = FrameStats()
        if count is None:
            count = len(self._sizes) - first
        self._check(self.lib.pf_render_learned(self.ctx, first, count, C.byref(st)), self.ctx)
        return st.to_dict()

    def render_auto(self, first: int = 0, count: Optional[int] = None) -> Dict[str, float]:
        """The frame the library picks: the learned one where it measured faster, else the exact one."""
        st = FrameStats()
        if count is None:
            count = len(self._sizes) - first
        self._check(self.lib.pf_render_auto(self.ctx, first, count, C.byref(st)), self.ctx)
        return st.to_dict()

    def last_auto_choice(self) -> Dict[str, object]:
        """What render_auto did: the frame its last call ran, the settled choice (None while it is
        still timing) and the device times it measured."""
        last, choice = C.c_int(), C.c_int()
        ems, lms = C.c_float(), C.c_float()
        self._check(self.lib.pf_auto_choice(self.ctx, C.byref(last), C.byref(choice), C.byref(ems), C.byref(lms)),
                    self.ctx)
        names = {0: "exact", 1: "learned"}
        return {"last": names[last.value], "choice": names.get(choice.value), "exact_ms": ems.value,
                "learned_ms": lms.value}

    # -- launch parameters and the autotuner ------------------------------------------------
    def tuning(self) -> Dict[str, object]:
        t = Tuning()
        self._check(self.lib.pf_tuning_get(self.ctx, C.byref(t)), self.ctx)
        return t.to_dict()

    def set_tuning(self, d: Dict[str, object]) -> None:
        t = Tuning.from_dict(d)
        self._check(self.lib.pf_tuning_set(self.ctx, C.byref(t)), self.ctx)

    def load_render_config(self, path: str = DEFAULT_RENDER_CONFIG) -> Dict[str, object]:
        """Apply the launch parameters of a RenderConfig JSON file (tune.py writes it)."""
        import json
        with open(path) as f:
            cfg = json.load(f)
        self.set_tuning(cfg["tuning"])
        return cfg

    def autotune(self, first: int = 0, count: Optional[int] = None, frames: int = 5):
        """Search the launch parameters on the uploaded scenes; returns (best, best_ms, start_ms)
        and leaves the best set."""
        if count is None:
            count = len(self._sizes) - first
        t = Tuning()
        best, start = C.c_float(), C.c_float()
        self._check(self.lib.pf_autotune(self.ctx, first, count, frames, C.byref(t), C.byref(best), C.byref(start)),
                    self.ctx)
        return t.to_dict(), best.value, start.value

    def sizer_init(self, seed: int = 0) -> None:
        self._check(self.lib.pf_sizer_init(self.ctx, C.c_uint64(seed)), self.ctx)

    def sizer_params(self) -> np.ndarray:
        n = self.lib.pf_sizer_param_count()
        out = np.empty(n, np.float32)
        self._check(self.lib.pf_sizer_get_params(self.ctx, C.c_void_p(out.ctypes.data), C.c_size_t(n)), self.ctx)
        return out

    def set_sizer_params(self, params: np.ndarray) -> None:
        params = np.ascontiguousarray(params, np.float32)
        self._check(self.lib.pf_sizer_set_params(self.ctx, C.c_void_p(params.ctypes.data), C.c_size_t(params.size)),
                    self.ctx)

    def sizer_margin(self, mul: float, add: float, pool: float = 0.10) -> None:
        self._check(self.lib.pf_sizer_set_margin(self.ctx, C.c_float(mul), C.c_float(add), C.c_float(pool)),
                    self.ctx)

    def sizer_last_frame(self):
        """(paths over their leaf budget, spill-pool slots used) of the last learned frame."""
        a, b = C.c_uint32(), C.c_uint32()
        self._check(self.lib.pf_sizer_last_frame(self.ctx, C.byref(a), C.byref(b)), self.ctx)
        return a.value, b.value

    def sizer_predict(self, feat: np.ndarray) -> np.ndarray:
        feat = np.ascontiguousarray(feat, np.float32)
        out = np.empty((feat.shape[0], N_OUTPUTS), np.float32)
        self._check(self.lib.pf_sizer_predict(self.ctx, C.c_void_p(feat.ctypes.data), C.c_uint32(feat.shape[0]),
                                              C.c_void_p(out.ctypes.data)), self.ctx)
        return out

    def sizer_gradient(self, feat: np.ndarray, target: np.ndarray):
        feat = np.ascontiguousarray(feat, np.float32)
        target = np.ascontiguousarray(target, np.float32)
        grad = np.empty(self.lib.pf_sizer_param_count(), np.float32)
        loss = C.c_float()
        self._check(self.lib.pf_sizer_gradient(self.ctx, C.c_void_p(feat.ctypes.data), C.c_void_p(target.ctypes.data),
                                               C.c_uint32(feat.shape[0]), C.c_void_p(grad.ctypes.data),
                                               C.byref(loss)), self.ctx)
        return grad, loss.value

    def sizer_train(self, feat: np.ndarray, target: np.ndarray, epochs: int, batch: int = 4096, lr: float = 1e-3,
                    seed: int = 0) -> np.ndarray:
        feat = np.ascontiguousarray(feat, np.float32)
        target = np.ascontiguousarray(target, np.float32)
        losses = np.zeros(epochs, np.float32)
        self._check(self.lib.pf_sizer_train(self.ctx, C.c_void_p(feat.ctypes.data), C.c_void_p(target.ctypes.data),
                                            C.c_uint32(feat.shape[0]), C.c_uint32(epochs), C.c_uint32(batch),
                                            C.c_float(lr), C.c_uint64(seed), C.c_void_p(losses.ctypes.data)),
                    self.ctx)
        return losses

    def sizer_save(self, path: str) -> None:
        self._check(self.lib.pf_sizer_save(self.ctx, path.encode()), self.ctx)

    def sizer_load(self, path: str = DEFAULT_WEIGHTS) -> None:
        self._check(self.lib.pf_sizer_load(self.ctx, path.encode()), self.ctx)

    def path_features(self, n_paths: int) -> np.ndarray:
        out = np.empty((n_paths, N_FEATURES), np.float32)
        self._check(self.lib.pf_path_features(self.ctx, C.c_void_p(out.ctypes.data), C.c_size_t(out.size)),
                    self.ctx)
        return out

    def path_counts(self, n_paths: int):
        leaves = np.empty(n_paths, np.uint32)
        fills = np.empty(n_paths, np.uint32)
        self._check(self.lib.pf_path_counts(self.ctx, C.c_void_p(leaves.ctypes.data), C.c_void_p(fills.ctypes.data),
                                            C.c_size_t(n_paths)), self.ctx)
        return leaves, fills

    def coverage(self) -> np.ndarray:
        n = C.c_uint64()
        self._check(self.lib.pf_read_coverage(self.ctx, None, C.c_size_t(0), C.byref(n)), self.ctx)
        out = np.empty((n.value, 16, 16), np.float32)
        self._check(self.lib.pf_read_coverage(self.ctx, C.c_void_p(out.ctypes.data), C.c_size_t(out.size),
                                              C.byref(n)), self.ctx)
        return out

    def draw(self, scene) -> np.ndarray:
        """Upload, render and read back one scene (the whole frame through the C-ABI)."""
        v, keep = scene_view(scene)
        w, h = int(np.ceil(scene.width)), int(np.ceil(scene.height))
        out = np.empty((h, w, 4), np.uint8)
        self._check(self.lib.pf_draw(self.ctx, C.byref(v), C.c_void_p(out.ctypes.data), out.nbytes, None),
                    self.ctx)
        self._sizes = [(w, h)]
        return out


def device_count() -> int:
    lib = load()
    n = C.c_int(0)
    st = lib.pf_device_count(C.byref(n))
    return n.value if st == PF_OK else 0
