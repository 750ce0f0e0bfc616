"""ctypes front end of the CPU oracle.

TEST INFRASTRUCTURE ONLY: imported by tests/, the smoke check and bench.py's
CPU-baseline leg, as the checker or the timed CPU baseline.  The product path
never imports this module.

``restated``  -> oracle/_build/libpforacle.so, the plain-C restatement
                 (pf_oracle.c) of the reference's d3d9 CPU tiler plus the FP64
                 coverage / composite oracle.
``reference`` -> oracle/_ref/libpfref.so, the reference's own tiler compiled
                 from its sources (only where the reference tree exists).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Dict, Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_ORACLE = os.path.join(HERE, "_build", "libpforacle.so")
LIB_REF = os.path.join(HERE, "_ref", "libpfref.so")


def _reference_root() -> str:
    """The reference checkout: PF_REFERENCE_ROOT, else the default of the oracle's Makefile
    (the one recipe that names where the checkout lies)."""
    env = os.environ.get("PF_REFERENCE_ROOT")
    if env:
        return env
    try:
        out = subprocess.run(["make", "-s", "-C", HERE, "ref-root"], capture_output=True, text=True, timeout=30)
        return out.stdout.strip() if out.returncode == 0 else ""
    except (OSError, subprocess.SubprocessError):
        return ""


REF_ROOT = _reference_root()

Z_D3D9 = 0
Z_D3D11 = 1


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


class Outline(C.Structure):
    _fields_ = [
        ("n_points", C.c_uint32), ("n_contours", C.c_uint32), ("n_paths", C.c_uint32),
        ("points", C.c_void_p), ("point_flags", C.c_void_p), ("contour_start", C.c_void_p),
        ("path_start", C.c_void_p), ("fill_rule", C.c_void_p),
    ]


class Result(C.Structure):
    _fields_ = [
        ("n_paths", C.c_uint32), ("path_rect", C.c_void_p), ("path_tile_first", C.c_void_p),
        ("path_column_first", C.c_void_p), ("n_tiles", C.c_uint64), ("tile_alpha", C.c_void_p),
        ("tile_backdrop", C.c_void_p), ("tile_fill_count", C.c_void_p), ("n_fills", C.c_uint64),
        ("fills", C.c_void_p), ("n_columns", C.c_uint64), ("column_backdrop", C.c_void_p),
        ("fb_tiles_x", C.c_uint32), ("fb_tiles_y", C.c_uint32), ("z", C.c_void_p),
        ("fb_list_first", C.c_void_p), ("n_list", C.c_uint64), ("fb_list", C.c_void_p),
        ("n_microlines", C.c_uint64), ("path_microlines", C.c_void_p), ("path_fills", C.c_void_p),
        ("tile_mask", C.c_void_p), ("tile_clip", C.c_void_p), ("tile_dest_backdrop", C.c_void_p),
    ]


def scene_view(scene) -> "tuple[SceneView, list]":
    """Build a pf_scene_view over a scenes.Scene; returns (view, keepalive)."""
    arrs = [np.ascontiguousarray(scene.points, np.float32), np.ascontiguousarray(scene.flags, np.uint8),
            np.ascontiguousarray(scene.contour_start, np.uint32),
            np.ascontiguousarray(scene.path_start, np.uint32),
            np.ascontiguousarray(scene.fill_rule, np.uint8), np.ascontiguousarray(scene.color, np.uint32)]
    v = SceneView(*(a.ctypes.data for a in arrs), scene.n_points, scene.n_contours, scene.n_paths,
                  scene.width, scene.height, scene.clear)
    if getattr(scene, "path_clip", None) is not None:
        clip = np.ascontiguousarray(scene.path_clip, np.uint32)
        is_clip = np.ascontiguousarray(scene.path_is_clip, np.uint8)
        v.path_clip, v.path_is_clip = clip.ctypes.data, is_clip.ctypes.data
        arrs += [clip, is_clip]
    if getattr(scene, "path_stroke", None) is not None:
        st = np.ascontiguousarray(scene.path_stroke)
        assert st.dtype.itemsize == 24
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
        v.view_box = vb.ctypes.data
        arrs.append(vb)
    v.load_action = int(getattr(scene, "load_action", 0))
    return v, arrs


def _arr(ptr, n, dtype):
    if n == 0 or not ptr:
        return np.zeros(0, dtype)
    buf = (C.c_char * (int(n) * np.dtype(dtype).itemsize)).from_address(ptr)
    return np.frombuffer(buf, dtype=dtype).copy()


def result_to_dict(r: Result) -> Dict[str, np.ndarray]:
    nfb = r.fb_tiles_x * r.fb_tiles_y
    d = {
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
    if r.path_fills:
        d["path_fills"] = _arr(r.path_fills, r.n_paths, np.uint32)
    if r.path_microlines:
        d["path_microlines"] = _arr(r.path_microlines, r.n_paths, np.uint32)
    return d


def build(reference: bool = False, quiet: bool = True) -> None:
    """Compile the restatement (and, if asked and possible, the reference harness)."""
    out = subprocess.DEVNULL if quiet else None
    subprocess.run(["make", "-C", HERE, "all"], check=True, stdout=out)
    if reference and os.path.isdir(os.path.join(REF_ROOT, "pathfinder")):
        subprocess.run(["make", "-C", HERE, "ref", "-j8", f"REF_ROOT={REF_ROOT}"], check=True, stdout=out)


_libs: Dict[str, C.CDLL] = {}


def _lib(path: str) -> C.CDLL:
    if path not in _libs:
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} is not built (run oracle.build())")
        lib = C.CDLL(path)
        _libs[path] = lib
    return _libs[path]


def have_reference() -> bool:
    return os.path.exists(LIB_REF)


def _outline_scene(scene, o: Outline):
    import dataclasses
    pts = _arr(o.points, 2 * o.n_points, np.float32).reshape(-1, 2)
    return dataclasses.replace(
        scene, points=pts, flags=_arr(o.point_flags, o.n_points, np.uint8),
        contour_start=_arr(o.contour_start, o.n_contours + 1, np.uint32),
        path_start=_arr(o.path_start, o.n_paths + 1, np.uint32),
        fill_rule=_arr(o.fill_rule, o.n_paths, np.uint8), path_stroke=None, contour_closed=None, dashes=None)


def stroke_scene(scene, reference: bool = False):
    """The scene's fill outline: stroked paths dashed and converted to stroke outlines
    (pf_stroke.c, or with reference=True the reference's own OutlineDash/OutlineStrokeToFill)."""
    lib = _lib(LIB_REF if reference else LIB_ORACLE)
    v, keep = scene_view(scene)
    o = Outline()
    st = (lib.pfref_stroke_scene if reference else lib.pfo_stroke_scene)(C.byref(v), C.byref(o))
    if st != 0:
        raise RuntimeError(f"stroke_scene failed with status {st}")
    try:
        return _outline_scene(scene, o)
    finally:
        if reference:
            for name in ("points", "point_flags", "contour_start", "path_start", "fill_rule"):
                C.CDLL(None).free(C.c_void_p(getattr(o, name)))
        else:
            lib.pfo_outline_free(C.byref(o))


class ColorStop(C.Structure):
    _fields_ = [("offset", C.c_float), ("color", C.c_uint32)]


def _ramps(scene, fn) -> np.ndarray:
    """[n_paths, 256] ramps of the gradient paths (zeros for solid paths)."""
    out = np.zeros((scene.n_paths, 256), np.uint32)
    pp = getattr(scene, "path_paint", None)
    if pp is None:
        return out
    stops = np.ascontiguousarray(scene.stops)
    for p in range(scene.n_paths):
        if pp[p]["type"] == 0:
            continue
        first, n = int(pp[p]["stop_first"]), int(pp[p]["stop_count"])
        arr = (ColorStop * max(n, 1))(*[ColorStop(float(stops[first + i]["offset"]), int(stops[first + i]["color"]))
                                        for i in range(n)])
        ramp = (C.c_uint32 * 256)()
        fn(arr, n, ramp)
        out[p] = np.frombuffer(ramp, np.uint32)
    return out


def ramps(scene) -> np.ndarray:
    """The restated gradient ramps (pf_paint.c)."""
    return _ramps(scene, _lib(LIB_ORACLE).pfo_gradient_ramp)


def reference_ramps(scene) -> np.ndarray:
    """The reference's own Gradient ramps (GradientTileBuilder::allocate's sampling)."""
    return _ramps(scene, _lib(LIB_REF).pfref_gradient_ramp)


class SvgOut(C.Structure):
    _fields_ = [("n_points", C.c_uint32), ("n_contours", C.c_uint32), ("n_paths", C.c_uint32),
                ("n_dashes", C.c_uint32), ("n_stops", C.c_uint32), ("width", C.c_float), ("height", C.c_float),
                ("points", C.c_void_p), ("point_flags", C.c_void_p), ("contour_start", C.c_void_p),
                ("contour_closed", C.c_void_p), ("path_start", C.c_void_p), ("fill_rule", C.c_void_p),
                ("color", C.c_void_p), ("path_stroke", C.c_void_p), ("dashes", C.c_void_p),
                ("path_paint", C.c_void_p), ("stops", C.c_void_p), ("ramps", C.c_void_p)]


def reference_svg_scene(text, dpi: float = 96.0) -> Dict[str, np.ndarray]:
    """The reference's nanosvg + SvgScene replay of an SVG document, in the scene layout:
    points, flags, contour_start, contour_closed, path_start, fill_rule, color, dashes (typed);
    path_stroke, path_paint, stops as raw bytes (pf_stroke 24 B, pf_paint 64 B, pf_color_stop
    8 B per item); ramps [n_paths, 256] of the reference's Gradient; width and height."""
    lib = _lib(LIB_REF)
    data = text.encode() if isinstance(text, str) else bytes(text)
    lib.pfref_svg_scene.argtypes = [C.c_char_p, C.c_size_t, C.c_float, C.POINTER(SvgOut)]
    lib.pfref_svg_free.argtypes, lib.pfref_svg_free.restype = [C.POINTER(SvgOut)], None
    o = SvgOut()
    st = lib.pfref_svg_scene(data, len(data), dpi, C.byref(o))
    if st != 0:
        raise RuntimeError(f"pfref_svg_scene failed with status {st}")
    try:
        n_p, n_c, n_n = o.n_points, o.n_contours, o.n_paths
        return {
            "points": _arr(o.points, 2 * n_p, np.float32).reshape(-1, 2),
            "flags": _arr(o.point_flags, n_p, np.uint8),
            "contour_start": _arr(o.contour_start, n_c + 1, np.uint32),
            "contour_closed": _arr(o.contour_closed, n_c, np.uint8),
            "path_start": _arr(o.path_start, n_n + 1, np.uint32),
            "fill_rule": _arr(o.fill_rule, n_n, np.uint8),
            "color": _arr(o.color, n_n, np.uint32),
            "dashes": _arr(o.dashes, o.n_dashes, np.float32),
            "path_stroke": _arr(o.path_stroke, 24 * n_n, np.uint8),
            "path_paint": _arr(o.path_paint, 64 * n_n, np.uint8),
            "stops": _arr(o.stops, 8 * o.n_stops, np.uint8),
            "ramps": _arr(o.ramps, 256 * n_n, np.uint32).reshape(-1, 256),
            "width": np.float32(o.width), "height": np.float32(o.height),
        }
    finally:
        lib.pfref_svg_free(C.byref(o))


def half_trunc(values, reference: bool = False) -> np.ndarray:
    """umHalf's float -> half -> float round trip (restated, or the reference's own)."""
    lib = _lib(LIB_REF if reference else LIB_ORACLE)
    fn = lib.pfref_half if reference else lib.pfo_half_trunc
    fn.restype, fn.argtypes = C.c_float, [C.c_float]
    return np.array([fn(float(v)) for v in np.asarray(values, np.float32)], np.float32)


def fill_scene(scene):
    """A scene with strokes turned into fills (the oracle's stroker); others unchanged."""
    st = getattr(scene, "path_stroke", None)
    if st is None or not np.any(st["line_width"] > 0):
        return scene
    return stroke_scene(scene)


def tile_scene(scene, z_rule: int = Z_D3D11, threads: int = 1) -> Dict[str, np.ndarray]:
    """Restated d3d9 tiler over a scene: canonical integer outputs."""
    lib = _lib(LIB_ORACLE)
    scene = fill_scene(scene)
    v, keep = scene_view(scene)
    r = Result()
    st = lib.pfo_tile_scene_mt(C.byref(v), C.c_int(z_rule), C.c_int(threads), C.byref(r))
    if st != 0:
        raise RuntimeError(f"pfo_tile_scene failed with status {st}")
    try:
        d = result_to_dict(r)
        d["n_microlines"] = int(r.n_microlines)
        return d
    finally:
        lib.pfo_free(C.byref(r))


def reference_tile_scene(scene) -> Dict[str, np.ndarray]:
    """The reference's own tiler (z rule D3D9) over a scene (strokes through the reference's own
    stroker first)."""
    lib = _lib(LIB_REF)
    st = getattr(scene, "path_stroke", None)
    if st is not None and np.any(st["line_width"] > 0):
        scene = stroke_scene(scene, reference=True)
    v, keep = scene_view(scene)
    r = Result()
    st = lib.pfref_tile_scene(C.byref(v), C.byref(r))
    if st != 0:
        raise RuntimeError(f"pfref_tile_scene failed with status {st}")
    try:
        return result_to_dict(r)
    finally:
        lib.pfref_free(C.byref(r))


def render(scene, z_rule: int = Z_D3D11, threads: int = 1, coverage: bool = False,
           tiled: Optional[Dict[str, np.ndarray]] = None, dest: Optional[np.ndarray] = None):
    """FP64 analytic-area coverage + src-over composite; returns (rgba u8 [H,W,4], coverage|None).
    A scene with load_action 1 composites over ``dest`` (u8 [H,W,4]; zeros when None)."""
    lib = _lib(LIB_ORACLE)
    scene = fill_scene(scene)
    v, keep = scene_view(scene)
    r = Result()
    st = lib.pfo_tile_scene_mt(C.byref(v), C.c_int(z_rule), C.c_int(threads), C.byref(r))
    if st != 0:
        raise RuntimeError(f"pfo_tile_scene failed with status {st}")
    try:
        w = int(np.ceil(scene.width))
        h = int(np.ceil(scene.height))
        rgba = np.zeros((h, w, 4), np.uint8)
        if dest is not None:
            rgba[...] = np.asarray(dest, np.uint8).reshape(h, w, 4)
        cov = np.zeros((int(r.n_tiles), 16, 16), np.float32) if coverage else None
        st = lib.pfo_render(C.byref(v), C.byref(r), C.c_void_p(rgba.ctypes.data),
                            C.c_void_p(cov.ctypes.data if cov is not None else 0), C.c_int(threads))
        if st != 0:
            raise RuntimeError(f"pfo_render failed with status {st}")
        if tiled is not None:
            tiled.update(result_to_dict(r))
        return rgba, cov
    finally:
        lib.pfo_free(C.byref(r))


def composite_lists(d: Dict[str, np.ndarray]):
    """Per framebuffer tile composite list as a list of int arrays."""
    first = d["fb_list_first"].astype(np.int64)
    return [d["fb_list"][first[i]:first[i + 1]] for i in range(len(first) - 1)]


def compare(a: Dict[str, np.ndarray], b: Dict[str, np.ndarray], keys=None) -> list:
    """Names of canonical arrays that differ between two results."""
    keys = keys or ["path_rect", "path_tile_first", "path_column_first", "tile_alpha",
                    "tile_backdrop", "tile_fill_count", "fills", "column_backdrop", "fb_tiles",
                    "fb_list_first", "fb_list", "tile_mask", "tile_clip", "tile_dest_backdrop"]
    bad = []
    for k in keys:
        if a[k].shape != b[k].shape or not np.array_equal(a[k], b[k]):
            bad.append(k)
    return bad
