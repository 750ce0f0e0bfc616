"""Seeded synthetic scenes for the GPU-driven fill pipeline.

A scene is stored the way the reference's ``Scene`` holds its draw paths
(``pathfinder/core/scene.h``): every draw path owns an ``Outline`` made of
``Contour``s, and every contour is a run of points with a ``PointFlag`` per
point (``pathfinder/core/data/data.h:120-129``: 0 = on-curve, 1 = first
control point, 2 = second control point).  Outlines are already in canvas
space (``Canvas::push_path`` applies the transform before the tiler runs,
``pathfinder/core/canvas.cpp:180-190``).

The random stream is a counter-based splitmix64 in numpy ``uint64`` arithmetic,
and every coordinate is made from +, -, *, / and sqrt only, so a scene is the
same bit for bit on x86 and Arm hosts (no libm transcendental is involved).

Generators (their shapes follow the benchmark configurations):

* :func:`plain_small`  - closed paths of 8-24 cubic segments, control points
  uniform over the canvas, nonzero rule, opaque colours.
* :func:`large_single` - log-uniform path boxes (8-2048 px), 60 % cubic /
  40 % quadratic segments, alternating nonzero / even-odd, 30 % translucent.
* :func:`glyphs`       - many small quadratic outlines with 1-3 contours on a
  jittered grid; inner contours run the other way so they cut holes.
* :func:`batched`      - a list of independent scenes of uneven size.
* :func:`mixed`        - a mixture of the three path families on one canvas.
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional

import numpy as np

# pf_stroke (include/pfcuda.h): StrokeStyle plus the canvas's line dash
STROKE_DTYPE = np.dtype([("line_width", "<f4"), ("miter_limit", "<f4"), ("line_cap", "u1"),
                         ("line_join", "u1"), ("reserved", "<u2"), ("dash_first", "<u4"),
                         ("dash_count", "<u4"), ("dash_offset", "<f4")])
CAP_BUTT, CAP_SQUARE, CAP_ROUND = 0, 1, 2
# pf_paint / pf_color_stop (include/pfcuda.h): gradient paints
PAINT_DTYPE = np.dtype([("type", "<u4"), ("wrap", "<u4"), ("stop_first", "<u4"), ("stop_count", "<u4"),
                        ("line", "<f4", (4,)), ("radii", "<f4", (2,)), ("transform", "<f4", (6,))])
STOP_DTYPE = np.dtype([("offset", "<f4"), ("color", "<u4")])
PAINT_SOLID, PAINT_LINEAR, PAINT_RADIAL = 0, 1, 2
WRAP_CLAMP, WRAP_REPEAT = 0, 1
JOIN_MITER, JOIN_BEVEL, JOIN_ROUND = 0, 1, 2

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def _mix(z: np.ndarray) -> np.ndarray:
    z = (z ^ (z >> np.uint64(30))) * _M1
    z = (z ^ (z >> np.uint64(27))) * _M2
    return z ^ (z >> np.uint64(31))


class Rng:
    """Counter-based splitmix64 stream (platform independent)."""

    def __init__(self, seed: int, stream: int = 0):
        with np.errstate(over="ignore"):
            base = np.array([seed * 0x100000001B3 + stream * 0x9E37 + 1], dtype=np.uint64)
            self._key = _mix(base * _GOLDEN)[0]
        self._ctr = 0

    def bits(self, n: int) -> np.ndarray:
        idx = np.arange(self._ctr, self._ctr + n, dtype=np.uint64)
        self._ctr += n
        with np.errstate(over="ignore"):
            return _mix(idx * _GOLDEN + self._key)

    def uniform(self, n: int) -> np.ndarray:
        """float64 in [0, 1)."""
        return (self.bits(n) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)

    def integers(self, lo: int, hi: int, n: int) -> np.ndarray:
        """int64 uniform over the closed range [lo, hi]."""
        return lo + np.floor(self.uniform(n) * (hi - lo + 1)).astype(np.int64)


def _exp2(x: np.ndarray) -> np.ndarray:
    """2**x from +,* only (monotone, < 0.2 % from the true value); deterministic everywhere."""
    k = np.floor(x)
    f = x - k
    p = 1.0 + f * (0.6951786 + f * (0.2261681 + f * 0.0786533))
    return p * np.power(2.0, k)  # power of two with an integral exponent is exact


def _log_uniform(rng: Rng, lo: float, hi: float, n: int) -> np.ndarray:
    octaves = math.log2(hi / lo)
    return lo * _exp2(rng.uniform(n) * octaves)


@dataclasses.dataclass
class Scene:
    """One scene in outline form; the layout handed to ``pf_scene_view``."""

    points: np.ndarray          # float32 [P, 2]
    flags: np.ndarray           # uint8  [P]   PointFlag
    contour_start: np.ndarray   # uint32 [C + 1] offsets into points
    path_start: np.ndarray      # uint32 [N + 1] offsets into contours
    fill_rule: np.ndarray       # uint8  [N]   0 nonzero (winding), 1 even-odd
    color: np.ndarray           # uint32 [N]   RGBA8, red in the low byte
    width: float
    height: float
    clear: int = 0              # RGBA8 clear colour, red in the low byte
    path_clip: Optional[np.ndarray] = None     # uint32 [N] clip path of each path, or NO_CLIP
    path_is_clip: Optional[np.ndarray] = None  # uint8 [N] 1 for clip paths (after the draw paths)
    path_stroke: Optional[np.ndarray] = None   # STROKE_DTYPE [N]: how each path is stroked
    contour_closed: Optional[np.ndarray] = None  # uint8 [C] Contour::closed (strokes only)
    dashes: Optional[np.ndarray] = None        # float32 [D] dash patterns of the strokes
    path_paint: Optional[np.ndarray] = None    # PAINT_DTYPE [N]: solid or gradient paint per path
    stops: Optional[np.ndarray] = None         # STOP_DTYPE [S] colour stops of the gradients
    view_box: Optional[np.ndarray] = None      # float32 [4] left, top, right, bottom (None: the canvas)
    load_action: int = 0                       # 0 clear to `clear`, 1 composite over the image there

    @property
    def n_paths(self) -> int:
        return int(self.fill_rule.shape[0])

    @property
    def n_points(self) -> int:
        return int(self.points.shape[0])

    @property
    def n_contours(self) -> int:
        return int(self.contour_start.shape[0] - 1)

    def nbytes(self) -> int:
        return int(self.points.nbytes + self.flags.nbytes + self.contour_start.nbytes
                   + self.path_start.nbytes + self.fill_rule.nbytes + self.color.nbytes)

    def subset(self, paths) -> "Scene":
        """A scene made of the given draw paths (in the given order)."""
        paths = np.asarray(paths, dtype=np.int64)
        cs, ps = self.contour_start.astype(np.int64), self.path_start.astype(np.int64)
        pts, fl, cstart, pstart = [], [], [0], [0]
        for p in paths:
            for c in range(ps[p], ps[p + 1]):
                pts.append(self.points[cs[c]:cs[c + 1]])
                fl.append(self.flags[cs[c]:cs[c + 1]])
                cstart.append(cstart[-1] + cs[c + 1] - cs[c])
            pstart.append(pstart[-1] + ps[p + 1] - ps[p])
        return Scene(
            points=np.concatenate(pts) if pts else np.zeros((0, 2), np.float32),
            flags=np.concatenate(fl) if fl else np.zeros(0, np.uint8),
            contour_start=np.asarray(cstart, np.uint32),
            path_start=np.asarray(pstart, np.uint32),
            fill_rule=self.fill_rule[paths].copy(),
            color=self.color[paths].copy(),
            width=self.width, height=self.height, clear=self.clear)


def pack_rgba(r, g, b, a) -> np.ndarray:
    r, g, b, a = (np.asarray(v, dtype=np.uint32) for v in (r, g, b, a))
    return r | (g << np.uint32(8)) | (b << np.uint32(16)) | (a << np.uint32(24))


def _assemble(contour_pts: List[np.ndarray], contour_flags: List[np.ndarray],
              contours_per_path: np.ndarray, fill_rule, color, width, height, clear=0) -> Scene:
    lens = np.array([len(c) for c in contour_pts], dtype=np.int64)
    cstart = np.zeros(len(lens) + 1, dtype=np.uint32)
    np.cumsum(lens, out=cstart[1:])
    pstart = np.zeros(len(contours_per_path) + 1, dtype=np.uint32)
    np.cumsum(contours_per_path, out=pstart[1:])
    return Scene(points=np.ascontiguousarray(np.concatenate(contour_pts).astype(np.float32)),
                 flags=np.concatenate(contour_flags).astype(np.uint8),
                 contour_start=cstart, path_start=pstart,
                 fill_rule=np.asarray(fill_rule, np.uint8), color=np.asarray(color, np.uint32),
                 width=float(width), height=float(height), clear=int(clear))


def _cubic_paths(rng: Rng, n_paths: int, box_lo: np.ndarray, box_size: np.ndarray,
                 seg_lo: int, seg_hi: int):
    """Closed single-contour paths of cubic segments, control points uniform in each box."""
    nseg = rng.integers(seg_lo, seg_hi, n_paths)
    npts = 1 + 3 * nseg
    total = int(npts.sum())
    owner = np.repeat(np.arange(n_paths), npts)
    uv = rng.uniform(2 * total).reshape(total, 2)
    pts = (box_lo[owner] + uv * box_size[owner][:, None]).astype(np.float32)
    start = np.zeros(n_paths + 1, np.int64)
    np.cumsum(npts, out=start[1:])
    local = np.arange(total) - start[owner]
    flags = np.where(local == 0, 0, np.array([0, 1, 2], np.uint8)[local % 3]).astype(np.uint8)
    return [pts[start[p]:start[p + 1]] for p in range(n_paths)], \
           [flags[start[p]:start[p + 1]] for p in range(n_paths)]


def plain_small(seed: int = 0, n_paths: int = 240, side: int = 1024, seg_lo: int = 8,
                seg_hi: int = 24) -> Scene:
    """240 closed cubic paths over a side x side canvas, nonzero, opaque solid colours."""
    rng = Rng(seed, 1)
    lo = np.zeros((n_paths, 2))
    size = np.full(n_paths, float(side))
    cpts, cfl = _cubic_paths(rng, n_paths, lo, size, seg_lo, seg_hi)
    rgb = rng.integers(0, 255, 3 * n_paths).reshape(n_paths, 3)
    color = pack_rgba(rgb[:, 0], rgb[:, 1], rgb[:, 2], np.full(n_paths, 255))
    return _assemble(cpts, cfl, np.ones(n_paths, np.int64), np.zeros(n_paths, np.uint8), color,
                     side, side)


def large_single(seed: int = 0, n_paths: int = 20000, side: int = 4096) -> Scene:
    """Log-uniform path boxes, 60/40 cubic/quadratic, alternating fill rule, 30 % translucent."""
    rng = Rng(seed, 2)
    s = _log_uniform(rng, 8.0, 2048.0, n_paths)
    origin = rng.uniform(2 * n_paths).reshape(n_paths, 2) * (side - s)[:, None]
    nseg = rng.integers(4, 64, n_paths)
    cpts, cfl = [], []
    for p in range(n_paths):
        k = int(nseg[p])
        cubic = rng.uniform(k) < 0.6
        per = np.where(cubic, 3, 2)
        total = 1 + int(per.sum())
        uv = rng.uniform(2 * total).reshape(total, 2)
        cpts.append((origin[p] + uv * s[p]).astype(np.float32))
        fl = [np.zeros(1, np.uint8)]
        for c in cubic:
            fl.append(np.array([1, 2, 0] if c else [1, 0], np.uint8))
        cfl.append(np.concatenate(fl))
    rgb = rng.integers(0, 255, 3 * n_paths).reshape(n_paths, 3)
    translucent = rng.uniform(n_paths) < 0.3
    alpha = np.where(translucent, np.floor(255.0 * (0.2 + 0.7 * rng.uniform(n_paths)) + 0.5), 255)
    color = pack_rgba(rgb[:, 0], rgb[:, 1], rgb[:, 2], alpha.astype(np.int64))
    fill_rule = (np.arange(n_paths) % 2).astype(np.uint8)
    return _assemble(cpts, cfl, np.ones(n_paths, np.int64), fill_rule, color, side, side)


def _unit_loop(u: np.ndarray):
    """Points on the unit circle from a rational quadrant parametrisation (u in [0,1))."""
    q = np.floor(4.0 * u)
    t = 4.0 * u - q
    den = 1.0 + t * t
    x, y = (1.0 - t * t) / den, (2.0 * t) / den
    for _ in range(3):
        rot = q >= 1.0
        x, y = np.where(rot, -y, x), np.where(rot, x, y)
        q = q - rot
    return x, y


def _glyph_loops(rng: Rng, cx, cy, radius, k, reverse):
    """Closed quadratic loops, one per entry: k[i] segments around (cx[i], cy[i])."""
    n = len(k)
    k = np.asarray(k, np.int64)
    first = np.zeros(n + 1, np.int64)
    np.cumsum(k, out=first[1:])
    total = int(first[-1])
    owner = np.repeat(np.arange(n), k)
    local = np.arange(total) - first[owner]
    u = (local + 0.5 * rng.uniform(total)) / k[owner]
    x, y = _unit_loop(u)
    r = radius[owner] * (0.85 + 0.3 * rng.uniform(total))
    on = np.stack([cx[owner] + x * r, cy[owner] + y * r], axis=1)
    # reversed loops walk their points backwards (holes)
    rev = reverse[owner]
    src = np.where(rev, first[owner] + (k[owner] - 1 - local), np.arange(total))
    on = on[src]
    nxt_idx = np.where(local + 1 < k[owner], np.arange(total) + 1, first[owner])
    nxt = on[nxt_idx]
    c = np.stack([cx[owner], cy[owner]], axis=1)
    d = 0.5 * (on + nxt) - c
    dl = np.sqrt((d * d).sum(axis=1))
    dl = np.where(dl > 1e-6, dl, 1.0)
    bulge = 1.0 + 0.15 * rng.uniform(total)
    ctrl = c + d * ((radius[owner] / dl) * bulge)[:, None]
    # each loop: on0 c0 on1 c1 ... on_{k-1} c_{k-1} on0   (2k + 1 points)
    npts = 2 * k + 1
    pfirst = np.zeros(n + 1, np.int64)
    np.cumsum(npts, out=pfirst[1:])
    pts = np.empty((int(pfirst[-1]), 2))
    flags = np.zeros(int(pfirst[-1]), np.uint8)
    base = pfirst[owner] + 2 * local
    pts[base] = on
    pts[base + 1] = ctrl
    flags[base + 1] = 1
    pts[pfirst[1:] - 1] = on[first[:-1]]
    return pts.astype(np.float32), flags, npts


def glyphs(seed: int = 0, n_paths: int = 150000, side: int = 2048) -> Scene:
    """Glyph-like quadratic outlines (1-3 contours, holes reversed), black on white."""
    rng = Rng(seed, 3)
    g = int(math.ceil(math.sqrt(n_paths)))
    cell = side / g
    idx = np.arange(n_paths)
    jit = rng.uniform(2 * n_paths).reshape(n_paths, 2)
    centers = (np.stack([idx % g, idx // g], axis=1) + 0.25 + 0.5 * jit) * cell
    R = 0.5 * (12.0 + 36.0 * rng.uniform(n_paths))
    ncont = rng.integers(1, 3, n_paths)
    total = rng.integers(10, 40, n_paths)
    inner = np.where(ncont > 1, np.maximum(3, total // (2 * ncont)), 0)
    outer = np.maximum(4, total - inner * (ncont - 1))
    # contour table: outer contour of each path, then its inner ones
    owner = np.repeat(idx, ncont)
    cfirst = np.zeros(n_paths + 1, np.int64)
    np.cumsum(ncont, out=cfirst[1:])
    is_inner = (np.arange(len(owner)) - cfirst[owner]) > 0
    off = (rng.uniform(2 * len(owner)).reshape(-1, 2) - 0.5) * 0.6 * R[owner][:, None]
    rr = R[owner] * np.where(is_inner, 0.15 + 0.15 * rng.uniform(len(owner)), 1.0)
    cx = centers[owner, 0] + np.where(is_inner, off[:, 0], 0.0)
    cy = centers[owner, 1] + np.where(is_inner, off[:, 1], 0.0)
    k = np.where(is_inner, inner[owner], outer[owner])
    pts, flags, npts = _glyph_loops(rng, cx, cy, rr, k, is_inner)
    cstart = np.zeros(len(owner) + 1, np.uint32)
    np.cumsum(npts, out=cstart[1:])
    pstart = cfirst.astype(np.uint32)
    color = pack_rgba(0, 0, 0, np.full(n_paths, 255))
    return Scene(points=pts, flags=flags, contour_start=cstart, path_start=pstart,
                 fill_rule=np.zeros(n_paths, np.uint8), color=color, width=float(side),
                 height=float(side), clear=int(pack_rgba(255, 255, 255, 255)))


def batched(n_scenes: int = 512, first_seed: int = 1000, lo_paths: int = 16,
            hi_paths: int = 4096, sides=(256, 512, 1024, 2048)) -> List[Scene]:
    """Independent scenes: log-uniform path count, canvas side drawn from ``sides``."""
    out = []
    for i in range(n_scenes):
        rng = Rng(first_seed + i, 4)
        n = int(np.floor(_log_uniform(rng, float(lo_paths), float(hi_paths), 1))[0])
        side = int(sides[int(rng.integers(0, len(sides) - 1, 1)[0])])
        out.append(plain_small(seed=first_seed + i, n_paths=n, side=side))
    return out


def concat(parts: List[Scene], width: float, height: float, clear: int = 0) -> Scene:
    """Draw the paths of several scenes, in order, on one canvas."""
    pts, fl, cs, ps, fr, col = [], [], [np.zeros(1, np.uint32)], [np.zeros(1, np.uint32)], [], []
    pbase = cbase = 0
    for s in parts:
        pts.append(s.points)
        fl.append(s.flags)
        cs.append(s.contour_start[1:] + np.uint32(pbase))
        ps.append(s.path_start[1:] + np.uint32(cbase))
        fr.append(s.fill_rule)
        col.append(s.color)
        pbase += s.n_points
        cbase += s.n_contours
    return Scene(points=np.concatenate(pts), flags=np.concatenate(fl),
                 contour_start=np.concatenate(cs), path_start=np.concatenate(ps),
                 fill_rule=np.concatenate(fr), color=np.concatenate(col),
                 width=float(width), height=float(height), clear=int(clear))


NO_CLIP = 0xFFFFFFFF


def with_clips(draw: Scene, clips: Scene, assign: np.ndarray) -> Scene:
    """`draw`'s paths followed by `clips`'s paths as clip paths; draw path i is clipped by
    clip path assign[i] (an index into `clips`, or -1 for none)."""
    out = concat([draw, clips], draw.width, draw.height, draw.clear)
    n_draw, n_clip = draw.n_paths, clips.n_paths
    pc = np.full(n_draw + n_clip, NO_CLIP, np.uint32)
    a = np.asarray(assign, np.int64)
    pc[:n_draw] = np.where(a >= 0, a + n_draw, NO_CLIP).astype(np.uint32)
    out.path_clip = pc
    out.path_is_clip = np.concatenate([np.zeros(n_draw, np.uint8), np.ones(n_clip, np.uint8)])
    return out


def clipped(seed: int = 0, n_paths: int = 240, side: int = 1024, n_clips: int = 8,
            clip_share: float = 0.6) -> Scene:
    """The 240-path cubic scene with clip paths: n_clips closed cubic shapes, each a quarter to
    a whole of the canvas wide, alternately nonzero and even-odd; each draw path is clipped by a
    random one with probability clip_share; 30 % of the draw paths translucent."""
    rng = Rng(seed, 6)
    draw = plain_small(seed=seed, n_paths=n_paths, side=side)
    alpha = np.where(rng.uniform(n_paths) < 0.3, (rng.uniform(n_paths) * 180 + 40).astype(np.uint32), 255)
    draw.color = (draw.color & np.uint32(0x00FFFFFF)) | (alpha.astype(np.uint32) << np.uint32(24))
    size = side * (0.25 + 0.75 * rng.uniform(n_clips))
    lo = rng.uniform(2 * n_clips).reshape(n_clips, 2) * (side - size)[:, None]
    cpts, cfl = _cubic_paths(rng, n_clips, lo, np.asarray(size, np.float64), 3, 8)
    clips = _assemble(cpts, cfl, np.ones(n_clips, np.int64), (np.arange(n_clips) % 2).astype(np.uint8),
                      np.full(n_clips, 0xFFFFFFFF, np.uint32), side, side)
    assign = np.where(rng.uniform(n_paths) < clip_share, rng.integers(0, n_clips - 1, n_paths), -1)
    return with_clips(draw, clips, assign)


def add_clips(draw: Scene, seed: int, n_clips: int = 8, clip_share: float = 0.6) -> Scene:
    """`draw` with n_clips clip paths appended: closed cubic shapes a quarter to a whole of the
    canvas wide, alternately nonzero and even-odd; each draw path is clipped by a random one
    with probability clip_share."""
    rng = Rng(seed, 7)
    side = float(min(draw.width, draw.height))
    size = side * (0.25 + 0.75 * rng.uniform(n_clips))
    lo = rng.uniform(2 * n_clips).reshape(n_clips, 2) * (side - size)[:, None]
    cpts, cfl = _cubic_paths(rng, n_clips, lo, np.asarray(size, np.float64), 3, 8)
    clips = _assemble(cpts, cfl, np.ones(n_clips, np.int64), (np.arange(n_clips) % 2).astype(np.uint8),
                      np.full(n_clips, 0xFFFFFFFF, np.uint32), draw.width, draw.height)
    n = draw.n_paths
    assign = np.where(rng.uniform(n) < clip_share, rng.integers(0, n_clips - 1, n), -1)
    return with_clips(draw, clips, assign)


def batched_clipped(n_scenes: int = 512, first_seed: int = 1000, n_clips: int = 8, clip_share: float = 0.6,
                    **kw) -> List[Scene]:
    """The batched scenes, each with n_clips clip paths (add_clips, seeded by the scene's seed)."""
    return [add_clips(sc, first_seed + i, n_clips, clip_share)
            for i, sc in enumerate(batched(n_scenes=n_scenes, first_seed=first_seed, **kw))]


def stroked(seed: int = 0, n_paths: int = 200, side: int = 1024, dash_share: float = 0.3,
            fill_share: float = 0.0) -> Scene:
    """Stroked paths (Canvas::stroke_path): 1-3 contours each, a random walk of 1-12 segments
    (lines, quadratic and cubic curves, points uniform in a log-uniform 16 px-to-canvas box),
    40 % of the contours closed; line width log-uniform 0.5-24 px; caps, joins and miter limits
    (1-12) uniform; dash_share of the paths dashed with a 2- or 4-entry pattern of 1-40 px (a
    third of them with a phase); fill_share of the paths filled instead.  Colours translucent
    (40 %) or opaque, nonzero rule."""
    rng = Rng(seed, 8)
    n = n_paths
    n_contours = rng.integers(1, 3, n)
    width = _log_uniform(rng, 0.5, 24.0, n)
    caps = rng.integers(0, 2, n)
    joins = rng.integers(0, 2, n)
    miter = 1.0 + 11.0 * rng.uniform(n)
    dashed = rng.uniform(n) < dash_share
    filled = rng.uniform(n) < fill_share
    box = _log_uniform(rng, 16.0, float(side), n)
    origin = rng.uniform(2 * n).reshape(n, 2) * (side - box)[:, None]
    k_path = np.repeat(np.arange(n), n_contours)                  # path of each contour
    nk = len(k_path)
    nseg = rng.integers(1, 12, nk)
    kinds = rng.integers(0, 2, int(nseg.sum()))                   # 0 line, 1 quadratic, 2 cubic
    seg_contour = np.repeat(np.arange(nk), nseg)
    per_contour = 1 + np.bincount(seg_contour, weights=kinds + 1, minlength=nk).astype(np.int64)
    cstart = np.zeros(nk + 1, np.int64)
    np.cumsum(per_contour, out=cstart[1:])
    n_pts = int(cstart[-1])
    flags = np.zeros(n_pts, np.uint8)
    # segment s starts after its contour's first point and the points of the segments before it
    seg_first = np.zeros(len(kinds), np.int64)
    np.cumsum(kinds + 1, out=seg_first)
    seg_first -= kinds + 1
    contour_seg0 = np.zeros(nk + 1, np.int64)
    np.cumsum(nseg, out=contour_seg0[1:])
    before = seg_first - np.repeat(np.concatenate([[0], np.cumsum(kinds + 1)])[contour_seg0[:-1]], nseg)
    p0 = cstart[seg_contour] + 1 + before                          # first point after the segment start
    flags[p0[kinds >= 1]] = 1
    flags[p0[kinds == 2] + 1] = 2
    u = rng.uniform(2 * n_pts).reshape(n_pts, 2)
    pt_path = np.repeat(k_path, per_contour)
    pts = origin[pt_path] + u * box[pt_path][:, None]
    closed = (rng.uniform(nk) < 0.4).astype(np.uint8)
    pstart = np.zeros(n + 1, np.int64)
    np.cumsum(n_contours, out=pstart[1:])
    st = np.zeros(n, STROKE_DTYPE)
    st["line_width"] = np.where(filled, 0.0, width)
    st["miter_limit"] = miter
    st["line_cap"] = caps
    st["line_join"] = joins
    use = dashed & ~filled
    m = np.where(rng.uniform(n) < 0.5, 2, 4) * use
    first = np.zeros(n + 1, np.int64)
    np.cumsum(m, out=first[1:])
    pat = 1.0 + 39.0 * rng.uniform(int(first[-1]))
    totals = np.add.reduceat(pat, first[:-1][use]) if use.any() else np.zeros(0)
    phase = np.where(rng.uniform(n) < 0.33, rng.uniform(n), 0.0)
    st["dash_first"] = first[:-1]
    st["dash_count"] = m
    offs = np.zeros(n)
    offs[use] = phase[use] * totals
    st["dash_offset"] = offs
    rgb = rng.integers(0, 0xFFFFFF, n).astype(np.uint32)
    alpha = np.where(rng.uniform(n) < 0.4, (rng.uniform(n) * 180 + 60).astype(np.uint32), 255)
    sc = Scene(points=pts.astype(np.float32), flags=flags, contour_start=cstart.astype(np.uint32),
               path_start=pstart.astype(np.uint32), fill_rule=np.zeros(n, np.uint8),
               color=rgb | (alpha.astype(np.uint32) << np.uint32(24)), width=float(side), height=float(side))
    sc.path_stroke = st
    sc.contour_closed = closed
    sc.dashes = np.asarray(pat if len(pat) else [1.0], np.float32)
    return sc


def batched_stroked(n_scenes: int = 512, first_seed: int = 1000, lo_paths: int = 16, hi_paths: int = 4096,
                    sides=(256, 512, 1024, 2048), dash_share: float = 0.3) -> List[Scene]:
    """The batched layout (log-uniform path counts, canvas sides) with stroked scenes."""
    out = []
    for i in range(n_scenes):
        rng = Rng(first_seed + i, 4)
        n = int(np.floor(_log_uniform(rng, float(lo_paths), float(hi_paths), 1))[0])
        side = int(sides[int(rng.integers(0, len(sides) - 1, 1)[0])])
        out.append(stroked(seed=first_seed + i, n_paths=n, side=side, dash_share=dash_share))
    return out


def with_gradients(sc: Scene, seed: int, share: float = 0.5) -> Scene:
    """`sc` with a share of its paths painted with gradients (Paint::from_gradient): half
    linear, half radial (two circles, a quarter of them under a rotation and scale), 2-5 stops
    (unsorted, sometimes repeated offsets, 40 % of the gradients with translucent stops), 30 %
    repeating.  Geometry is drawn around each path's bounding box."""
    rng = Rng(seed, 9)
    n = sc.n_paths
    pts = sc.points.astype(np.float64)
    cs, ps = sc.contour_start.astype(np.int64), sc.path_start.astype(np.int64)
    pt_first, pt_end = cs[ps[:-1]], cs[ps[1:]]
    grad = rng.uniform(n) < share
    kind = np.where(rng.uniform(n) < 0.5, PAINT_LINEAR, PAINT_RADIAL)
    wrap = np.where(rng.uniform(n) < 0.3, WRAP_REPEAT, WRAP_CLAMP)
    nstops = rng.integers(2, 5, n)
    translucent = rng.uniform(n) < 0.4
    paint = np.zeros(n, PAINT_DTYPE)
    paint["transform"] = [1, 0, 0, 1, 0, 0]
    stops = []
    u = rng.uniform(8 * n).reshape(n, 8)
    for p in range(n):
        if not grad[p] or pt_end[p] == pt_first[p]:
            continue
        q = pts[pt_first[p]:pt_end[p]]
        lo, hi = q.min(axis=0), q.max(axis=0)
        size = np.maximum(hi - lo, 1.0)
        a = lo + u[p, 0:2] * size
        b = lo + u[p, 2:4] * size
        paint[p]["type"] = kind[p]
        paint[p]["wrap"] = wrap[p]
        paint[p]["stop_first"] = len(stops)
        paint[p]["stop_count"] = nstops[p]
        paint[p]["line"] = [a[0], a[1], b[0], b[1]]
        if kind[p] == PAINT_RADIAL:
            r1 = 0.1 * size.max() + u[p, 4] * size.max()
            paint[p]["radii"] = [u[p, 5] * 0.3 * r1, r1]
            if u[p, 6] < 0.25:  # a rotation and scale about the first centre
                c, s_ = 0.8 + 0.4 * u[p, 7], 0.5 * u[p, 6]
                paint[p]["transform"] = [c, s_, -s_, c, a[0] - c * a[0] + s_ * a[1], a[1] - s_ * a[0] - c * a[1]]
        offs = rng.uniform(int(nstops[p]))
        if nstops[p] > 2 and u[p, 7] < 0.2:
            offs[1] = offs[0]
        cols = rng.integers(0, 0xFFFFFF, int(nstops[p])).astype(np.uint32)
        alpha = np.where(translucent[p] & (rng.uniform(int(nstops[p])) < 0.6),
                         (rng.uniform(int(nstops[p])) * 200 + 30).astype(np.uint32), 255)
        for o_, c_, a_ in zip(offs, cols, alpha):
            stops.append((o_, int(c_) | (int(a_) << 24)))
    out = dataclasses.replace(sc)
    out.path_paint = paint
    out.stops = np.asarray(stops if stops else [(0.0, 0)], STOP_DTYPE)
    return out


def gradient_scene(seed: int = 0, n_paths: int = 240, side: int = 1024, share: float = 0.6) -> Scene:
    """Large paths (scenes.large_single's families) with gradient paints."""
    return with_gradients(large_single(seed=seed, n_paths=n_paths, side=side), seed, share)


def batched_gradients(n_scenes: int = 512, first_seed: int = 1000, share: float = 0.5, **kw) -> List[Scene]:
    """The batched scenes with gradient paints on a share of the paths."""
    return [with_gradients(sc, first_seed + i, share)
            for i, sc in enumerate(batched(n_scenes=n_scenes, first_seed=first_seed, **kw))]


def mixed(seed: int = 7, n_paths: int = 8192, side: int = 4096) -> Scene:
    """A mixture of the three path families on one canvas (held-out evaluation scene)."""
    rng = Rng(seed, 5)
    n_a = n_paths // 8
    n_b = (n_paths * 3) // 8
    n_c = n_paths - n_a - n_b
    a = plain_small(seed=seed * 31 + 1, n_paths=n_a, side=side)
    # shrink the canvas-wide cubic paths into random sub-boxes so they stay varied
    s_box = _log_uniform(rng, 64.0, float(side), n_a)
    o_box = rng.uniform(2 * n_a).reshape(n_a, 2) * (side - s_box)[:, None]
    cs, ps = a.contour_start.astype(np.int64), a.path_start.astype(np.int64)
    pts = a.points.astype(np.float64)
    for p in range(n_a):
        lo, hi = cs[ps[p]], cs[ps[p + 1]]
        pts[lo:hi] = o_box[p] + pts[lo:hi] * (s_box[p] / side)
    a.points = pts.astype(np.float32)
    b = large_single(seed=seed * 31 + 2, n_paths=n_b, side=side)
    c = glyphs(seed=seed * 31 + 3, n_paths=n_c, side=side)
    out = concat([a, b, c], side, side)
    order = np.argsort(rng.uniform(n_paths), kind="stable")
    return out.subset(order)


CONFIGS = {
    "plain_small": plain_small,
    "large_single": large_single,
    "glyphs": glyphs,
    "mixed": mixed,
}
