"""Empty and ragged inputs: scenes without paths, a one-pixel canvas, paths of a single line,
alone and inside batches, through the exact frame, the learned frame (plain and replayed from its
graph) and the default frame.

Every scene's integer tile data must equal the oracle's bit for bit and equal the same scene
rendered alone; its pixels must be within one RGBA8 code of the FP64 oracle (a scene without
paths is its clear colour exactly).
"""
import numpy as np
import pytest

import scenes as S
from conftest import TILE_KEYS

pytestmark = pytest.mark.gpu

LIST_KEYS = ["fb_tiles", "z", "fb_list_first", "fb_list"]
CANON = TILE_KEYS + LIST_KEYS
PIXEL_TOL = 1  # RGBA8 codes


def empty(width=64.0, height=48.0, clear=0x80402010):
    return S.Scene(points=np.zeros((0, 2), np.float32), flags=np.zeros(0, np.uint8),
                   contour_start=np.zeros(1, np.uint32), path_start=np.zeros(1, np.uint32),
                   fill_rule=np.zeros(0, np.uint8), color=np.zeros(0, np.uint32), width=width, height=height,
                   clear=clear)


def lines(segments, width, height, clear=0xff000000):
    """One closed path per list of points (lines only), opaque colours."""
    pts, fl, cs, ps = [], [], [0], [0]
    for k, poly in enumerate(segments):
        p = np.asarray(poly, np.float32).reshape(-1, 2)
        pts.append(p)
        fl.append(np.zeros(len(p), np.uint8))
        cs.append(cs[-1] + len(p))
        ps.append(k + 1)
    n = len(segments)
    return S.Scene(points=np.concatenate(pts), flags=np.concatenate(fl), contour_start=np.asarray(cs, np.uint32),
                   path_start=np.asarray(ps, np.uint32), fill_rule=np.zeros(n, np.uint8),
                   color=np.asarray([0xff0000ff + 0x00100000 * k for k in range(n)], np.uint32),
                   width=float(width), height=float(height), clear=clear)


def ragged_scenes():
    return [
        empty(),
        S.plain_small(seed=11, n_paths=24, side=256),
        empty(width=1.0, height=1.0, clear=0xffffffff),
        lines([[(0.25, 0.25), (0.75, 0.5)]], 1, 1),                    # a one-pixel canvas, one sliver
        lines([[(3.0, 5.0), (40.0, 5.0)]], 50, 20),                    # a zero-area closed path
        lines([[(2.0, 2.0), (30.0, 9.0), (7.0, 29.0)], [(31.5, 0.0), (31.5, 31.5), (0.0, 31.5)]], 32, 32),
        empty(width=2048.0, height=16.0),
        S.plain_small(seed=12, n_paths=1, side=64, seg_lo=1, seg_hi=2),
    ]


def _check_against_oracle(oracle_mod, got, img, sc):
    tiled = {}
    want_img, _ = oracle_mod.render(sc, oracle_mod.Z_D3D11, tiled=tiled)
    for k in CANON:
        assert got[k].shape == tiled[k].shape and np.array_equal(got[k], tiled[k]), k
    d = np.abs(img.astype(np.int16) - want_img.astype(np.int16))
    assert int(d.max()) <= PIXEL_TOL
    if sc.n_paths == 0:
        assert np.array_equal(img, want_img)


def test_empty_scene_alone_every_frame(pf, oracle_mod):
    sc = empty()
    with pf.Renderer() as r:
        r.sizer_load()
        r.upload(sc)
        for frame in (r.render, r.render_learned, r.render_learned, r.render_learned, r.render_auto):
            st = frame()
            assert st["paths"] == 0 and st["fills"] == 0 and st["tiles"] == 0
            _check_against_oracle(oracle_mod, r.canon(), r.image(), sc)


def test_batch_of_only_empty_scenes(pf):
    scs = [empty(), empty(width=300.0, height=17.0, clear=0xff00ff00), empty(width=1.0, height=1.0)]
    with pf.Renderer() as r:
        r.sizer_load()
        r.upload(scs)
        for frame in (r.render, r.render_learned, r.render_learned, r.render_learned):
            st = frame()
            assert st["paths"] == 0 and st["fills"] == 0
            for i, sc in enumerate(scs):
                img = r.image(i)
                assert img.shape == (int(np.ceil(sc.height)), int(np.ceil(sc.width)), 4)
                want = np.frombuffer(np.uint32(sc.clear).tobytes(), np.uint8)
                assert (img.reshape(-1, 4) == want).all()


def test_ragged_batch_equals_scenes_alone_and_oracle(pf, oracle_mod):
    scs = ragged_scenes()
    with pf.Renderer() as frame, pf.Renderer() as alone:
        frame.sizer_load()
        frame.upload(scs)
        runs = [("exact", frame.render), ("learned", frame.render_learned), ("learned", frame.render_learned),
                ("replay", frame.render_learned)]
        for name, run in runs:
            run()
            for i, sc in enumerate(scs):
                got, img = frame.canon(i), frame.image(i)
                alone.upload(sc)
                alone.render()
                one = alone.canon()
                for k in CANON:
                    assert np.array_equal(got[k], one[k]), (name, i, k)
                assert np.array_equal(img, alone.image()), (name, i)
                _check_against_oracle(oracle_mod, got, img, sc)


def test_sub_ranges_of_a_ragged_batch(pf, oracle_mod):
    scs = ragged_scenes()
    with pf.Renderer() as r:
        r.upload(scs)
        for first, count in ((0, 1), (2, 3), (6, 2), (1, 7)):
            r.render(first, count)
            for i in range(first, first + count):
                _check_against_oracle(oracle_mod, r.canon(i), r.image(i), scs[i])
