"""The reference-facing semantics of the boundary: view boxes and the destination load action.

* A view box (Scene::set_view_box, pathfinder/core/scene.cpp:169-176) clips and tiles every path
  against its rect (core/d3d9/tiler.cpp:141-153, 317-335); the golden view-box fixtures pin the
  tiles against the reference itself (test_gpu_parity.py runs every fixture), and here batches
  of view-box scenes equal the scenes rendered alone.
* LOAD_ACTION_LOAD (Renderer::draw with clear_dst_texture = false, core/d3d11/renderer.cpp:376-380;
  tile.comp:744-757): the frame composites over the destination already there.  Pixels must be
  within one RGBA8 code of the FP64 oracle composited over the same destination.
"""
import dataclasses

import numpy as np
import pytest

import scenes as S
from conftest import TILE_KEYS, load_golden

pytestmark = pytest.mark.gpu

LIST_KEYS = ["fb_tiles", "z", "fb_list_first", "fb_list"]
PIXEL_TOL = 1


def _err(a, b):
    return int(np.abs(a.astype(np.int16) - b.astype(np.int16)).max())


def _translucent(sc, seed):
    rng = np.random.default_rng(seed)
    alpha = rng.integers(40, 230, sc.n_paths).astype(np.uint32)
    return dataclasses.replace(sc, color=(sc.color & np.uint32(0x00ffffff)) | (alpha << np.uint32(24)))


def test_load_composites_over_the_destination(pf, oracle_mod):
    sc = _translucent(S.plain_small(seed=21, n_paths=80, side=512), 3)
    sc.load_action = 1
    dest = np.random.default_rng(4).integers(0, 256, (512, 512, 4), dtype=np.uint8)
    with pf.Renderer() as r:
        r.upload(sc)
        r.write_image(0, dest)
        r.render()
        got = r.image()
        want, _ = oracle_mod.render(sc, threads=8, dest=dest)
        assert _err(got, want) <= PIXEL_TOL
        # a second LOAD frame composites over the first one's output
        r.render()
        again = r.image()
        want2, _ = oracle_mod.render(sc, threads=8, dest=got)
        assert _err(again, want2) <= PIXEL_TOL
        assert not np.array_equal(again, got)


def test_load_untouched_where_nothing_is_drawn(pf):
    # one small square: every other framebuffer tile keeps the destination exactly
    pts = np.array([[40, 40], [70, 40], [70, 70], [40, 70]], np.float32)
    sc = S.Scene(points=pts, flags=np.zeros(4, np.uint8), contour_start=np.array([0, 4], np.uint32),
                 path_start=np.array([0, 1], np.uint32), fill_rule=np.zeros(1, np.uint8),
                 color=np.array([0x80ff0000], np.uint32), width=200.0, height=150.0, clear=0xff00ff00,
                 load_action=1)
    dest = np.random.default_rng(8).integers(0, 256, (150, 200, 4), dtype=np.uint8)
    with pf.Renderer() as r:
        r.upload(sc)
        r.write_image(0, dest)
        r.render()
        got = r.image()
    mask = np.ones((150, 200), bool)
    mask[32:80, 32:80] = False  # the framebuffer tiles the square touches
    assert np.array_equal(got[mask], dest[mask])
    assert not np.array_equal(got[~mask], dest[~mask])


def test_learned_frame_and_replay_with_load(pf, oracle_mod):
    sc = _translucent(S.plain_small(seed=22, n_paths=120, side=1024), 5)
    sc.load_action = 1
    dest = np.random.default_rng(6).integers(0, 256, (1024, 1024, 4), dtype=np.uint8)
    with pf.Renderer() as r:
        r.sizer_load(pf.DEFAULT_WEIGHTS)
        r.upload(sc)
        prev = dest
        r.write_image(0, dest)
        for k in range(3):  # a plain learned frame, then graph replays
            st = r.render_learned()
            got = r.image()
            want, _ = oracle_mod.render(sc, threads=8, dest=prev)
            assert _err(got, want) <= PIXEL_TOL, k
            prev = got
        assert st["host_syncs"] == 1  # the last one was a replay


def test_batch_mixing_view_boxes_and_load_equals_alone(pf):
    inner, _ = load_golden("view_box_inner")
    outside, _ = load_golden("view_box_outside")
    clipped, _ = load_golden("view_box_clipped")
    plain = _translucent(S.plain_small(seed=23, n_paths=60, side=384), 9)
    plain.load_action = 1
    scs = [inner, plain, outside, clipped]
    rng = np.random.default_rng(2)
    dests = [rng.integers(0, 256, (int(np.ceil(s.height)), int(np.ceil(s.width)), 4), dtype=np.uint8) for s in scs]
    with pf.Renderer() as r:
        r.upload(scs)
        for i, d in enumerate(dests):
            r.write_image(i, d)
        r.render()
        batch = [(r.canon(i), r.image(i)) for i in range(len(scs))]
        for i, sc in enumerate(scs):
            r.upload(sc)
            r.write_image(0, dests[i])
            r.render()
            one = r.canon()
            for k in TILE_KEYS + LIST_KEYS:
                assert np.array_equal(batch[i][0][k], one[k]), (i, k)
            assert np.array_equal(batch[i][1], r.image()), i


def test_view_box_pixels_outside_the_box_are_clear(pf, oracle_mod):
    sc, _ = load_golden("view_box_inner")
    sc = dataclasses.replace(sc, clear=0xff204060)
    with pf.Renderer() as r:
        img = r.draw(sc)
    want, _ = oracle_mod.render(sc, threads=8)
    assert _err(img, want) <= PIXEL_TOL
    # nothing is drawn left of the box's first tile column or above its first tile row
    assert np.all(img[:, :32].reshape(-1, 4) == [0x60, 0x40, 0x20, 0xff])
    assert np.all(img[:16].reshape(-1, 4) == [0x60, 0x40, 0x20, 0xff])


def test_boundary_arguments_are_checked(pf):
    sc = S.plain_small(seed=1, n_paths=4, side=64)
    with pf.Renderer() as r:
        for box in ([10, 0, 5, 64], [0, 0, 64, np.inf], [0, 0, 1e6, 64]):
            with pytest.raises(pf.PfError) as e:
                r.upload(dataclasses.replace(sc, view_box=np.asarray(box, np.float32)))
            assert e.value.status == 1
        with pytest.raises(pf.PfError):
            r.upload(dataclasses.replace(sc, load_action=2))
        r.upload(sc)
        with pytest.raises(ValueError):
            r.write_image(0, np.zeros((10, 10, 4), np.uint8))
        bad = r.lib.pf_write_image(r.ctx, 0, None, 64 * 64 * 4)
        assert bad == 1
