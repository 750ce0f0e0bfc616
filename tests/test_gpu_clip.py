"""Clip paths on the GPU against the oracle.

A clipped draw tile follows Tiler::prepare_tiles (pathfinder/core/d3d9/tiler.cpp:386-431):
culled outside the clip path's tile rect or over a blank clip tile; a solid tile over a clip
alpha tile is drawn with the clip's mask; two alpha tiles are drawn with their masks combined
as tile_clip_combine.frag does (min of |mask + backdrop|).  Tile data (with the clip
assignments) must be bit-exact, pixels within one code of the FP64 oracle.  The golden clip
fixtures go through the generic golden tests; these cover larger scenes, batches mixing
clipped and unclipped scenes, the learned frame and the layout checks.
"""
import numpy as np
import pytest

import scenes as S
from conftest import TILE_KEYS

pytestmark = pytest.mark.gpu

LIST_KEYS = ["fb_tiles", "z", "fb_list_first", "fb_list"]
PIXEL_TOL = 1


def _check(got, want, keys):
    for k in keys:
        assert got[k].shape == want[k].shape, (k, got[k].shape, want[k].shape)
        assert np.array_equal(got[k], want[k]), k


@pytest.mark.parametrize("seed,n_paths,side,n_clips", [(41, 240, 1024, 8), (42, 1500, 2048, 24),
                                                        (43, 600, 512, 3)])
def test_clipped_scene_bit_exact_and_pixels(renderer, oracle_mod, seed, n_paths, side, n_clips):
    sc = S.clipped(seed=seed, n_paths=n_paths, side=side, n_clips=n_clips)
    renderer.upload(sc)
    renderer.render()
    got, img = renderer.canon(), renderer.image()
    want = oracle_mod.tile_scene(sc, oracle_mod.Z_D3D11, threads=8)
    _check(got, want, TILE_KEYS + LIST_KEYS)
    modes = np.bincount(got["tile_mask"], minlength=3)
    assert modes[1] > 0 and modes[2] > 0, modes  # both clip modes are exercised
    ref, _ = oracle_mod.render(sc, threads=16)
    diff = np.abs(img.astype(np.int32) - ref.astype(np.int32))
    print(f"clipped s{seed}: modes {modes.tolist()}, pixel max err {diff.max()} mean {diff.mean():.2e}")
    assert diff.max() <= PIXEL_TOL


def test_batch_mixing_clipped_and_plain_scenes(renderer, oracle_mod):
    scs = [S.clipped(seed=51, n_paths=300, side=512), S.plain_small(seed=52, n_paths=200, side=512),
           S.clipped(seed=53, n_paths=500, side=1024, n_clips=5)]
    renderer.upload(scs)
    renderer.render()
    batch = [(renderer.canon(i), renderer.image(i)) for i in range(len(scs))]
    for i, sc in enumerate(scs):
        want = oracle_mod.tile_scene(sc, oracle_mod.Z_D3D11, threads=8)
        _check(batch[i][0], want, TILE_KEYS + LIST_KEYS)
        renderer.upload(sc)
        renderer.render()
        assert np.array_equal(renderer.image(), batch[i][1])


def test_learned_frame_with_clips_equals_exact(pf):
    scs = [S.clipped(seed=61 + i, n_paths=200 + 150 * i, side=1024) for i in range(4)]
    with pf.Renderer(device=0) as r:
        r.upload(scs)
        r.sizer_load()
        r.render()
        exact = [(r.canon(i), r.image(i)) for i in range(len(scs))]
        for _ in range(3):  # plain learned frame, capture, replay
            st = r.render_learned()
            assert st["overflow"] == 0
            for i in range(len(scs)):
                _check(r.canon(i), exact[i][0], TILE_KEYS + LIST_KEYS)
                assert np.array_equal(r.image(i), exact[i][1])


def test_invalid_clip_layouts_are_rejected(renderer, pf):
    sc = S.clipped(seed=71, n_paths=20, side=256, n_clips=2)
    n = len(sc.fill_rule)
    cases = []
    # a draw path after a clip path
    order = np.r_[np.arange(n - 3), n - 2, n - 3, n - 1]
    bad = sc.subset(order)
    bad.path_clip = sc.path_clip[order].copy()
    bad.path_is_clip = sc.path_is_clip[order].copy()
    cases.append(bad)
    # a clipped clip path
    b2 = S.Scene(**{**sc.__dict__, "path_clip": sc.path_clip.copy()})
    b2.path_clip[n - 1] = n - 2
    cases.append(b2)
    # a draw path naming a draw path, or out of range
    for target in (0, n + 5):
        b3 = S.Scene(**{**sc.__dict__, "path_clip": sc.path_clip.copy()})
        b3.path_clip[1] = target
        cases.append(b3)
    # only one of the two arrays
    cases.append(S.Scene(**{**sc.__dict__, "path_is_clip": None}))
    for bad in cases:
        with pytest.raises(pf.PfError) as e:
            renderer.upload(bad)
        assert e.value.status == 1
    renderer.upload(sc)  # the context stays usable
    renderer.render()
