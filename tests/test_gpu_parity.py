"""CUDA pipeline against the reference's tiler (golden fixtures) and the oracle.

Integer tile data (tile rects, alpha flags, propagated int8 backdrops, fills,
column sums) must be bit-exact; composite lists and z follow the d3d11 z rule;
RGBA8 pixels must be within 1/255 (one code) of the FP64 analytic-area oracle
and alpha-tile coverage within 1/255 of it.
"""
import json
import os

import numpy as np
import pytest

import scenes as S
from conftest import TILE_KEYS, golden_names, load_golden

pytestmark = pytest.mark.gpu

LIST_KEYS = ["fb_tiles", "z", "fb_list_first", "fb_list"]
PIXEL_TOL = 1          # RGBA8 codes
COVERAGE_TOL = 1.0 / 255.0


def render(renderer, sc):
    renderer.upload(sc)
    stats = renderer.render()
    return stats, renderer.canon(), renderer.image()


def assert_canon(got, want, keys):
    for k in keys:
        assert got[k].shape == want[k].shape, (k, got[k].shape, want[k].shape)
        assert np.array_equal(got[k], want[k]), k


@pytest.mark.parametrize("name", golden_names())
def test_tile_data_bit_exact_vs_reference(renderer, oracle_mod, name):
    sc, ref = load_golden(name)
    _, got, img = render(renderer, sc)
    assert_canon(got, ref, TILE_KEYS)
    assert_canon(got, oracle_mod.tile_scene(sc, oracle_mod.Z_D3D11), LIST_KEYS)


@pytest.mark.parametrize("name", golden_names())
def test_pixels_within_one_code_of_fp64_oracle(renderer, oracle_mod, name):
    sc, _ = load_golden(name)
    if sc.path_paint is not None:
        pytest.skip("gradient fixtures have their own pixel rule (test_gpu_gradient.py)")
    _, _, img = render(renderer, sc)
    want, _ = oracle_mod.render(sc, threads=8)
    diff = np.abs(img.astype(np.int32) - want.astype(np.int32))
    assert diff.max() <= PIXEL_TOL, (diff.max(), diff.mean())


@pytest.mark.parametrize("name", ["gen_plain_small_s1", "gen_large_mixed_s2", "gen_glyphs_s3", "int8_wrap",
                                  "star_even_odd", "half_pixel_rect"])
def test_coverage_within_tolerance_of_fp64_oracle(renderer, oracle_mod, name):
    sc, _ = load_golden(name)
    render(renderer, sc)
    got = renderer.coverage()
    tiled = {}
    _, cov = oracle_mod.render(sc, coverage=True, tiled=tiled, threads=8)
    want = cov[tiled["tile_alpha"] == 1]
    assert got.shape == want.shape
    err = np.abs(got - want)
    print(f"{name}: coverage max err {err.max():.3e} mean {err.mean():.3e} over {got.shape[0]} alpha tiles")
    path = os.environ.get("PF_PARITY_LOG")
    if path:
        with open(path, "a") as f:
            f.write(json.dumps({"config": f"coverage:{name}", "alpha_tiles": int(got.shape[0]),
                                "coverage_max_err": float(err.max()), "coverage_mean_err": float(err.mean())}) + "\n")
    assert err.max() <= COVERAGE_TOL


def test_plain_small_full_size(renderer, oracle_mod):
    sc = S.plain_small()
    stats, got, img = render(renderer, sc)
    want = oracle_mod.tile_scene(sc, oracle_mod.Z_D3D11, threads=8)
    assert_canon(got, want, TILE_KEYS + LIST_KEYS)
    # the frame counters (the session renderer has them on): alpha and visible tiles
    assert stats["alpha_tiles"] == int(want["tile_alpha"].sum())
    assert stats["visible_tiles"] == int(((want["tile_alpha"] != 0) | (want["tile_backdrop"] != 0)).sum())
    ref_img, _ = oracle_mod.render(sc, threads=16)
    diff = np.abs(img.astype(np.int32) - ref_img.astype(np.int32))
    print(f"plain_small: {stats['fills']} fills, pixel max err {diff.max()} mean {diff.mean():.2e}")
    assert diff.max() <= PIXEL_TOL


@pytest.mark.parametrize("make", [
    lambda: S.large_single(seed=3, n_paths=2000, side=4096),
    lambda: S.glyphs(seed=3, n_paths=20000, side=2048),
    lambda: S.mixed(seed=7, n_paths=1024, side=4096),
])
def test_medium_scenes_bit_exact_and_pixels(renderer, oracle_mod, make):
    sc = make()
    stats, got, img = render(renderer, sc)
    want = oracle_mod.tile_scene(sc, oracle_mod.Z_D3D11, threads=16)
    assert_canon(got, want, TILE_KEYS + LIST_KEYS)
    ref_img, _ = oracle_mod.render(sc, threads=16)
    diff = np.abs(img.astype(np.int32) - ref_img.astype(np.int32))
    assert diff.max() <= PIXEL_TOL, (diff.max(), diff.mean())


def test_batched_equals_unbatched(renderer):
    scs = S.batched(n_scenes=6, first_seed=31, hi_paths=300)
    renderer.upload(scs)
    renderer.render()
    batch = [(renderer.canon(i), renderer.image(i)) for i in range(len(scs))]
    for i, sc in enumerate(scs):
        _, c1, img1 = render(renderer, sc)
        assert_canon(batch[i][0], c1, TILE_KEYS + LIST_KEYS)
        assert np.array_equal(batch[i][1], img1)


def test_deterministic_across_runs(renderer):
    sc = S.large_single(seed=5, n_paths=800, side=2048)
    _, c1, i1 = render(renderer, sc)
    _, c2, i2 = render(renderer, sc)
    assert_canon(c1, c2, TILE_KEYS + LIST_KEYS)
    assert np.array_equal(i1, i2)


def test_invalid_scenes_are_rejected(renderer, pf):
    sc = S.plain_small(n_paths=4, side=64)
    bad = S.Scene(**{**sc.__dict__, "path_start": sc.path_start[::-1].copy()})
    with pytest.raises(pf.PfError) as e:
        renderer.upload(bad)
    assert e.value.status == 1
    nan = S.Scene(**{**sc.__dict__, "points": sc.points.copy()})
    nan.points[3, 0] = np.nan
    renderer.upload(nan)
    with pytest.raises(pf.PfError) as e:
        renderer.render()
    assert e.value.status == 1
    # the context stays usable
    _, got, _ = render(renderer, sc)
    assert got["path_rect"].shape == (4, 4)


def test_fill_buffer_grows_and_frame_is_redone(pf, oracle_mod):
    # Long straight edges give many fills per line: a fresh context's first frame overruns its
    # starting fills capacity (about three per line), is counted, and binned again.
    pts = np.array([[3.5, 5.25], [2040.0, 7.0], [2043.5, 2041.0], [9.0, 2039.5],
                    [100.0, 100.0], [1900.0, 130.0], [1000.0, 1950.0]], np.float32)
    sc = S.Scene(points=pts, flags=np.zeros(7, np.uint8),
                 contour_start=np.array([0, 4, 7], np.uint32), path_start=np.array([0, 1, 2], np.uint32),
                 fill_rule=np.array([0, 1], np.uint8),
                 color=np.array([0xff2040c0, 0x80c02010], np.uint32), width=2048.0, height=2048.0)
    with pf.Renderer(device=0) as r:
        stats, got, img = render(r, sc)
        assert stats["fills"] > 3 * stats["microlines"]
        want = oracle_mod.tile_scene(sc, oracle_mod.Z_D3D11, threads=4)
        assert_canon(got, want, TILE_KEYS + LIST_KEYS)
        ref_img, _ = oracle_mod.render(sc, threads=8)
        assert np.abs(img.astype(np.int32) - ref_img.astype(np.int32)).max() <= PIXEL_TOL
        # the context keeps the larger buffer: the next frame needs no second binning
        stats2, got2, _ = render(r, sc)
        assert stats2["host_syncs"] < stats["host_syncs"]
        assert_canon(got2, want, TILE_KEYS + LIST_KEYS)
