"""The restated oracle against the reference's own tiler (golden fixtures, digests, live runs)."""
import hashlib
import json
import os

import numpy as np
import pytest

from conftest import CANON_KEYS, GOLDEN, OUTLINE_KEYS, golden_names, golden_with, load_golden


@pytest.mark.parametrize("name", golden_names())
def test_restated_tiler_matches_reference_golden(oracle_mod, name):
    sc, ref = load_golden(name)
    ours = oracle_mod.tile_scene(sc, oracle_mod.Z_D3D9)
    for k in CANON_KEYS:
        assert ours[k].shape == ref[k].shape, k
        assert np.array_equal(ours[k], ref[k]), k


STROKED = golden_with("out_points")


@pytest.mark.parametrize("name", STROKED)
def test_restated_stroker_matches_reference_golden(oracle_mod, name):
    """The restated OutlineDash + OutlineStrokeToFill against the reference's own output, bit for
    bit (points compared as bit patterns)."""
    sc, ref = load_golden(name)
    ours = oracle_mod.stroke_scene(sc)
    for k in OUTLINE_KEYS:
        a, b = getattr(ours, k), ref["out_" + k]
        assert a.shape == b.shape, k
        assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), k


@pytest.mark.parametrize("seed", [11, 12, 13, 14])
def test_restated_stroker_matches_live_reference(oracle_mod, seed):
    import scenes as S
    if not oracle_mod.have_reference():
        pytest.skip("reference harness not built")
    sc = S.stroked(seed=seed, n_paths=80, side=512, dash_share=0.5, fill_share=0.1)
    a, b = oracle_mod.stroke_scene(sc), oracle_mod.stroke_scene(sc, reference=True)
    for k in OUTLINE_KEYS:
        assert np.array_equal(getattr(a, k).view(np.uint8), getattr(b, k).view(np.uint8)), k
    assert oracle_mod.compare(oracle_mod.tile_scene(sc, oracle_mod.Z_D3D9), oracle_mod.reference_tile_scene(sc)) == []


def test_stroke_layout_checks(oracle_mod):
    import scenes as S
    sc = S.stroked(seed=3, n_paths=6, side=128, dash_share=1.0)
    bad = S.Scene(**{**sc.__dict__, "dashes": np.zeros_like(sc.dashes)})  # patterns of total 0
    with pytest.raises(RuntimeError):
        oracle_mod.stroke_scene(bad)
    st = sc.path_stroke.copy()
    st["line_cap"][0] = 7
    with pytest.raises(RuntimeError):
        oracle_mod.stroke_scene(S.Scene(**{**sc.__dict__, "path_stroke": st}))


GRADIENT = golden_with("ref_ramps")


@pytest.mark.parametrize("name", GRADIENT)
def test_restated_gradient_ramps_match_reference_golden(oracle_mod, name):
    """GradientTileBuilder's ramp rows (Gradient::add / sample, ColorF lerp, 8-bit truncation),
    restated, against the reference's own stored ramps."""
    sc, ref = load_golden(name)
    assert np.array_equal(oracle_mod.ramps(sc), ref["ramps"])


def test_restated_gradients_and_half_floats_match_live_reference(oracle_mod):
    import scenes as S
    if not oracle_mod.have_reference():
        pytest.skip("reference harness not built")
    rng = np.random.default_rng(5)
    vals = np.concatenate([rng.standard_normal(4000) * 10 ** rng.uniform(-9, 6, 4000),
                           [0.0, -0.0, 65504.0, 7e4, 1e-8, -3e-6, np.inf, -np.inf, np.nan]]).astype(np.float32)
    a, b = oracle_mod.half_trunc(vals), oracle_mod.half_trunc(vals, reference=True)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    sc = S.gradient_scene(seed=31, n_paths=150, side=512, share=1.0)
    assert np.array_equal(oracle_mod.ramps(sc), oracle_mod.reference_ramps(sc))
    assert oracle_mod.compare(oracle_mod.tile_scene(sc, oracle_mod.Z_D3D9), oracle_mod.reference_tile_scene(sc)) == []


def _digest(a):
    a = np.ascontiguousarray(a)
    return hashlib.sha256(a.dtype.str.encode() + str(a.shape).encode() + a.tobytes()).hexdigest()


def test_restated_tiler_full_plain_small_digests(oracle_mod):
    import scenes as S
    with open(os.path.join(GOLDEN, "digests.json")) as f:
        want = json.load(f)["plain_small_1024"]
    sc = S.plain_small()
    h = hashlib.sha256()
    for k in ["points", "flags", "contour_start", "path_start", "fill_rule", "color"]:
        h.update(_digest(getattr(sc, k)).encode())
    h.update(np.asarray([sc.width, sc.height, sc.clear], np.float64).tobytes())
    assert h.hexdigest() == want["scene"], "the generator no longer produces the pinned scene"
    ours = oracle_mod.tile_scene(sc, oracle_mod.Z_D3D9)
    for k in CANON_KEYS:
        assert _digest(ours[k]) == want["canon"][k], k


def test_restated_tiler_threads_agree(oracle_mod):
    import ctypes as C
    import scenes as S
    sc = S.large_single(seed=9, n_paths=300, side=1024)
    one = oracle_mod.tile_scene(sc)
    lib = oracle_mod._lib(oracle_mod.LIB_ORACLE)
    v, keep = oracle_mod.scene_view(sc)
    r = oracle_mod.Result()
    assert lib.pfo_tile_scene_mt(C.byref(v), C.c_int(1), C.c_int(4), C.byref(r)) == 0
    many = oracle_mod.result_to_dict(r)
    lib.pfo_free(C.byref(r))
    assert oracle_mod.compare(one, many) == []


@pytest.mark.parametrize("seed", [11, 12, 13, 14])
def test_restated_tiler_matches_live_reference(oracle_mod, seed):
    if not os.path.isdir(os.path.join(oracle_mod.REF_ROOT, "pathfinder")):
        pytest.skip("reference tree not present")
    oracle_mod.build(reference=True)
    import scenes as S
    scs = [S.plain_small(seed=seed, n_paths=16, side=320), S.large_single(seed=seed, n_paths=60, side=700),
           S.glyphs(seed=seed, n_paths=200, side=300)]
    for sc in scs:
        ref = oracle_mod.reference_tile_scene(sc)
        ours = oracle_mod.tile_scene(sc, oracle_mod.Z_D3D9)
        assert oracle_mod.compare(ref, ours, CANON_KEYS) == []


@pytest.mark.parametrize("seed", [21, 22, 23])
def test_restated_clipping_matches_live_reference(oracle_mod, seed):
    if not os.path.isdir(os.path.join(oracle_mod.REF_ROOT, "pathfinder")):
        pytest.skip("reference tree not present")
    oracle_mod.build(reference=True)
    import scenes as S
    sc = S.clipped(seed=seed, n_paths=80, side=384, n_clips=5)
    ref = oracle_mod.reference_tile_scene(sc)
    ours = oracle_mod.tile_scene(sc, oracle_mod.Z_D3D9)
    assert oracle_mod.compare(ref, ours, CANON_KEYS) == []
    assert set(np.unique(ours["tile_mask"])) == {0, 1, 2}  # every clip case occurs


def test_clip_pixel_known_answers(oracle_mod):
    # an opaque square over [0, 64)^2 clipped by a pixel-aligned rectangle [16, 48) x [8, 40):
    # the intersection is covered, everything else shows the clear colour.  As for any path,
    # add_fill's clamp to 4095/256 px (object_builder.cpp:33-35) leaves the last pixel column of
    # a tile 1/256 off: 254 inside, and at most 1 code of leak below the clip's bottom edge.
    import sys
    import scenes as S
    sys.path.insert(0, os.path.join(os.path.dirname(__file__), "golden"))
    from make_golden import build_scene, poly
    draw = build_scene([([poly(0, 0, 64, 0, 64, 64, 0, 64)], 0, (255, 0, 0, 255))], 64, 64)
    clip = build_scene([([poly(16, 8, 48, 8, 48, 40, 16, 40)], 0, (255, 255, 255, 255))], 64, 64)
    sc = S.with_clips(draw, clip, np.array([0]))
    img, _ = oracle_mod.render(sc)
    inside = img[8:40, 16:48]
    assert (inside[..., 0] >= 254).all() and (inside[..., 3] >= 254).all()
    outside = img.copy()
    outside[8:40, 16:48] = 0
    assert (outside <= 1).all() and (outside[:8] == 0).all() and (outside[:, :16] == 0).all()


def test_z_rules_differ_only_on_even_odd_even_backdrop(oracle_mod):
    sc, _ = load_golden("int8_wrap")
    d9 = oracle_mod.tile_scene(sc, oracle_mod.Z_D3D9)
    d11 = oracle_mod.tile_scene(sc, oracle_mod.Z_D3D11)
    for k in ["tile_alpha", "tile_backdrop", "fills", "column_backdrop"]:
        assert np.array_equal(d9[k], d11[k])


def test_pixel_oracle_known_answers(oracle_mod):
    # 16x16-aligned square: fully covered inside, untouched outside.  add_fill clamps
    # tile-local coordinates to 4095/256 px (object_builder.cpp:33-35), so the top edge's
    # fill stops 1/256 px short of the tile's right edge and the last pixel column of each
    # tile is covered 255/256 -> alpha 254.
    sc, _ = load_golden("aligned_square")
    img, _ = oracle_mod.render(sc)
    inner = img[16:48, 16:48]
    assert (inner[:, :, 1:3] == 0).all()
    cols = inner[:, :, 3].min(axis=0)
    assert (cols[[15, 31]] == 254).all() and (np.delete(cols, [15, 31]) == 255).all()
    assert (img[:16] == 0).all() and (img[48:] == 0).all()
    # half-pixel rectangle: edge pixels half covered (alpha 128 of 255 -> 127.5 rounds to 128)
    sc, _ = load_golden("half_pixel_rect")
    img, cov = oracle_mod.render(sc, coverage=True)
    assert img[20, 10, 3] in (127, 128) and img[20, 37, 3] in (127, 128)
    assert img[20, 20, 3] == 255 and img[20, 5, 3] == 0
    # hole: white inside the inner square, black ring
    sc, _ = load_golden("hole")
    img, _ = oracle_mod.render(sc)
    assert (img[30, 30] == [255, 255, 255, 255]).all()
    assert (img[12, 30] == [0, 0, 0, 255]).all()


def test_even_odd_hole_and_nonzero_fill(oracle_mod):
    sc, _ = load_golden("star_even_odd")
    img, _ = oracle_mod.render(sc)
    # the pentagon at the centre of the star is a hole under even-odd (only the translucent copy shows)
    assert img[52, 50, 0] < 128
