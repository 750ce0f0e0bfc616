"""Stroke-to-fill and dashing on the GPU against the reference and the oracle.

The upload converts stroked paths on the GPU (OutlineDash, then OutlineStrokeToFill, as
Canvas::stroke_path does, pathfinder/core/canvas.cpp:270-300).  The stroke outline must equal
the reference's bit for bit (golden fixtures made by the reference's own stroker; the oracle
restatement on larger scenes); tiles follow from it bit for bit and pixels stay within one
RGBA8 code of the FP64 oracle.
"""
import numpy as np
import pytest

import scenes as S
from conftest import OUTLINE_KEYS, TILE_KEYS, golden_with, load_golden

pytestmark = pytest.mark.gpu

LIST_KEYS = ["fb_tiles", "z", "fb_list_first", "fb_list"]
PIXEL_TOL = 1
STROKED = golden_with("out_points")


def _same_outline(got, want):
    for k in OUTLINE_KEYS:
        assert got[k].shape == want[k].shape, (k, got[k].shape, want[k].shape)
        assert np.array_equal(got[k].view(np.uint8), want[k].view(np.uint8)), k


def _outline_dict(sc):
    return {k: getattr(sc, k) for k in OUTLINE_KEYS}


@pytest.mark.parametrize("name", STROKED)
def test_stroke_outline_bit_exact_vs_reference(renderer, name):
    sc, ref = load_golden(name)
    renderer.upload(sc)
    _same_outline(renderer.outline(), {k: ref["out_" + k] for k in OUTLINE_KEYS})


@pytest.mark.parametrize("seed,n_paths,side,dash", [(21, 300, 1024, 0.3), (22, 800, 2048, 0.5), (23, 120, 256, 1.0)])
def test_stroked_scene_outline_tiles_and_pixels(renderer, oracle_mod, seed, n_paths, side, dash):
    sc = S.stroked(seed=seed, n_paths=n_paths, side=side, dash_share=dash, fill_share=0.1)
    renderer.upload(sc)
    _same_outline(renderer.outline(), _outline_dict(oracle_mod.stroke_scene(sc)))
    renderer.render()
    got, img = renderer.canon(), renderer.image()
    want = oracle_mod.tile_scene(sc, oracle_mod.Z_D3D11, threads=8)
    for k in TILE_KEYS + LIST_KEYS:
        assert np.array_equal(got[k], want[k]), k
    ref, _ = oracle_mod.render(sc, threads=16)
    diff = np.abs(img.astype(np.int32) - ref.astype(np.int32))
    print(f"stroked s{seed}: {renderer.outline()['points'].shape[0]} outline points, "
          f"pixel max err {diff.max()} mean {diff.mean():.2e}")
    assert diff.max() <= PIXEL_TOL


def test_batch_of_stroked_clipped_and_plain_scenes(renderer, oracle_mod):
    scs = [S.stroked(seed=31, n_paths=150, side=512), S.plain_small(seed=32, n_paths=100, side=512),
           S.stroked(seed=33, n_paths=90, side=256, dash_share=0.8), S.clipped(seed=34, n_paths=80, side=512)]
    renderer.upload(scs)
    for i, sc in enumerate(scs):
        _same_outline(renderer.outline(i), _outline_dict(oracle_mod.fill_scene(sc)))
    renderer.render()
    batch = [(renderer.canon(i), renderer.image(i)) for i in range(len(scs))]
    for i, sc in enumerate(scs):
        renderer.upload(sc)
        renderer.render()
        for k in TILE_KEYS + LIST_KEYS:
            assert np.array_equal(batch[i][0][k], renderer.canon()[k]), (i, k)
        assert np.array_equal(batch[i][1], renderer.image())


def test_learned_frame_with_strokes_equals_exact(pf):
    scs = [S.stroked(seed=41 + i, n_paths=100 + 80 * i, side=1024, dash_share=0.4) for i in range(3)]
    with pf.Renderer(device=0) as r:
        r.upload(scs)
        r.sizer_load()
        r.render()
        exact = [r.image(i) for i in range(len(scs))]
        for _ in range(3):
            assert r.render_learned()["overflow"] == 0
            for i in range(len(scs)):
                assert np.array_equal(r.image(i), exact[i])


def test_invalid_strokes_are_rejected(renderer, pf):
    sc = S.stroked(seed=51, n_paths=8, side=128, dash_share=1.0)
    cases = []
    for field, value in (("line_cap", 7), ("line_join", 3), ("line_width", -1.0), ("miter_limit", np.inf)):
        st = sc.path_stroke.copy()
        st[field][2] = value
        cases.append(S.Scene(**{**sc.__dict__, "path_stroke": st}))
    cases.append(S.Scene(**{**sc.__dict__, "dashes": np.zeros_like(sc.dashes)}))      # all-zero patterns
    st = sc.path_stroke.copy()
    st["dash_first"][0] = len(sc.dashes)                                              # outside the array
    cases.append(S.Scene(**{**sc.__dict__, "path_stroke": st}))
    nan = S.Scene(**{**sc.__dict__, "points": sc.points.copy()})
    nan.points[1, 0] = np.nan                                                          # in a stroked path
    cases.append(nan)
    for bad in cases:
        with pytest.raises(pf.PfError) as e:
            renderer.upload(bad)
        assert e.value.status == 1
    renderer.upload(sc)  # the context stays usable
    renderer.render()


def test_dash_step_bound_is_an_error(renderer, pf):
    # a 100 px line dashed every 1e-5 px needs ten million steps: past the 2^22 bound
    sc = S.Scene(points=np.array([[10, 10], [110, 10]], np.float32), flags=np.zeros(2, np.uint8),
                 contour_start=np.array([0, 2], np.uint32), path_start=np.array([0, 1], np.uint32),
                 fill_rule=np.zeros(1, np.uint8), color=np.array([0xff0000ff], np.uint32), width=128.0, height=128.0)
    st = np.zeros(1, S.STROKE_DTYPE)
    st[0] = (2.0, 10.0, 0, 0, 0, 0, 2, 0.0)
    sc.path_stroke, sc.dashes = st, np.array([1e-5, 1e-5], np.float32)
    with pytest.raises(pf.PfError) as e:
        renderer.upload(sc)
    assert e.value.status == 5
    sc.dashes = np.array([4.0, 3.0], np.float32)
    renderer.upload(sc)
    renderer.render()
