"""SVG documents end to end on the GPU: parsed on the host (pf_svg_parse), uploaded straight from
the parser's arrays (strokes converted on the GPU), tiled and composited.

The fixtures hold the reference's own scene for each document (nanosvg + SvgScene through the
reference harness) with its stroke outline and tiles; larger documents are checked against the
oracle.  Tile data and outlines are bit-exact; pixels follow the gradient rule of
test_gpu_gradient.py (within one RGBA8 code, radial edges aside).
"""
import os

import numpy as np
import pytest

import scenes as S
import svg_docs
from conftest import GOLDEN, OUTLINE_KEYS, TILE_KEYS, golden_with, load_golden

pytestmark = pytest.mark.gpu

LIST_KEYS = ["fb_tiles", "z", "fb_list_first", "fb_list"]
PIXEL_TOL = 1
RADIAL_EDGE_SHARE = 2e-3


def _pixels(img, want, sc, label):
    diff = np.abs(img.astype(np.int32) - want.astype(np.int32)).max(axis=2)
    over = int((diff > PIXEL_TOL).sum())
    print(f"{label}: pixel max err {diff.max()}, {over} of {diff.size} beyond {PIXEL_TOL}")
    radial = sc.path_paint is not None and np.any(sc.path_paint["type"] == S.PAINT_RADIAL)
    assert over <= (RADIAL_EDGE_SHARE * diff.size if radial else 0)


def _text(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as d:
        return d["svg_text"].tobytes()


@pytest.mark.parametrize("name", golden_with("svg_text"))
def test_document_outline_and_tiles_match_reference(pf, renderer, oracle_mod, name):
    sc, ref = load_golden(name)
    with pf.SvgDocument(_text(name)) as doc:
        renderer.upload_views([doc.view])
    out = renderer.outline()
    for k in OUTLINE_KEYS:
        assert np.array_equal(out[k].view(np.uint8), ref["out_" + k].view(np.uint8)), k
    renderer.render()
    got = renderer.canon()
    for k in TILE_KEYS:
        assert np.array_equal(got[k], ref[k]), k
    want, _ = oracle_mod.render(sc, threads=8)
    _pixels(renderer.image(), want, sc, name)


@pytest.mark.parametrize("seed,n_shapes", [(501, 300), (502, 600), (503, 1200)])
def test_large_documents_match_oracle(pf, renderer, oracle_mod, seed, n_shapes):
    text = svg_docs.random_document(seed, n_shapes=n_shapes)
    sc = pf.parse_svg(text)
    with pf.SvgDocument(text) as doc:
        renderer.upload_views([doc.view])
    out = renderer.outline()
    want_outline = oracle_mod.stroke_scene(sc)
    for k in OUTLINE_KEYS:
        assert np.array_equal(out[k].view(np.uint8), getattr(want_outline, k).view(np.uint8)), k
    renderer.render()
    got = renderer.canon()
    want = oracle_mod.tile_scene(sc, oracle_mod.Z_D3D11, threads=8)
    for k in TILE_KEYS + LIST_KEYS:
        assert np.array_equal(got[k], want[k]), k
    ref, _ = oracle_mod.render(sc, threads=16)
    _pixels(renderer.image(), ref, sc, f"svg s{seed}")


def test_batch_of_documents_equals_one_by_one(pf, renderer):
    docs = [pf.SvgDocument(svg_docs.random_document(600 + i, n_shapes=60 + 20 * i)) for i in range(12)]
    docs.append(pf.SvgDocument(svg_docs.HAND["svg_gradients"]))
    renderer.upload_views([d.view for d in docs])
    renderer.render()
    batch = [(renderer.canon(i), renderer.image(i)) for i in range(len(docs))]
    for i, d in enumerate(docs):
        renderer.upload_views([d.view])
        renderer.render()
        for k in TILE_KEYS + LIST_KEYS:
            assert np.array_equal(batch[i][0][k], renderer.canon()[k]), (i, k)
        assert np.array_equal(batch[i][1], renderer.image())
    for d in docs:
        d.close()


def test_learned_frame_on_documents_equals_exact(pf):
    """The sizer was fitted on the synthetic batches, not on documents: where it sizes a buffer
    too small the frame is redone exactly, and the images are the exact frame's either way."""
    docs = [pf.SvgDocument(svg_docs.random_document(700 + i, n_shapes=200)) for i in range(4)]
    with pf.Renderer(device=0) as r:
        r.upload_views([d.view for d in docs])
        r.sizer_load()
        r.render()
        exact = [r.image(i) for i in range(len(docs))]
        for _ in range(2):
            print("learned frame on documents: overflow", r.render_learned()["overflow"])
            for i in range(len(docs)):
                assert np.array_equal(r.image(i), exact[i])
    for d in docs:
        d.close()


def test_document_without_shapes_renders_clear(pf, renderer):
    with pf.SvgDocument(svg_docs.HAND["svg_empty"]) as doc:
        assert doc.view.n_paths == 0
        renderer.upload_views([doc.view])
    renderer.render()
    img = renderer.image()
    assert img.shape == (32, 64, 4) and not img.any()
    with pf.SvgDocument("<svg></svg>") as doc:
        with pytest.raises(pf.PfError) as e:
            renderer.upload_views([doc.view])
        assert e.value.status == 1
