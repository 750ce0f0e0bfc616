"""SVG ingestion (pf_svg_parse, host code) against the reference's nanosvg + SvgScene.

The parser must produce the scene the reference's canvas builds from the same document, bit for
bit: the points of every contour (nanosvg's float arithmetic, then Path2d's segment rules), the
contour and path structure, fill rules, colours, stroke styles, dash arrays and gradient paints.
Fixtures hold the reference's scene with the document's text; live runs compare against the
reference harness where it is built.  No GPU is needed: the parse is host code.
"""
import os

import numpy as np
import pytest

import svg_docs
from conftest import golden_with, load_golden

SCENE_KEYS = ["points", "flags", "contour_start", "path_start", "fill_rule", "color", "contour_closed", "dashes"]
RAW_KEYS = ["path_stroke", "path_paint", "stops"]
SVG_FIXTURES = golden_with("svg_text")


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint8).ravel()


def _same_as_reference(got, ref):
    for k in SCENE_KEYS:
        assert getattr(got, k).shape == ref[k].shape, (k, getattr(got, k).shape, ref[k].shape)
        assert np.array_equal(_bits(getattr(got, k)), _bits(ref[k])), k
    for k in RAW_KEYS:
        assert np.array_equal(_bits(getattr(got, k)), ref[k]), k
    assert (np.float32(got.width), np.float32(got.height)) == (ref["width"], ref["height"])


@pytest.mark.parametrize("name", SVG_FIXTURES)
def test_parse_matches_reference_fixture(pf, name):
    sc, _ = load_golden(name)
    with np.load(os.path.join(os.path.dirname(__file__), "golden", name + ".npz")) as d:
        text = d["svg_text"].tobytes()
    got = pf.parse_svg(text)
    for k in ["points", "flags", "contour_start", "path_start", "fill_rule", "color", "contour_closed", "dashes"]:
        assert np.array_equal(_bits(getattr(got, k)), _bits(getattr(sc, k))), k
    assert np.array_equal(_bits(got.path_stroke), _bits(sc.path_stroke))
    if sc.path_paint is None:
        assert not np.any(got.path_paint["type"]) and got.stops.size == 0
    else:
        assert np.array_equal(_bits(got.path_paint), _bits(sc.path_paint))
        assert np.array_equal(_bits(got.stops), _bits(sc.stops))
    assert (got.width, got.height) == (sc.width, sc.height)


def _reference(oracle_mod):
    if not oracle_mod.have_reference():
        pytest.skip("reference harness not built")
    return oracle_mod


@pytest.mark.parametrize("name", sorted(svg_docs.HAND))
def test_hand_written_documents_match_live_reference(pf, oracle_mod, name):
    O = _reference(oracle_mod)
    text = svg_docs.HAND[name]
    got, ref = pf.parse_svg(text), O.reference_svg_scene(text)
    _same_as_reference(got, ref)
    assert np.array_equal(O.ramps(got), ref["ramps"])


@pytest.mark.parametrize("first", range(0, 200, 25))
def test_random_documents_match_live_reference(pf, oracle_mod, first):
    O = _reference(oracle_mod)
    for seed in range(first, first + 25):
        text = svg_docs.random_document(seed)
        got, ref = pf.parse_svg(text), O.reference_svg_scene(text)
        _same_as_reference(got, ref)
        assert np.array_equal(O.ramps(got), ref["ramps"]), seed


@pytest.mark.parametrize("asset", ["features.svg", "tiger.svg"])
def test_reference_demo_assets_match_live_reference(pf, oracle_mod, asset):
    """The documents the reference's demo renders (read from the reference tree, not copied)."""
    O = _reference(oracle_mod)
    path = os.path.join(O.REF_ROOT, "assets", asset)
    if not os.path.exists(path):
        pytest.skip("reference assets absent")
    with open(path, "rb") as f:
        text = f.read()
    got, ref = pf.parse_svg(text), O.reference_svg_scene(text)
    assert got.n_paths > 10
    _same_as_reference(got, ref)
    assert np.array_equal(O.ramps(got), ref["ramps"])
    # the stroke outlines the upload will produce: the restated stroker on the parsed scene
    # equals the reference's own stroker on the reference's scene
    a = O.stroke_scene(got)
    b = O.stroke_scene(got, reference=True)
    for k in ["points", "flags", "contour_start", "path_start", "fill_rule"]:
        assert np.array_equal(_bits(getattr(a, k)), _bits(getattr(b, k))), k


def test_parsed_strokes_convert_like_the_reference(pf, oracle_mod):
    O = _reference(oracle_mod)
    for seed in range(300, 310):
        got = pf.parse_svg(svg_docs.random_document(seed, n_shapes=40))
        a, b = O.stroke_scene(got), O.stroke_scene(got, reference=True)
        for k in ["points", "flags", "contour_start", "path_start", "fill_rule"]:
            assert np.array_equal(_bits(getattr(a, k)), _bits(getattr(b, k))), (seed, k)


def test_documents_without_shapes(pf, oracle_mod):
    for text in [svg_docs.HAND["svg_empty"], "", "not xml at all", "<svg", "<svg><g><rect width='0' height='5'/></g>",
                 "<svg width='10' height='10'><path d='M 5 5'/><path d=''/><circle r='0'/><ellipse rx='4'/></svg>"]:
        sc = pf.parse_svg(text)
        assert sc.n_paths == 0 and sc.n_points == 0 and sc.n_contours == 0, text
        if oracle_mod.have_reference():
            ref = oracle_mod.reference_svg_scene(text)
            assert ref["color"].size == 0
            assert (np.float32(sc.width), np.float32(sc.height)) == (ref["width"], ref["height"])


def test_truncated_and_odd_documents_follow_the_reference(pf, oracle_mod):
    O = _reference(oracle_mod)
    full = svg_docs.random_document(7)
    cases = [full[:n] for n in (40, len(full) // 3, len(full) // 2, len(full) - 9)]
    cases += [full.replace('"', "'"), full.replace(" ", "\n\t "), full.replace("<path", "<!-- x --><path", 3),
              "<svg><path d='M10 10 L 20 20 Z Z z M 5 5 L 40 5 L40 40' stroke='red'/></svg>",
              "<svg><path d='M10,10 10,40 40,40 X 50 50 L 60 60' fill='#abc'/></svg>",
              "<svg><path d='L 10 10 M 20 20 30 20 30 30 h' fill='rgb(300, -5, 20)'/></svg>",
              "<svg><rect width='50' height='40' rx='60' fill='rgb(10%, 200%, 50.5%)' stroke='#zzz'/></svg>"]
    for text in cases:
        _same_as_reference(pf.parse_svg(text), O.reference_svg_scene(text))


def test_dpi_scales_physical_units(pf, oracle_mod):
    text = ("<svg width='2in' height='30mm'><rect x='1pc' y='2pt' width='1cm' height='0.5in' stroke='black' "
            "stroke-width='1mm' stroke-dasharray='2pt 1pc'/></svg>")
    a, b = pf.parse_svg(text, dpi=96.0), pf.parse_svg(text, dpi=300.0)
    assert b.width > a.width and b.points[:, 0].max() > a.points[:, 0].max()
    if oracle_mod.have_reference():
        for dpi, got in ((96.0, a), (300.0, b)):
            _same_as_reference(got, oracle_mod.reference_svg_scene(text, dpi))


def test_invalid_arguments(pf):
    import ctypes as C
    lib = pf.load()
    h = C.c_void_p()
    assert lib.pf_svg_parse(None, 0, 96.0, C.byref(h)) == 1
    assert lib.pf_svg_parse(b"<svg/>", 6, 96.0, None) == 1
    assert lib.pf_svg_scene(None, None) == 1
    lib.pf_svg_free(None)
