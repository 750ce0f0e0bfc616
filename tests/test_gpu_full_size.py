"""Parity at the configurations' full sizes.

* the large single scene (20,000 paths at 4096 x 4096, seed 0),
* the glyph-like scene (150,000 outlines at 2048 x 2048, seed 0),
* the held-out mixed scene of the learned sizer (8,192 paths at 4096 x 4096, seed 7),
* every one of the 512 scenes of the batched configuration (seeds 1000-1511), rendered in one
  learned frame.

Each scene's integer tile data (tile rects, alpha flags, propagated int8 backdrops, fills after
the canonical sort, column sums, composite lists and z with the d3d11 z rule) must equal the
oracle's bit for bit, and its RGBA8 pixels must be within one code of the FP64 analytic-area
oracle.  The learned frame must equal the exact frame, and each batched scene must equal the
same scene rendered alone (a frame of one scene, from a second context).

The maximum and mean RGBA8 errors are printed and, when PF_PARITY_LOG names a file, appended
to it as one JSON line per configuration.
"""
import concurrent.futures as cf
import json
import os

import numpy as np
import pytest

import scenes as S
from conftest import TILE_KEYS

pytestmark = pytest.mark.gpu

LIST_KEYS = ["fb_tiles", "z", "fb_list_first", "fb_list"]
CANON = TILE_KEYS + LIST_KEYS
PIXEL_TOL = 1  # RGBA8 codes (1/255)
THREADS = max(1, min(16, os.cpu_count() or 1))


def _log(entry):
    print(json.dumps(entry))
    path = os.environ.get("PF_PARITY_LOG")
    if path:
        with open(path, "a") as f:
            f.write(json.dumps(entry) + "\n")


def _differs(a, b, keys=CANON):
    return [k for k in keys if a[k].shape != b[k].shape or not np.array_equal(a[k], b[k])]


class PixelErr:
    """Running max / mean of |GPU - oracle| over RGBA8 channels."""

    def __init__(self):
        self.max, self.sum, self.n, self.over = 0, 0, 0, 0

    def add(self, got, want):
        d = np.abs(got.astype(np.int16) - want.astype(np.int16))
        self.max = max(self.max, int(d.max()) if d.size else 0)
        self.sum += int(d.sum(dtype=np.int64))
        self.n += d.size
        self.over += int((d > PIXEL_TOL).sum())

    def entry(self):
        return {"rgba8_max_err": self.max, "rgba8_mean_err": self.sum / max(self.n, 1), "channels": self.n,
                "channels_over_tol": self.over}


def _oracle(oracle_mod, sc, threads):
    tiled = {}
    img, _ = oracle_mod.render(sc, oracle_mod.Z_D3D11, threads=threads, tiled=tiled)
    return tiled, img


@pytest.mark.parametrize("name,make", [
    ("large_single_20000_4096", lambda: S.large_single()),
    ("glyphs_150000_2048", lambda: S.glyphs()),
    ("mixed_8192_4096_held_out", lambda: S.mixed(seed=7, n_paths=8192, side=4096)),
])
def test_single_scene_full_size(pf, oracle_mod, name, make):
    sc = make()
    with cf.ThreadPoolExecutor(1) as ex:
        want_fut = ex.submit(_oracle, oracle_mod, sc, THREADS)
        with pf.Renderer() as r:
            r.sizer_load(pf.DEFAULT_WEIGHTS)
            r.upload(sc)
            st_exact = r.render()
            exact, exact_img = r.canon(), r.image()
            st_learned = r.render_learned()
            learned, learned_img = r.canon(), r.image()
        want, want_img = want_fut.result()
    assert _differs(exact, want) == []
    assert _differs(learned, exact) == []
    assert np.array_equal(learned_img, exact_img)
    err = PixelErr()
    err.add(exact_img, want_img)
    _log({"config": name, "paths": sc.n_paths, "fills": int(st_exact["fills"]), "tiles": int(st_exact["tiles"]),
          "alpha_tiles": int(want["tile_alpha"].sum()), "composite_entries": int(len(want["fb_list"])),
          "tiles_bit_exact": True, "learned_equals_exact": True,
          "learned_redone_exactly": bool(st_learned["overflow"]), **err.entry()})
    assert err.max <= PIXEL_TOL


def test_batched_512_full_size(pf, oracle_mod):
    scs = S.batched()
    assert len(scs) == 512
    err = PixelErr()
    fills = tiles = 0
    chunk = 2 * THREADS
    with pf.Renderer() as frame, pf.Renderer() as alone, cf.ThreadPoolExecutor(THREADS) as ex:
        frame.sizer_load(pf.DEFAULT_WEIGHTS)
        frame.upload(scs)
        st = frame.render_learned()
        alone.upload(scs)
        futs = {i: ex.submit(_oracle, oracle_mod, scs[i], 1) for i in range(min(chunk, len(scs)))}
        for i in range(len(scs)):
            # keep a bounded window of oracle scenes in flight
            nxt = i + chunk
            if nxt < len(scs):
                futs[nxt] = ex.submit(_oracle, oracle_mod, scs[nxt], 1)
            got, got_img = frame.canon(i), frame.image(i)
            alone.render(i, 1)
            one, one_img = alone.canon(i), alone.image(i)
            want, want_img = futs.pop(i).result()
            assert _differs(got, want) == [], f"scene {i}: batched frame differs from the oracle"
            assert _differs(one, got) == [], f"scene {i}: batched frame differs from the scene alone"
            assert np.array_equal(one_img, got_img), f"scene {i}: image differs from the scene alone"
            err.add(got_img, want_img)
            assert err.max <= PIXEL_TOL, f"scene {i}: pixel error {err.max}"
            fills += len(got["fills"])
            tiles += len(got["tile_alpha"])
    assert fills == st["fills"] and tiles == st["tiles"]
    _log({"config": "batched_512", "scenes": len(scs), "paths": int(st["paths"]), "fills": fills, "tiles": tiles,
          "frame": "learned", "learned_redone_exactly": bool(st["overflow"]), "tiles_bit_exact": True,
          "equals_scenes_alone": True, **err.entry()})
