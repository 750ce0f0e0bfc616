"""What the learned sizer gains, and pf_render_auto, which runs it only where it pays.

The reference sizes its buffers by counting, reading the counts back and growing the buffers
(core/d3d11/renderer.cpp:540-577); the exact frame here does the same with exact counts (three
host synchronisations).  The learned frame sizes them from the sizer's per-path predictions in
one pass (one synchronisation after set-up, and its CUDA-graph replay one in all).

* On the batched configuration (512 scenes) the learned frame takes fewer host
  synchronisations and less device time than the exact frame, and pf_render_auto settles on it.
* On the held-out mixed scene, a batch of SVG documents and a batch of stroked scenes,
  pf_render_auto costs no more than the faster of the two frames (5% and 0.05 ms of slack for
  timing noise): it runs the learned frame only where it measured faster.
* Output is the same whichever frame runs.
"""
import numpy as np
import pytest

import scenes as S
from conftest import TILE_KEYS

pytestmark = pytest.mark.gpu

LIST_KEYS = ["fb_tiles", "z", "fb_list_first", "fb_list"]


def _median_ms(fn, n=5):
    return float(np.median([fn()["ms_total"] for _ in range(n)]))


def _settle(r, n=8):
    for _ in range(n):
        st = r.render_auto()
    return st


def _svg_batch(n):
    import pfcuda
    import svg_docs
    return [pfcuda.parse_svg(svg_docs.random_document(3000 + i, n_shapes=16 + (i * 37) % 600)) for i in range(n)]


def test_learned_frame_gains_on_the_batched_configuration(pf):
    scs = S.batched()
    with pf.Renderer(stage_timing=True) as r:
        r.sizer_load()
        r.upload(scs)
        _settle(r)
        auto = r.last_auto_choice()
        exact = [r.render() for _ in range(4)][1:]
        learned = [r.render_learned() for _ in range(4)][1:]  # the last three are replays
        ex_ms = float(np.median([s["ms_total"] for s in exact]))
        le_ms = float(np.median([s["ms_total"] for s in learned]))
        print(f"batched 512: exact {ex_ms:.2f} ms ({exact[-1]['host_syncs']} syncs), learned {le_ms:.2f} ms "
              f"({learned[-1]['host_syncs']} syncs); auto measured {auto}")
        assert all(s["overflow"] == 0 for s in learned)
        assert learned[-1]["host_syncs"] < exact[-1]["host_syncs"]
        assert le_ms < ex_ms
        assert auto["choice"] == "learned" and auto["last"] == "learned"
        assert learned[-1]["fills"] == exact[-1]["fills"] and learned[-1]["microlines"] == exact[-1]["microlines"]


@pytest.mark.parametrize("name,make", [
    ("mixed_8192_4096_held_out", lambda: [S.mixed(seed=7, n_paths=8192, side=4096)]),
    ("svg_64_documents", lambda: _svg_batch(64)),
    ("stroked_64_scenes", lambda: S.batched_stroked(n_scenes=64, first_seed=1000)),
])
def test_auto_frame_is_never_slower_than_the_faster_frame(pf, name, make):
    scs = make()
    with pf.Renderer(stage_timing=True) as r:
        r.sizer_load()
        r.upload(scs)
        _settle(r)
        auto_ms = _median_ms(r.render_auto)
        choice = r.last_auto_choice()
        r.render()
        ex_ms = _median_ms(r.render)
        r.render_learned()
        le_ms = _median_ms(r.render_learned)
        print(f"{name}: exact {ex_ms:.3f} ms, learned {le_ms:.3f} ms, auto {auto_ms:.3f} ms ({choice})")
        assert choice["choice"] in ("exact", "learned")
        assert auto_ms <= 1.05 * min(ex_ms, le_ms) + 0.05


def test_auto_frame_output_equals_exact_and_keeps_its_choice_across_uploads(pf):
    scs = S.batched(n_scenes=8, first_seed=801, hi_paths=600)
    with pf.Renderer() as r:
        r.sizer_load()
        r.upload(scs)
        r.render()
        want = [(r.canon(i), r.image(i)) for i in range(len(scs))]
        seen, choices = set(), []
        for _ in range(8):
            r.render_auto()
            seen.add(r.last_auto_choice()["last"])
            choices.append(r.last_auto_choice()["choice"])
            for i in range(len(scs)):
                got = r.canon(i)
                for k in TILE_KEYS + LIST_KEYS:
                    assert np.array_equal(got[k], want[i][0][k]), k
                assert np.array_equal(r.image(i), want[i][1])
        assert seen == {"exact", "learned"}  # both frames were timed
        # two timed frames of each kind decide: an untimed first exact frame and two timed ones,
        # an untimed first learned frame, the one that records its graph, two timed replays
        assert choices[:6] == [None] * 6 and None not in choices[6:]
        settled = r.last_auto_choice()
        assert settled["choice"] is not None and settled["exact_ms"] > 0 and settled["learned_ms"] > 0
        # a new upload of the same scenes keeps the measurements: no exact frame to re-time
        r.upload(scs)
        r.render_auto()
        assert r.last_auto_choice()["exact_ms"] == settled["exact_ms"]
        # without weights the auto frame is the exact one
    with pf.Renderer() as r:
        r.upload(scs)
        r.render_auto()
        assert r.last_auto_choice() == {"last": "exact", "choice": "exact", "exact_ms": 0.0, "learned_ms": 0.0}
