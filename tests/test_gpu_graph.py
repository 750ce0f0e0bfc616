"""The learned frame replayed as a CUDA graph equals the frame it was captured from.

The second learned frame in a row over the same scenes (the first one has sized the buffers)
is recorded as a graph and replayed; later learned frames replay it (one launch, one
synchronisation).
Any change of scenes, sizer, buffers or flags drops the graph.
"""
import numpy as np
import pytest

import scenes as S
from conftest import TILE_KEYS

pytestmark = pytest.mark.gpu

LIST_KEYS = ["fb_tiles", "z", "fb_list_first", "fb_list"]


def _outputs(r, n):
    return [(r.canon(i), r.image(i)) for i in range(n)]


def _same(a, b):
    for (ca, ia), (cb, ib) in zip(a, b):
        for k in TILE_KEYS + LIST_KEYS:
            assert np.array_equal(ca[k], cb[k]), k
        assert np.array_equal(ia, ib)


def test_replayed_learned_frame_equals_exact_frame(pf):
    scs = S.batched(n_scenes=6, first_seed=501, hi_paths=400)
    with pf.Renderer(device=0, stage_timing=True) as r:
        r.upload(scs)
        r.sizer_load()
        r.render()
        exact = _outputs(r, len(scs))
        first = r.render_learned()            # plain learned frame
        assert first["host_syncs"] >= 2
        _same(_outputs(r, len(scs)), exact)
        for _ in range(3):                    # recorded and replayed, then replays
            st = r.render_learned()
            assert st["host_syncs"] == 1, st
            assert st["overflow"] == 0
            assert st["ms_total"] > 0 and st["ms_bin"] > 0  # stage events recorded by the replay
            assert st["fills"] == first["fills"] and st["microlines"] == first["microlines"]
            _same(_outputs(r, len(scs)), exact)


def test_graph_is_dropped_when_scenes_or_sizer_change(pf):
    a = S.batched(n_scenes=3, first_seed=601, hi_paths=200)
    b = S.batched(n_scenes=4, first_seed=701, hi_paths=300)
    with pf.Renderer(device=0) as r:
        r.sizer_load()
        r.upload(a)
        r.render_learned()
        assert r.render_learned()["host_syncs"] == 1
        # new scenes: a plain frame again, with the new scenes' output
        r.upload(b)
        st = r.render_learned()
        assert st["host_syncs"] >= 2
        got = _outputs(r, len(b))
        r.render()
        _same(got, _outputs(r, len(b)))
        # an exact frame in between, then a replay still matches
        r.render_learned()
        st = r.render_learned()
        _same(_outputs(r, len(b)), got)
        # new margins: the graph's budgets are stale, so the next frame is a plain one
        r.sizer_margin(1.5, 16.0, 0.2)
        assert r.render_learned()["host_syncs"] >= 2
        _same(_outputs(r, len(b)), got)
        # a subset of the scenes is another frame
        r.render_learned(1, 2)
        assert r.render_learned(1, 2)["host_syncs"] == 1
        for i in (1, 2):
            assert np.array_equal(r.image(i), got[i][1])
