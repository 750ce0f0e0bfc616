"""Launch parameters (pf_tuning) and the autotuner that searches them.

Output never depends on the launch parameters: every setting the autotuner may pick renders the
same tiles and pixels, in the exact frame and in the learned frame's graph replay (concurrent
binning classes run on side streams inside the recorded graph).  pf_autotune returns a setting
no slower than the one it started from, and bad settings are rejected.
"""
import numpy as np
import pytest

import scenes as S
from conftest import TILE_KEYS

pytestmark = pytest.mark.gpu

LIST_KEYS = ["fb_tiles", "z", "fb_list_first", "fb_list"]

SETTINGS = [
    {"bin_ctas_per_sm": [0, 0, 0], "long_line": 8.0, "bin_concurrent": 1, "seg_sorted": 1, "composite_ticket": 4},
    {"bin_ctas_per_sm": [1, 2, 1], "long_line": 4.0, "bin_concurrent": 1, "seg_sorted": 0, "composite_ticket": 1},
    {"bin_ctas_per_sm": [3, 1, 2], "long_line": 32.0, "bin_concurrent": 0, "seg_sorted": 1, "composite_ticket": 0},
    {"bin_ctas_per_sm": [0, 4, 0], "long_line": 1.0, "bin_concurrent": 0, "seg_sorted": 0, "composite_ticket": 16},
]


def _outputs(r, n):
    return [(r.canon(i), r.image(i)) for i in range(n)]


def _same(a, b):
    for (ca, ia), (cb, ib) in zip(a, b):
        for k in TILE_KEYS + LIST_KEYS:
            assert np.array_equal(ca[k], cb[k]), k
        assert np.array_equal(ia, ib)


@pytest.mark.parametrize("setting", SETTINGS)
def test_output_does_not_depend_on_launch_parameters(pf, setting):
    scs = S.batched(n_scenes=12, first_seed=2100, hi_paths=1500) + [S.clipped(seed=5, n_paths=300, side=1024)]
    with pf.Renderer() as r:
        r.sizer_load()
        r.upload(scs)
        r.render()
        want = _outputs(r, len(scs))
        r.set_tuning(setting)
        assert r.tuning() == setting
        r.render()
        _same(_outputs(r, len(scs)), want)
        for _ in range(3):  # plain learned frame, recorded + replayed, replayed
            st = r.render_learned()
            _same(_outputs(r, len(scs)), want)
        assert st["host_syncs"] == 1


def test_autotune_returns_a_setting_no_slower_than_the_start(pf):
    scs = S.batched(n_scenes=24, first_seed=2200, hi_paths=1200)
    with pf.Renderer() as r:
        r.sizer_load()
        r.upload(scs)
        r.render()
        want = _outputs(r, len(scs))
        best, best_ms, start_ms = r.autotune(frames=2)
        print(f"autotune: {start_ms:.3f} ms -> {best_ms:.3f} ms with {best}")
        assert best_ms <= start_ms
        assert r.tuning() == best
        r.render()
        _same(_outputs(r, len(scs)), want)


def test_bad_launch_parameters_are_rejected(pf):
    with pf.Renderer() as r:
        good = r.tuning()
        for bad in ({**good, "long_line": 0.5}, {**good, "bin_concurrent": 2}, {**good, "bin_ctas_per_sm": [0, 65, 0]},
                    {**good, "composite_ticket": 5000}):
            with pytest.raises(pf.PfError) as e:
                r.set_tuning(bad)
            assert e.value.status == 1
        assert r.tuning() == good
