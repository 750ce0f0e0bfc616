import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "pathfinder-cpp_gb300")
for p in (os.path.join(ROOT, "oracle"), PKG, ROOT):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")
CANON_KEYS = ["path_rect", "path_tile_first", "path_column_first", "tile_alpha", "tile_backdrop",
              "tile_fill_count", "fills", "column_backdrop", "fb_tiles", "z", "fb_list_first", "fb_list",
              "tile_mask", "tile_clip", "tile_dest_backdrop"]
# the stroke outline stored with stroked fixtures (out_<key>)
OUTLINE_KEYS = ["points", "flags", "contour_start", "path_start", "fill_rule"]
TILE_KEYS = ["path_rect", "path_tile_first", "path_column_first", "tile_alpha", "tile_backdrop",
             "tile_fill_count", "fills", "column_backdrop", "tile_mask", "tile_clip", "tile_dest_backdrop"]


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


def golden_names():
    return sorted(os.path.basename(f)[:-4] for f in glob.glob(os.path.join(GOLDEN, "*.npz")))


def golden_with(key):
    """Names of the golden fixtures that hold the array ``key``."""
    out = []
    for name in golden_names():
        with np.load(os.path.join(GOLDEN, name + ".npz")) as d:
            if key in d.files:
                out.append(name)
    return out


def load_golden(name):
    import scenes as S
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    w, h, clear = d["meta"]
    sc = S.Scene(points=d["points"], flags=d["flags"], contour_start=d["contour_start"],
                 path_start=d["path_start"], fill_rule=d["fill_rule"], color=d["color"],
                 width=float(w), height=float(h), clear=int(clear),
                 path_clip=d["path_clip"] if "path_clip" in d else None,
                 path_is_clip=d["path_is_clip"] if "path_is_clip" in d else None,
                 path_stroke=d["path_stroke"] if "path_stroke" in d else None,
                 contour_closed=d["contour_closed"] if "contour_closed" in d else None,
                 dashes=d["dashes"] if "dashes" in d else None,
                 path_paint=d["path_paint"] if "path_paint" in d else None,
                 stops=d["stops"] if "stops" in d else None,
                 view_box=d["view_box"] if "view_box" in d else None)
    ref = {k: d["ref_" + k] for k in CANON_KEYS}
    for k in OUTLINE_KEYS:
        if "out_" + k in d:
            ref["out_" + k] = d["out_" + k]
    if "ref_ramps" in d:
        ref["ramps"] = d["ref_ramps"]
    return sc, ref


@pytest.fixture(scope="session")
def oracle_mod():
    import oracle
    oracle.build()
    return oracle


@pytest.fixture(scope="session")
def pf():
    """The CUDA library, built here if needed; on a machine without a GPU GPU tests are skipped."""
    import build as pf_build
    pf_build.build()
    import pfcuda
    pfcuda.load()
    return pfcuda


@pytest.fixture(scope="session")
def renderer(pf):
    if pf.device_count() < 1:
        pytest.fail("no CUDA device visible to a GPU test")
    r = pf.Renderer(stage_timing=True, counters=True)
    yield r
    r.close()
