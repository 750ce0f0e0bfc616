"""The learned sizer: GPU gradients against the FP64 oracle, training, and the learned
one-pass frame against the exact two-pass frame (identical output, with and without overflow)."""
import os

import numpy as np
import pytest

import mlp_oracle as M
import scenes as S
from conftest import TILE_KEYS

pytestmark = pytest.mark.gpu
LIST_KEYS = ["fb_tiles", "z", "fb_list_first", "fb_list"]


def _features_and_labels(renderer, scenes_list):
    feats, labels = [], []
    for sc in scenes_list:
        renderer.upload(sc)
        renderer.render()
        feats.append(renderer.path_features(sc.n_paths))
        l, f = renderer.path_counts(sc.n_paths)
        labels.append(np.log1p(np.stack([l, f], axis=1).astype(np.float32)))
    return np.concatenate(feats), np.concatenate(labels)


def test_gradient_matches_fp64_oracle(renderer):
    renderer.sizer_init(seed=3)
    params = renderer.sizer_params()
    rng = np.random.default_rng(1)
    x = np.abs(rng.normal(2.0, 1.5, (777, M.N_IN))).astype(np.float32)
    t = rng.normal(3.0, 1.0, (777, M.N_OUT)).astype(np.float32)
    g, loss = renderer.sizer_gradient(x, t)
    lo, go = M.loss_and_grad(params.astype(np.float64), x, t, round_bf16=True)
    assert abs(loss - lo) <= 1e-4 * abs(lo) + 1e-6, (loss, lo)
    err = np.abs(g.astype(np.float64) - go)
    print(f"sizer gradient: max abs err {err.max():.3e}, max |grad| {np.abs(go).max():.3e}")
    assert err.max() <= 2e-4 * np.abs(go).max() + 1e-7


def test_prediction_matches_oracle(renderer):
    renderer.sizer_init(seed=5)
    params = renderer.sizer_params()
    x = np.abs(np.random.default_rng(2).normal(2.0, 1.0, (300, M.N_IN))).astype(np.float32)
    got = renderer.sizer_predict(x)
    want = M.predict(params.astype(np.float64), x)
    assert np.abs(got - want).max() <= 1e-4 * np.abs(want).max() + 1e-5


def test_training_learns_counts(renderer):
    scs = [S.plain_small(seed=50 + i, n_paths=200, side=512) for i in range(3)]
    scs += [S.large_single(seed=60, n_paths=600, side=1024), S.glyphs(seed=61, n_paths=2000, side=512)]
    x, y = _features_and_labels(renderer, scs)
    mu, sd = x.mean(0), x.std(0) + 1e-6
    renderer.sizer_init(seed=7)
    losses = renderer.sizer_train((x - mu) / sd, y, epochs=40, batch=512, lr=3e-3, seed=1)
    print("training loss", losses[0], "->", losses[-1])
    assert losses[-1] < 0.25 * losses[0]
    assert losses[-1] < 0.1


@pytest.fixture(scope="module")
def trained(renderer, tmp_path_factory):
    """A sizer trained on a few scenes (features standardised, standardisation folded in)."""
    scs = [S.plain_small(seed=70 + i, n_paths=300, side=256 << (i % 4)) for i in range(6)]
    scs += [S.large_single(seed=80, n_paths=800, side=2048), S.glyphs(seed=81, n_paths=3000, side=512)]
    x, y = _features_and_labels(renderer, scs)
    mu, sd = x.mean(0), x.std(0) + 1e-6
    renderer.sizer_init(seed=9)
    renderer.sizer_train((x - mu) / sd, y, epochs=60, batch=512, lr=3e-3, seed=2)
    p = M.unpack(renderer.sizer_params().astype(np.float64))
    p["b1"] = p["b1"] - (p["W1"] * (mu / sd)[None, :]).sum(1)
    p["W1"] = p["W1"] / sd[None, :]
    renderer.set_sizer_params(M.pack(p).astype(np.float32))
    path = str(tmp_path_factory.mktemp("sizer") / "sizer.bin")
    renderer.sizer_save(path)
    return path


def _frame(renderer, sc, learned):
    renderer.upload(sc)
    st = renderer.render_learned() if learned else renderer.render()
    n = len(sc) if isinstance(sc, list) else 1
    return st, [renderer.canon(i) for i in range(n)], [renderer.image(i) for i in range(n)]


@pytest.mark.parametrize("make", [
    lambda: S.plain_small(seed=91, n_paths=240, side=1024),
    lambda: S.large_single(seed=92, n_paths=1500, side=2048),
    lambda: S.glyphs(seed=93, n_paths=5000, side=1024),
    lambda: S.batched(n_scenes=5, first_seed=94, hi_paths=400),
])
def test_learned_frame_equals_exact_frame(renderer, trained, make):
    sc = make()
    renderer.sizer_load(trained)
    renderer.sizer_margin(1.3, 8.0, 0.15)
    st_l, canon_l, img_l = _frame(renderer, sc, True)
    st_e, canon_e, img_e = _frame(renderer, sc, False)
    for a, b in zip(canon_l, canon_e):
        for k in TILE_KEYS + LIST_KEYS:
            assert np.array_equal(a[k], b[k]), k
    for a, b in zip(img_l, img_e):
        assert np.array_equal(a, b)
    assert st_l["fills"] == st_e["fills"] and st_l["microlines"] == st_e["microlines"]
    print("learned frame: overflow", st_l["overflow"], "syncs", st_l["host_syncs"], "vs", st_e["host_syncs"])


def test_forced_overflow_falls_back_to_exact(renderer, trained):
    sc = S.large_single(seed=95, n_paths=600, side=1024)
    renderer.sizer_load(trained)
    renderer.sizer_margin(1e-3, 0.0, 0.0)
    st_l, canon_l, img_l = _frame(renderer, sc, True)
    renderer.sizer_margin(1.3, 8.0, 0.15)
    st_e, canon_e, img_e = _frame(renderer, sc, False)
    assert st_l["overflow"] == 1
    for k in TILE_KEYS + LIST_KEYS:
        assert np.array_equal(canon_l[0][k], canon_e[0][k]), k
    assert np.array_equal(img_l[0], img_e[0])


def test_save_load_roundtrip(renderer, trained, tmp_path):
    renderer.sizer_load(trained)
    a = renderer.sizer_params()
    p = str(tmp_path / "copy.bin")
    renderer.sizer_save(p)
    renderer.sizer_init(seed=123)
    renderer.sizer_load(p)
    assert np.array_equal(a, renderer.sizer_params())
    with open(p, "r+b") as f:
        f.write(b"XXXX")
    with pytest.raises(Exception):
        renderer.sizer_load(p)
