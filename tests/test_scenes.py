"""Synthetic scene generators: shapes of the benchmark configurations, determinism."""
import numpy as np

import scenes as S


def test_plain_small_shape():
    sc = S.plain_small()
    assert sc.n_paths == 240 and sc.width == 1024
    nseg = (np.diff(sc.contour_start) - 1) // 3
    assert nseg.min() >= 8 and nseg.max() <= 24
    assert (sc.points >= 0).all() and (sc.points <= 1024).all()
    assert ((sc.color >> 24) == 255).all() and (sc.fill_rule == 0).all()


def test_large_single_shape():
    sc = S.large_single(n_paths=2000)
    assert set(np.unique(sc.fill_rule)) == {0, 1}
    alpha = sc.color >> 24
    assert 0.2 < (alpha < 255).mean() < 0.4
    assert alpha.min() >= 51


def test_glyphs_shape():
    sc = S.glyphs(n_paths=5000)
    nc = np.diff(sc.path_start)
    assert nc.min() >= 1 and nc.max() <= 3
    assert sc.clear == int(S.pack_rgba(255, 255, 255, 255))
    # quadratic loops only: flags 0/1 alternate
    assert set(np.unique(sc.flags)) == {0, 1}


def test_batched_sizes():
    scs = S.batched(n_scenes=16)
    n = np.array([s.n_paths for s in scs])
    assert n.min() >= 16 and n.max() <= 4096
    assert {s.width for s in scs} <= {256.0, 512.0, 1024.0, 2048.0}


def test_generators_are_deterministic():
    a, b = S.mixed(n_paths=300, side=1024), S.mixed(n_paths=300, side=1024)
    assert np.array_equal(a.points, b.points) and np.array_equal(a.flags, b.flags)
