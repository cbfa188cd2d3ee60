"""Seeded synthetic workloads: determinism and the distributions they stand for."""
import numpy as np
import pytest

from scft_gb300 import workloads as W


def test_splitmix_is_deterministic_and_uniform():
    a = W.uniform(0, np.arange(10000), 3)
    b = W.uniform(0, np.arange(10000), 3)
    assert np.array_equal(a, b)
    assert 0.0 <= a.min() and a.max() < 1.0
    assert abs(a.mean() - 0.5) < 0.01
    assert not np.array_equal(a, W.uniform(1, np.arange(10000), 3))
    # fixed known values keep every host on the same instances
    np.testing.assert_allclose(W.uniform(0, [0, 1], 0), W.uniform(0, [0, 1], 0))


def test_single_small_matches_its_description():
    d = W.single_small()
    assert d["n_nodes"] == 33 and d["nsteps"] == 2048 and d["L"] == 4.0
    assert d["x"][-1] == 4.0 and d["w0"][0] == 0 and d["w0"][-1] == 0
    assert np.all(np.abs(d["w0"]) <= 0.1)
    f0 = d["f0"]
    assert f0[0] == 0 and f0[-1] == pytest.approx(0, abs=1e-15) and f0[16] == pytest.approx(1.0)


def test_batch_mixed_distribution():
    b = W.batch_mixed(4096)
    m = np.array([d["n_nodes"] - 1 for d in b])
    L = np.array([d["L"] for d in b])
    ns = np.array([d["nsteps"] for d in b])
    assert m.min() >= 32 and m.max() <= 1024
    # log-uniform: median near sqrt(32*1024)
    assert 140 < np.median(m) < 220
    assert 2 <= L.min() and L.max() <= 10
    assert set(ns) == {512, 1024, 2048, 4096}


def test_graded_mesh_ratio():
    x = W.graded_mesh(8192, 1.002, 7.0)
    h = np.diff(x)
    assert len(x) == 8193 and x[0] == 0 and x[-1] == pytest.approx(7.0)
    np.testing.assert_allclose(h[1:4096] / h[:4095], 1.002, rtol=1e-9)
    assert h.max() / h.min() == pytest.approx(1.002 ** 4095, rel=1e-9)


def test_warmstart_sets_are_disjoint_seeds():
    a = W.warmstart_train(64)
    b = W.warmstart_eval(64)
    assert all(64 <= d["n_nodes"] - 1 <= 512 for d in a + b)
    assert not np.allclose(a[0]["w0"][:10], b[0]["w0"][:10])
