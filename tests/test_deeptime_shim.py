"""Host logic of the deeptime.clustering-shaped module (no GPU needed):
install/uninstall, the metric registry, seeds and argument checks, and that
every estimator call fails loudly without a CUDA device."""
import sys

import numpy as np
import pytest

from pyemma_gb300 import deeptime_clustering as dc


def test_install_resolves_deeptime_clustering():
    before = {name: sys.modules.get(name) for name in ("deeptime", "deeptime.clustering")}
    assert dc.install(force=True)
    try:
        from deeptime.clustering import ClusterModel, KMeans, MiniBatchKMeans, RegularSpace, metrics
        import deeptime.clustering as mod
        assert mod is dc
        assert KMeans is dc.KMeans and MiniBatchKMeans is dc.MiniBatchKMeans
        assert ClusterModel is dc.ClusterModel and RegularSpace is dc.RegularSpace and metrics is dc.metrics
    finally:
        dc.uninstall()
    assert {name: sys.modules.get(name) for name in before} == before


def test_metric_registry():
    assert "euclidean" in dc.metrics and "minRMSD" in dc.metrics
    assert set(dc.metrics.available) >= {"euclidean", "minRMSD"}
    assert hasattr(dc.metrics["minRMSD"], "compute_metric")
    assert hasattr(dc.metrics["euclidean"].kmeans, "init_centers_kmpp")
    with pytest.raises(KeyError):
        dc.metrics["hamming"]
    sentinel = object()
    saved = dc.metrics["minRMSD"]
    dc.metrics.register("minRMSD", sentinel)  # as regspace.py:89 does with its own module
    try:
        assert dc.metrics["minRMSD"] is sentinel
    finally:
        dc.metrics.register("minRMSD", saved)


def test_seed_rules():
    assert dc._seed(True) == 42
    assert dc._seed(7) == 7 and dc._seed(np.int64(2 ** 32 - 1)) == 2 ** 32 - 1
    for s in (False, None, -1, 2 ** 32):
        v = dc._seed(s)
        assert 0 <= v <= 2 ** 32 - 1


def test_argument_checks():
    with pytest.raises(ValueError):
        dc.KMeans(5, init_strategy="random")
    with pytest.raises(ValueError):
        dc.KMeans(0)
    with pytest.raises(ValueError):
        dc.KMeans(5, metric="hamming")
    with pytest.raises(ValueError):
        dc.ClusterModel(np.zeros(3, dtype=np.float32))
    with pytest.raises(ValueError):
        dc.RegularSpace(-1.0)
    with pytest.raises(ValueError):
        dc.RegularSpace(1.0, metric="hamming")
    assert dc.RegularSpace(1.0, metric="minRMSD").metric == "minRMSD"
    with pytest.raises(NotImplementedError):
        dc.MiniBatchKMeans(3).fit(np.zeros((10, 2), dtype=np.float32))
    km = dc.KMeans(3, 10, "euclidean", tolerance=1e-5, init_strategy="kmeans++", fixed_seed=42, n_jobs=1)
    assert km.fetch_model() is None and km.max_iter == 10
    km.initial_centers = [[0, 0], [1, 1], [2, 2]]
    assert km.initial_centers.dtype == np.float32 and km.initial_centers.flags["C_CONTIGUOUS"]
    assert dc.RegularSpace(0.5).fetch_model() is None


def test_calls_fail_without_a_gpu():
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    X = np.zeros((10, 3), dtype=np.float32)
    for call in (lambda: dc.KMeans(2).fit(X),
                 lambda: dc.ClusterModel(X[:2]).transform(X),
                 lambda: dc.RegularSpace(0.5).partial_fit(X),
                 lambda: dc.metrics["minRMSD"].compute_metric(X[0], X[1]),
                 lambda: dc.metrics["euclidean"].kmeans.init_centers_kmpp(X, 2, 1, 1, None)):
        with pytest.raises(RuntimeError):
            call()
