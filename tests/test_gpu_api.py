"""The drop-in API on the GPU, restating the reference's contract tests.

pyemma/coordinates/clustering/tests/test_cluster.py:36-190,
test_assign.py:47-239 and test_kmeans.py:39-426, with freshly generated
inputs; results are also compared with the oracle where one exists.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def coor():
    from pyemma_gb300 import coordinates
    return coordinates


@pytest.fixture(scope="module")
def blobs():
    rng = np.random.default_rng(0)
    means = [(-3, 0), (-1, 1), (0, 0), (1, -1), (4, 2)]
    X = np.zeros((5000, 2))
    for i, m in enumerate(means):
        X[i * 1000:(i + 1) * 1000] = 0.1 * rng.normal(size=(1000, 2)) + m
    return X, np.array(means, dtype=float)


def test_assign_exact_blobs(coor, blobs):
    X, centers = blobs
    ass = coor.assign_to_centers(data=X, centers=centers, return_dtrajs=False, n_jobs=1)
    assert len(ass.dtrajs) == 1
    assert ass.dtrajs[0].dtype == ass.output_type()
    np.testing.assert_array_equal(ass.dtrajs[0], np.arange(5000) // 1000)
    out = ass.get_output()
    assert len(out) == 1 and out[0].shape == (5000, 1) and out[0].dtype == np.int32
    Y = ass.transform(X)
    assert Y.shape == (5000, 1)
    np.testing.assert_array_equal(Y, out[0])
    assert ass.dimension() == 1
    assert ass.clustercenters.shape == (5, 2)
    assert ass.trajectory_length(0) == 5000
    with pytest.raises(IndexError):
        ass.trajectory_length(1)
    for itraj, chunk in ass:
        assert chunk.shape[1] == 1


def test_assign_return_dtrajs_and_chunksize(coor, blobs, oracle):
    X, centers = blobs
    rng = np.random.default_rng(1)
    big = X[rng.choice(1000, 100)]
    a = coor.assign_to_centers(X, big, n_jobs=2, chunksize=1000)
    b = coor.assign_to_centers(X, big, n_jobs=1, chunksize=1000)
    np.testing.assert_equal(a, b)
    np.testing.assert_array_equal(a[0], oracle.assign(X, big))


def test_assign_wrong_centers(coor):
    with pytest.raises(ValueError):
        coor.assign_to_centers(np.zeros((100, 3)), np.zeros((5, 4)))
    with pytest.raises(ValueError):
        coor.assign_to_centers(np.zeros((100, 3)), np.zeros(1))


def test_assign_list_and_skip_stride(coor, oracle):
    rng = np.random.default_rng(2)
    trajs = [rng.normal(size=(n, 3)) for n in (50, 1, 333)]
    C = rng.normal(size=(9, 3))
    d = coor.assign_to_centers(trajs, C, skip=3, stride=2)
    assert [len(x) for x in d] == [len(t[3::2]) for t in trajs]
    for x, t in zip(d, trajs):
        np.testing.assert_array_equal(x, oracle.assign(t[3::2], C))


@pytest.mark.parametrize("metric", ["euclidean", "minRMSD"])
def test_assign_split_across_batches(oracle, metric):
    # a 1,000-frame batch budget splits trajectories across batches
    from pyemma_gb300.coordinates import _device
    rng = np.random.default_rng(9)
    d = 12
    trajs = [rng.normal(size=(n, d)).astype(np.float32) for n in (0, 1, 2500, 999, 1001, 3)]
    C = rng.normal(size=(17, d)).astype(np.float32)
    for prec in (["fp32", "fp16"] if metric == "euclidean" else ["fp32"]):
        labels, stats = _device.assign_trajs(trajs, C, precision=prec, batch_bytes=4 * d * 1000, metric=metric)
        assert stats["n_frames"] == sum(len(t) for t in trajs)
        for got, t in zip(labels, trajs):
            want = oracle.assign_minrmsd(t, C) if metric == "minRMSD" else oracle.assign(t, C)
            np.testing.assert_array_equal(got, want)


def test_centers_from_file(coor, tmp_path, oracle):
    rng = np.random.default_rng(3)
    C = rng.normal(size=(6, 4)).astype(np.float32)
    X = rng.normal(size=(200, 4))
    p = str(tmp_path / "c.npy")
    np.save(p, C)
    np.testing.assert_array_equal(coor.assign_to_centers(X, p)[0], oracle.assign(X, C))


def test_kmeans_dtraj_and_save(coor, tmp_path):
    rng = np.random.default_rng(4)
    data = [rng.random((30, 100)), rng.random((37, 100))]
    km = coor.cluster_kmeans(data=data, k=5, max_iter=100)
    assert km.dtrajs[0].dtype == km.output_type()
    km.save_dtrajs(trajfiles=None, prefix="test", output_dir=str(tmp_path), extension=".dtraj")
    for i in range(2):
        os.stat(os.path.join(str(tmp_path), "test_%i.dtraj" % i))


def test_cluster_contract(coor):
    # test_cluster.py:36-163 for the kmeans estimator.
    rng = np.random.default_rng(5)
    means = [(-3, 0), (-1, 1), (0, 0), (1, -1), (4, 2)]
    X = np.zeros((5000, 2))
    for i, m in enumerate(means):
        X[i * 1000:(i + 1) * 1000, 0] = 0.3 * rng.normal() + m[0]
        X[i * 1000:(i + 1) * 1000, 1] = 2.0 * rng.normal() + m[1]
    for km in (coor.cluster_kmeans(data=X, k=100), coor.KmeansClustering(n_clusters=100).estimate(X)):
        assert isinstance(km.chunksize, (int, type(None)))
        assert km.clustercenters.shape == (km.n_clusters, 2)
        assert km.dimension() == 1
        assert len(km.dtrajs) == 1 and len(km.dtrajs[0]) == 5000
        out = km.get_output()
        assert out[0].shape == (5000, 1)
        np.testing.assert_array_equal(km.transform(X), out[0])
        assert km.n_frames_total() == 5000 and km.number_of_trajectories() == 1
        assert isinstance(km.describe(), str)
        assert km.output_type() == np.int32()


def test_kmeans_matches_oracle_end_to_end(coor, oracle):
    from pyemma_gb300 import datasets
    X = datasets.small_mixture(seed=1)
    km = coor.cluster_kmeans(X, k=50, max_iter=100, tolerance=1e-5, fixed_seed=42)
    C0, _ = oracle.kmpp(X, 50, 42)
    ref = oracle.lloyd(X, C0, 100, 1e-5)
    assert km.converged == ref["converged"] and km.n_iter == ref["n_iter"]
    np.testing.assert_allclose(km.clustercenters, ref["centers"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(km.inertias, ref["inertias"], rtol=1e-6)
    np.testing.assert_array_equal(km.dtrajs[0], oracle.assign(X, km.clustercenters))


def test_kmeans_equilibrium_and_outlier(coor):
    X = np.array([[1, 1, 1], [1, 1, -1], [1, -1, -1], [-1, -1, -1], [-1, 1, 1], [-1, -1, 1], [-1, 1, -1],
                  [1, -1, 1]], dtype=np.float32)
    km = coor.cluster_kmeans(X, k=1)
    np.testing.assert_equal(km.clustercenters.squeeze(), np.zeros(3))
    X2 = X.copy()
    X2[0, 1] = 1.5
    km2 = coor.cluster_kmeans(X2, k=2, clustercenters=np.array([[2, 0, 0], [-2, 0, 0]]), max_iter=500, n_jobs=1)
    assert np.all(np.abs(km2.clustercenters) <= 1)


def test_kmeans_seeds_and_resume(coor):
    rng = np.random.default_rng(42)
    X = np.hstack([rng.normal(size=200) - 2.0, rng.normal(size=200), rng.normal(size=200) + 2.0])
    for strategy in ("uniform", "kmeans++"):
        for seed in (True, 463498):
            km1 = coor.cluster_kmeans(X, k=50, init_strategy=strategy, fixed_seed=seed, n_jobs=1)
            km2 = coor.cluster_kmeans(X, k=50, init_strategy=strategy, fixed_seed=seed, n_jobs=1)
            assert len(km1.clustercenters) == 50 and km1.fixed_seed == km2.fixed_seed
            np.testing.assert_equal(km1.initial_centers_, km2.initial_centers_)
            while not km1.converged:
                km1.estimate(X=X, clustercenters=km1.clustercenters, keep_data=True)
            while not km2.converged:
                km2.estimate(X=X, clustercenters=km2.clustercenters, keep_data=True)
            np.testing.assert_allclose(km1.clustercenters, km2.clustercenters, atol=1e-6)
            cc = km1.clustercenters
            assert np.all(np.isfinite(cc)) and np.any((cc > -1.0) & (cc < 1.0))


def test_kmeans_memory_freed_and_kept(coor):
    rng = np.random.default_rng(32)
    X = np.hstack([rng.normal(size=1000) - 2.0, rng.normal(size=1000), rng.normal(size=1000) + 2.0])
    init = np.atleast_2d(X[rng.choice(1000, size=3)]).T
    cl = coor.cluster_kmeans(X, clustercenters=init, k=3, max_iter=1, keep_data=True)
    cl.estimate(X, clustercenters=cl.clustercenters, max_iter=1)
    assert not cl.converged
    assert hasattr(cl, "_in_memory_chunks")
    while not cl.converged:
        cl.estimate(X, clustercenters=cl.clustercenters, max_iter=5)
    assert not hasattr(cl, "_in_memory_chunks")
    # resume reduces the error (test_kmeans.py:357-374)
    cl = coor.cluster_kmeans(X, clustercenters=np.array([[20, 42, -29]]).T, max_iter=1, k=3, keep_data=True)
    resume = cl.clustercenters
    cl.estimate(X, clustercenters=resume, max_iter=50)
    true = np.array([-2, 0, 2])
    assert np.linalg.norm(true - np.sort(cl.clustercenters.ravel())) < np.linalg.norm(true - np.sort(resume.ravel()))


def test_kmeans_inefficient_resume_warns(coor, caplog):
    rng = np.random.default_rng(33)
    X = rng.normal(size=(3000, 1))
    cl = coor.cluster_kmeans(X, k=3, max_iter=1, keep_data=False)
    with caplog.at_level("WARNING"):
        cl.estimate(X, max_iter=1, clustercenters=cl.clustercenters)
    assert any("inefficient" in r.getMessage() for r in caplog.records)


def test_kmeans_trivial_blocks(coor):
    X = np.zeros((40000, 4))
    for b, v in enumerate((30.0, 60.0, 90.0, 120.0)):
        X[b * 10000:(b + 1) * 10000] = v
    cl = coor.cluster_kmeans(X, k=4)
    found = [False] * 4
    for center in cl.clustercenters:
        for i, e in enumerate((30.0, 60.0, 90.0, 120.0)):
            if np.all(center == e):
                found[i] = True
    assert all(found)


def test_kmeans_skip_and_default_k(coor):
    cl = coor.cluster_kmeans(np.random.rand(100, 3), skip=42)
    assert len(cl.dtrajs[0]) == 100 - 42
    assert cl.n_clusters == int(np.sqrt(58))


def test_kmeans_precisions_agree(coor):
    from pyemma_gb300 import datasets
    X = datasets.gaussian_mixture(30000, 128, 40, 0.3, 5.0, seed=8)
    a = coor.cluster_kmeans(X, k=20, max_iter=20, fixed_seed=3, precision="fp32")
    b = coor.cluster_kmeans(X, k=20, max_iter=20, fixed_seed=3, precision="fp16")
    assert a.n_iter == b.n_iter
    np.testing.assert_allclose(a.clustercenters, b.clustercenters, rtol=1e-5, atol=1e-6)
    np.testing.assert_array_equal(a.dtrajs[0], b.dtrajs[0])
