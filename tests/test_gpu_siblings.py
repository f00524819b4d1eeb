"""Sibling estimators on the same kernels: regular space, uniform time and
mini-batch k-means (pyemma/coordinates/clustering/regspace.py,
uniform_time.py, kmeans.py:340-447; tests modelled on the reference's
clustering/tests/test_regspace.py, test_uniform_time.py and
test_mini_batch_kmeans.py)."""
import itertools
import warnings

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,d,dmin", [(1000, 3, 0.3), (150000, 3, 0.05), (20000, 10, 1.5), (5000, 64, 9.0)])
def test_regspace_centers_match_oracle(oracle, n, d, dmin):
    import torch
    from pyemma_gb300 import _lib as L
    L.load()
    rng = np.random.default_rng(n + d)
    X = rng.random((n, d)).astype(np.float32) if d <= 3 else rng.normal(size=(n, d)).astype(np.float32)
    C_ref, conv_ref = oracle.regspace(X, dmin, 100000)
    C, conv = L.regspace(torch.from_numpy(X).cuda(), dmin, 100000)
    np.testing.assert_array_equal(C.cpu().numpy(), C_ref)
    assert conv == conv_ref
    assert len(C_ref) > 1


def test_regspace_max_centers(oracle):
    import torch
    from pyemma_gb300 import _lib as L
    rng = np.random.default_rng(3)
    X = rng.random((70000, 3)).astype(np.float32)
    C, conv = L.regspace(torch.from_numpy(X).cuda(), 1e-8, 50)
    C_ref, conv_ref = oracle.regspace(X, 1e-8, 50)
    assert not conv and not conv_ref
    np.testing.assert_array_equal(C.cpu().numpy(), C_ref)
    assert len(C_ref) == 50


def test_cluster_regspace_api(oracle):
    from pyemma_gb300.coordinates import cluster_regspace
    rng = np.random.default_rng(4)
    X = rng.random((1000, 3)).astype(np.float32)
    cl = cluster_regspace(X, dmin=0.3)
    for a, b in itertools.combinations(cl.clustercenters, 2):
        assert np.linalg.norm(a - b) >= 0.3
    dtraj = cl.dtrajs[0]
    assert dtraj.dtype == np.int32
    np.testing.assert_array_equal(dtraj, oracle.assign(X, cl.clustercenters))
    assert len(np.unique(dtraj)) == len(cl.clustercenters)
    # too small dmin: one warning, max_centers centers, the output still assigns
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        cl2 = cluster_regspace(X, dmin=1e-8, max_centers=50)
    assert len([x for x in w if "Maximum number of cluster centers" in str(x.message)]) == 1
    assert len(cl2.clustercenters) == 50 and not cl2.converged
    out = cl2.get_output()
    assert len(out) == 1 and len(out[0]) == 1000
    # 1-D data
    cluster_regspace(rng.random(100), dmin=0.3)


def test_uniform_time_centers(oracle):
    from pyemma_gb300.coordinates import cluster_uniform_time
    rng = np.random.default_rng(5)
    trajs = [rng.random((300, 3)).astype(np.float32), rng.random((200, 3)).astype(np.float32)]
    for k, skip in ((2, 0), (7, 0), (151, 0), (5, 20)):
        c = cluster_uniform_time(trajs, k=k, skip=skip)
        T = sum(len(t) - skip for t in trajs)
        next_t = (T // k) // 2
        pos = np.arange(next_t, T - next_t + 1, (T - 2 * next_t + 1) // k)[:k]
        flat = np.concatenate([t[skip:] for t in trajs])
        np.testing.assert_array_equal(c.clustercenters, flat[pos])
        for X, dt in zip(trajs, c.dtrajs):
            np.testing.assert_array_equal(dt, oracle.assign(X[skip:], c.clustercenters))
    c1 = cluster_uniform_time(rng.random(1000), k=2)
    assert c1.clustercenters.shape == (2, 1)


def test_mini_batch_kmeans(oracle):
    from pyemma_gb300.coordinates import cluster_mini_batch_kmeans
    np.random.seed(7)
    rng = np.random.default_rng(7)
    means = np.array([-10.0, 0.0, 10.0])
    X = np.concatenate([m + 0.5 * rng.normal(size=20000) for m in means]).astype(np.float32)
    cl = cluster_mini_batch_kmeans(X, k=3, max_iter=20, batch_size=0.2)
    centers = np.sort(cl.clustercenters[:, 0])
    np.testing.assert_allclose(centers, means, atol=0.2)
    assert len(cl.inertias) == cl.n_iter >= 1
    np.testing.assert_array_equal(cl.dtrajs[0], oracle.assign(X[:, None], cl.clustercenters))
    # multiple trajectories, resume from given centers
    trajs = [X[:30000, None], X[30000:, None]]
    cl2 = cluster_mini_batch_kmeans(trajs, k=3, max_iter=5, clustercenters=cl.clustercenters)
    np.testing.assert_allclose(np.sort(cl2.clustercenters[:, 0]), means, atol=0.2)
    with pytest.raises(ValueError):
        cluster_mini_batch_kmeans(X, k=3, batch_size=1.5)


def _regspace_minrmsd_data():
    from test_oracle_pins import rotated_clusters
    rng = np.random.default_rng(22)
    return np.concatenate([rotated_clusters(rng, n_clusters=4, n_particles=4, per_cluster=30),
                           rng.uniform(-2, 2, size=(60, 12)).astype(np.float32)])


@pytest.mark.parametrize("dmin,max_centers", [(0.9, 1000), (0.5, 1000), (0.5, 7)])
def test_regspace_minrmsd_equals_oracle(oracle, dmin, max_centers):
    # test_regspace.py:107-115,137-141: regular space under minRMSD, centers
    # equal to the oracle's sequential walk, dtrajs to its assignment
    from pyemma_gb300.coordinates import cluster_regspace
    X = _regspace_minrmsd_data()
    want, conv = oracle.regspace_minrmsd(X, dmin, max_centers)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        cl = cluster_regspace(X, dmin=dmin, max_centers=max_centers, metric="minRMSD")
    np.testing.assert_array_equal(cl.clustercenters, want)
    assert cl.converged == conv
    np.testing.assert_array_equal(cl.dtrajs[0], oracle.assign_minrmsd(X, want))


def test_regspace_minrmsd_block_boundaries_and_one_atom(oracle):
    import torch
    from pyemma_gb300.coordinates import cluster_regspace
    from pyemma_gb300.coordinates.clustering.regspace import minrmsd_leader_walk
    X = _regspace_minrmsd_data()
    Xd = torch.from_numpy(X).cuda()
    for block in (1, 7, 100):
        idx, done = minrmsd_leader_walk(Xd, 0.5, 1000, block=block)
        np.testing.assert_array_equal(X[idx], oracle.regspace_minrmsd(X, 0.5, 1000)[0])
        assert done
    # the reference test's data: single atoms are all at distance 0 after centering
    one = np.random.default_rng(3).uniform(-2, 2, size=(1000, 3)).astype(np.float32)
    cl = cluster_regspace(one, dmin=2.0, metric="minRMSD")
    assert len(cl.clustercenters) == 1
    assert (cl.assign(np.random.default_rng(4).random((1000, 3)).astype(np.float32), stride=1) == 0).all()


def test_regspace_minrmsd_through_deeptime_names(oracle):
    from pyemma_gb300 import deeptime_clustering as dc
    X = _regspace_minrmsd_data()
    est = dc.RegularSpace(dmin=0.5, max_centers=1000, metric="minRMSD")
    for a in range(0, len(X), 70):
        est.partial_fit(X[a:a + 70])
    np.testing.assert_array_equal(est.fetch_model().cluster_centers, oracle.regspace_minrmsd(X, 0.5, 1000)[0])
