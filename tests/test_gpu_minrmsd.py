"""GPU parity of the minRMSD metric (km_*_minrmsd) against the CPU oracle.

The kernels and the oracle follow the same order of operations (centering in
a 32-lane order, float fused multiply-adds for the correlation sums, the QCP
quartic in double without contraction), so the bars are:
  * labels, kmeans++ frames and metric values: equal bit for bit;
  * Lloyd runs: the same iteration count and labels, centers within 1e-5 and
    inertias within 1e-6 relative (float64 atomics add in a varying order).
"""
import ctypes

import numpy as np
import pytest

from test_oracle_pins import rotated_clusters

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch as _t
    return _t


@pytest.fixture(scope="module")
def L():
    from pyemma_gb300 import _lib
    _lib.load()
    return _lib


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


@pytest.mark.parametrize("n_atoms", [1, 2, 3, 15, 58, 100])
@pytest.mark.parametrize("k", [1, 5, 33, 300])
def test_assign_equals_oracle(torch, L, oracle, n_atoms, k):
    rng = np.random.default_rng(n_atoms * 1000 + k)
    n = 700
    X = rng.uniform(-5, 5, size=(n, 3 * n_atoms)).astype(np.float32)
    C = X[rng.choice(n, k, replace=False)] + 0.2 * rng.normal(size=(k, 3 * n_atoms)).astype(np.float32)
    lab, rmsd = L.assign_minrmsd(dev(torch, X), dev(torch, C), return_rmsd=True)
    want, msd = oracle.assign_minrmsd(X, C, return_msd=True)
    np.testing.assert_array_equal(lab.cpu().numpy(), want)
    np.testing.assert_array_equal(rmsd.cpu().numpy(), np.sqrt(msd).astype(np.float32))


def test_assign_ties_and_non_finite(torch, L, oracle):
    rng = np.random.default_rng(3)
    base = rng.normal(size=(20, 3 * 7)).astype(np.float32)
    C = np.concatenate([base, base, base[::-1]])  # every center three times
    r = _rot(0.7)
    moved = (base.reshape(20, 7, 3) @ r.T + 1.5).reshape(20, -1).astype(np.float32)
    X = np.concatenate([base, moved, base[:3]])
    X[-1, 4] = np.nan
    got = L.assign_minrmsd(dev(torch, X), dev(torch, C)).cpu().numpy()
    np.testing.assert_array_equal(got, oracle.assign_minrmsd(X, C))
    assert got[-1] == 0  # no finite distance: label 0


def _rot(theta):
    c, s = np.cos(theta), np.sin(theta)
    return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])


def test_rows_equal_oracle(torch, L, oracle):
    rng = np.random.default_rng(5)
    for n_atoms in (1, 4, 15, 211):
        X = rng.uniform(size=(300, 3 * n_atoms)).astype(np.float32)
        Y = rng.uniform(size=(300, 3 * n_atoms)).astype(np.float32)
        got = L.minrmsd_rows(dev(torch, X), dev(torch, Y)).cpu().numpy()
        np.testing.assert_array_equal(got, oracle.minrmsd_rows(X, Y))


@pytest.mark.parametrize("n,n_atoms,k,seed", [(1, 3, 1, 0), (500, 15, 15, 32), (3000, 10, 50, 7)])
def test_kmpp_equals_oracle(torch, L, oracle, n, n_atoms, k, seed):
    rng = np.random.RandomState(123)
    X = rng.uniform(-50, 50, size=(n, 3 * n_atoms)).astype(np.float32)
    C, idx = L.kmpp_minrmsd(dev(torch, X), k, seed)
    C_o, idx_o = oracle.kmpp_minrmsd(X, k, seed)
    np.testing.assert_array_equal(idx.cpu().numpy(), idx_o)
    np.testing.assert_array_equal(C.cpu().numpy(), C_o)


def test_lloyd_equals_oracle(torch, L, oracle):
    rng = np.random.default_rng(9)
    X = rotated_clusters(rng, n_clusters=6, n_particles=4, per_cluster=40)
    C0, _ = oracle.kmpp_minrmsd(X, 6, 3)
    C = dev(torch, C0)
    # tolerance 1e-5 (the reference's default): the float64 atomics of the
    # center sums can move a center by one float32 ulp between otherwise equal
    # iterations, which a tolerance near 0 would see as change
    res = L.lloyd_minrmsd(dev(torch, X), C, 20, 1e-5)
    ref = oracle.lloyd_minrmsd(X, C0, 20, 1e-5)
    assert res["n_iter"] == ref["n_iter"] and res["converged"] == ref["converged"]
    np.testing.assert_array_equal(res["labels"].cpu().numpy(), ref["labels"])
    np.testing.assert_allclose(C.cpu().numpy(), ref["centers"], rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(res["inertias"], ref["inertias"], rtol=1e-6)


def test_bad_dimension_rejected(L):
    lib = L.load()
    n = 10
    rc = lib.km_assign_minrmsd(ctypes.c_void_p(16), n, 4, ctypes.c_void_p(16), 2, ctypes.c_void_p(16), None,
                               None, 0, None)
    assert rc == L.KM_ERR_BAD_SHAPE
    assert b"divisible by 3" in lib.km_last_error()


def test_api_kmeans_rotated_clusters(torch, oracle):
    # test_kmeans.py:267-316 through the public API: every cluster of rotated
    # and translated copies ends with one label, and dtrajs equal the oracle's
    # assignment to the final centers.
    from pyemma_gb300 import coordinates as coor
    rng = np.random.default_rng(12)
    X = rotated_clusters(rng, n_clusters=5, n_particles=3, per_cluster=25)
    km = coor.cluster_kmeans(X, k=5, metric="minRMSD", max_iter=0, fixed_seed=11)
    km2 = coor.cluster_kmeans(X, k=5, metric="minRMSD", max_iter=0, fixed_seed=11)
    np.testing.assert_array_equal(km.dtrajs[0], km2.dtrajs[0])
    np.testing.assert_array_equal(km.clustercenters, km2.clustercenters)
    assert km.metric == "minRMSD"
    np.testing.assert_array_equal(km.dtrajs[0], oracle.assign_minrmsd(X, km.clustercenters))
    for i in range(5):
        assert len(np.unique(km.dtrajs[0][25 * i:25 * (i + 1)])) == 1
    km3 = coor.cluster_kmeans(X, k=5, metric="minRMSD", max_iter=30, fixed_seed=11)
    ref = oracle.lloyd_minrmsd(X, oracle.kmpp_minrmsd(X, 5, 11)[0], 30, 1e-5)
    assert km3.n_iter == ref["n_iter"]
    np.testing.assert_allclose(km3.clustercenters, ref["centers"], rtol=1e-5, atol=1e-5)


def test_api_assign_to_centers_minrmsd(torch, oracle):
    # test_assign.py:241-274: assignment with the metric, every center used.
    from pyemma_gb300 import coordinates as coor
    rng = np.random.default_rng(13)
    trajs = [rotated_clusters(rng, n_clusters=3, n_particles=5, per_cluster=30) for _ in range(3)]
    centers = np.concatenate([t[[0, 30, 60]] for t in trajs])  # 9 centers
    dtrajs = coor.assign_to_centers(trajs, centers=centers, metric="minRMSD", return_dtrajs=True)
    for t, d in zip(trajs, dtrajs):
        np.testing.assert_array_equal(d, oracle.assign_minrmsd(t, centers))
    assert len(np.unique(np.concatenate(dtrajs))) >= 3
    one = coor.assign_to_centers(trajs, centers=centers, metric="minRMSD", n_jobs=1)
    two = coor.assign_to_centers(trajs, centers=centers, metric="minRMSD", n_jobs=2)
    for a, b in zip(one, two):
        np.testing.assert_array_equal(a, b)
