"""Atom-pair distance features on the device (km_pair_distances) and
clustering of device-resident features."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _chain(rng, T, n_atoms=33):
    steps = rng.normal(size=(n_atoms - 1, 3))
    steps *= 0.38 / np.linalg.norm(steps, axis=1, keepdims=True)
    base = np.concatenate([np.zeros((1, 3)), np.cumsum(steps, axis=0)])
    return (base[None] + 0.05 * rng.normal(size=(T, n_atoms, 3))).astype(np.float32)


def test_pair_order_matches_featurizer_pairs():
    from pyemma_gb300.featurize import ca_pairs
    # Featurizer.pairs (featurizer.py:198-235) for residues 0..n-1
    for n, excl in ((33, 0), (33, 2), (7, 1), (3, 5)):
        ref = [[i, j] for i in range(n) for j in range(i + 1, n) if j > i + excl]
        assert ca_pairs(n, excl).tolist() == ref


@pytest.mark.parametrize("excl", [0, 2])
def test_ca_distances_match_oracle(oracle, excl):
    from pyemma_gb300.featurize import ca_distances, ca_pairs
    rng = np.random.default_rng(excl)
    xyz = _chain(rng, 5000)
    F = ca_distances(xyz, excluded_neighbors=excl)
    np.testing.assert_array_equal(F.cpu().numpy(), oracle.pair_distances(xyz, ca_pairs(33, excl)))
    # explicit pairs, including repeated and reversed ones
    pairs = np.array([[0, 32], [32, 0], [5, 6], [5, 6], [10, 3]])
    F2 = ca_distances(xyz, pairs=pairs)
    np.testing.assert_array_equal(F2.cpu().numpy(), oracle.pair_distances(xyz, pairs))


def test_cluster_device_features_equals_host(oracle):
    from pyemma_gb300.coordinates import cluster_kmeans, assign_to_centers
    from pyemma_gb300.featurize import ca_distances
    rng = np.random.default_rng(9)
    xyz = _chain(rng, 20000)
    F = ca_distances(xyz, excluded_neighbors=0)  # (20000, 528) on the device
    Fh = F.cpu().numpy()
    a = cluster_kmeans(F, k=40, max_iter=5, fixed_seed=3)
    b = cluster_kmeans(Fh, k=40, max_iter=5, fixed_seed=3)
    # same kmeans++ frames and the same iterations; the float64 center sums
    # are atomic adds, so centers agree to rounding, not bit for bit
    np.testing.assert_array_equal(a.initial_centers_, b.initial_centers_)
    np.testing.assert_allclose(a.clustercenters, b.clustercenters, rtol=1e-5)
    assert (a.dtrajs[0] == b.dtrajs[0]).mean() > 0.999
    np.testing.assert_array_equal(a.dtrajs[0], oracle.assign(Fh, a.clustercenters))
    d = assign_to_centers([F[:7000], F[7000:]], centers=a.clustercenters)
    np.testing.assert_array_equal(np.concatenate(d), a.dtrajs[0])
