"""Lag-tau transition counts (km_count_matrix) against the oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("sliding", [True, False])
@pytest.mark.parametrize("lag", [1, 3, 50])
def test_count_matrix_matches_oracle(oracle, sliding, lag):
    from pyemma_gb300.msm import count_matrix
    rng = np.random.default_rng(lag + 100 * sliding)
    dtrajs = []
    for T in (1000, 1, 49, 50, 51, 123457, 0, 7777):
        d = rng.integers(-1, 40, size=T).astype(np.int32)
        # metastable runs: long stretches of one state
        if T > 10000:
            d[1000:60000] = 7
        dtrajs.append(d)
    C = count_matrix(dtrajs, lag, sliding=sliding, sparse=False)
    np.testing.assert_array_equal(C, oracle.count_matrix(dtrajs, lag, sliding=sliding))
    Cs = count_matrix(dtrajs, lag, sliding=sliding, nstates=60)
    assert Cs.shape == (60, 60)
    np.testing.assert_array_equal(Cs.toarray(), oracle.count_matrix(dtrajs, lag, sliding=sliding, nstates=60))


def test_counts_after_clustering(oracle):
    from pyemma_gb300.coordinates import cluster_kmeans
    from pyemma_gb300.msm import count_matrix
    from pyemma_gb300 import datasets
    trajs = datasets.metastable_trajectories(n_traj=3, d=10, lmin=20000, lmax=40000, seed=4)
    cl = cluster_kmeans(trajs, k=50, max_iter=5, fixed_seed=1)
    C = count_matrix(cl.dtrajs, 10, sparse=False)
    np.testing.assert_array_equal(C, oracle.count_matrix(cl.dtrajs, 10, nstates=C.shape[0]))
    assert C.sum() == sum(len(t) - 10 for t in trajs)
