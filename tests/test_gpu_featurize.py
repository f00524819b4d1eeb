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


# ---------------------------------------------------------------------------
# The featurization fused into the discretization: coordinate frames whose
# pair distances are computed where the kernels read them (km_assign_pairs,
# km_lloyd_pairs, km_kmpp_pairs), against the same calls on the features
# km_pair_distances writes.
# ---------------------------------------------------------------------------
def _frames(torch, rng, T, excl=0, conf=6):
    # a few chain conformations with jitter, so that clusters and near-ties exist
    xyz = np.concatenate([_chain(rng, T // conf + 1) for _ in range(conf)])[:T]
    xyz = xyz[rng.permutation(len(xyz))]
    from pyemma_gb300.featurize import pair_distance_frames
    return pair_distance_frames(xyz, excluded_neighbors=excl)


@pytest.mark.parametrize("prec", ["fp32", "fp16", "bf16"])
@pytest.mark.parametrize("excl", [0, 2])
def test_assign_pairs_equals_assign_on_features(oracle, prec, excl):
    import torch
    from pyemma_gb300 import _lib as L
    rng = np.random.default_rng(40 + excl)
    src = _frames(torch, rng, 30000, excl)
    F = src.features()
    C = F[torch.from_numpy(rng.choice(len(F), 300, replace=False)).cuda()].contiguous()
    want, _ = L.assign(F, C, precision=prec)
    got, stats = L.assign_pairs(src.xyz, src.pairs, C, precision=prec)
    assert torch.equal(got, want)
    sample = rng.choice(len(F), 3000, replace=False)
    np.testing.assert_array_equal(got.cpu().numpy()[sample], oracle.assign(F.cpu().numpy()[sample], C.cpu().numpy()))


@pytest.mark.parametrize("prec", ["fp32", "fp16"])
def test_lloyd_pairs_equals_lloyd_on_features(prec):
    import torch
    from pyemma_gb300 import _lib as L
    rng = np.random.default_rng(51)
    src = _frames(torch, rng, 40000, 0)
    F = src.features()
    C0 = F[torch.from_numpy(rng.choice(len(F), 200, replace=False)).cuda()].contiguous()
    Ca, Cb = C0.clone(), C0.clone()
    ra = L.lloyd_pairs(src.xyz, src.pairs, Ca, 8, 1e-6, precision=prec)
    rb = L.lloyd(F, Cb, 8, 1e-6, precision=prec)
    assert ra["n_iter"] == rb["n_iter"] and ra["converged"] == rb["converged"]
    # the float64 centroid sums add in a different order (segment kernels)
    torch.testing.assert_close(Ca, Cb, rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(ra["inertias"], rb["inertias"], rtol=1e-6)
    assert (ra["labels"] == rb["labels"]).float().mean().item() > 0.9999
    # one iteration from the same centers: labels equal
    Ca, Cb = C0.clone(), C0.clone()
    ra = L.lloyd_pairs(src.xyz, src.pairs, Ca, 1, -1.0, precision=prec)
    rb = L.lloyd(F, Cb, 1, -1.0, precision=prec)
    assert torch.equal(ra["labels"], rb["labels"])


@pytest.mark.parametrize("n_atoms,excl", [(50, 0), (130, 120), (12, 0)])
def test_lloyd_pairs_other_shapes_equal_lloyd_on_features(n_atoms, excl):
    # 50 atoms: 1,225 features, two 1024-feature slices of the segment sums;
    # 130 atoms: beyond the ring-staged kernel's atom limit (the per-feature
    # gather kernel); 12 atoms: 66 features
    import torch
    from pyemma_gb300 import _lib as L
    from pyemma_gb300.featurize import pair_distance_frames
    rng = np.random.default_rng(60 + n_atoms)
    T = 12000
    xyz = np.concatenate([_chain(rng, T // 4 + 1, n_atoms) for _ in range(4)])[:T]
    src = pair_distance_frames(xyz[rng.permutation(T)], excluded_neighbors=excl)
    F = src.features()
    C0 = F[torch.from_numpy(rng.choice(T, 64, replace=False)).cuda()].contiguous()
    for prec in ("fp32", "fp16"):
        Ca, Cb = C0.clone(), C0.clone()
        ra = L.lloyd_pairs(src.xyz, src.pairs, Ca, 1, -1.0, precision=prec)
        rb = L.lloyd(F, Cb, 1, -1.0, precision=prec)
        assert torch.equal(ra["labels"], rb["labels"]), prec
        torch.testing.assert_close(Ca, Cb, rtol=1e-5, atol=1e-5)
        np.testing.assert_allclose(ra["inertias"], rb["inertias"], rtol=1e-6)


def test_lloyd_pairs_chunked_pass_equals_features():
    # 600,000 coordinate frames: the tensor-core pass runs in chunks, each
    # chunk's re-check computing the pair features of its listed frames
    import torch
    from pyemma_gb300 import _lib as L
    from pyemma_gb300.featurize import pair_distance_frames
    rng = np.random.default_rng(71)
    T = 600_000
    xyz = np.concatenate([_chain(rng, T // 8 + 1, 12) for _ in range(8)])[:T]
    src = pair_distance_frames(xyz[rng.permutation(T)], excluded_neighbors=0)
    F = src.features()
    C0 = F[torch.from_numpy(rng.choice(T, 256, replace=False)).cuda()].contiguous()
    Ca, Cb = C0.clone(), C0.clone()
    ra = L.lloyd_pairs(src.xyz, src.pairs, Ca, 1, -1.0, precision="fp16")
    rb = L.lloyd(F, Cb, 1, -1.0, precision="fp16")
    assert torch.equal(ra["labels"], rb["labels"])
    torch.testing.assert_close(Ca, Cb, rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(ra["inertias"], rb["inertias"], rtol=1e-6)


def test_kmpp_pairs_draws_equal_kmpp_on_features(oracle):
    import torch
    from pyemma_gb300 import _lib as L
    rng = np.random.default_rng(52)
    src = _frames(torch, rng, 25000, 2)
    F = src.features()
    for prune in ("0", "1"):
        import os
        os.environ["KM_KMPP_PRUNE"] = prune
        try:
            Ca, ia = L.kmpp_pairs(src.xyz, src.pairs, 64, 17)
            Cb, ib = L.kmpp(F, 64, 17)
        finally:
            del os.environ["KM_KMPP_PRUNE"]
        assert torch.equal(ia, ib)
        assert torch.equal(Ca, Cb)
    _, io = oracle.kmpp(F.cpu().numpy(), 64, 17)
    np.testing.assert_array_equal(ia.cpu().numpy(), io)


def test_estimators_on_pair_frames_equal_on_features():
    import torch
    from pyemma_gb300.coordinates import assign_to_centers, cluster_kmeans
    rng = np.random.default_rng(53)
    src = _frames(torch, rng, 30000, 2)
    F = src.features()
    a = cluster_kmeans(src, k=50, max_iter=6, fixed_seed=4)
    b = cluster_kmeans(F, k=50, max_iter=6, fixed_seed=4)
    # a kmeans++ start keeps no initial centers on either input
    assert len(a.initial_centers_) == 0 and len(b.initial_centers_) == 0
    np.testing.assert_allclose(a.clustercenters, b.clustercenters, rtol=1e-5, atol=1e-5)
    assert a.n_iter == b.n_iter
    np.testing.assert_array_equal(a.dtrajs[0], assign_to_centers(F, centers=a.clustercenters)[0])
    np.testing.assert_array_equal(assign_to_centers(src, centers=a.clustercenters)[0],
                                  assign_to_centers(F, centers=a.clustercenters)[0])
    # stride and skip take the same frames as on the features
    c = cluster_kmeans(src, k=20, max_iter=3, fixed_seed=5, stride=3, skip=11, init_strategy="uniform")
    e = cluster_kmeans(F, k=20, max_iter=3, fixed_seed=5, stride=3, skip=11, init_strategy="uniform")
    np.testing.assert_array_equal(c.initial_centers_, e.initial_centers_)
    assert c.initial_centers_.shape == (20, F.shape[1])
    np.testing.assert_allclose(c.clustercenters, e.clustercenters, rtol=1e-5, atol=1e-5)


def test_bad_pairs_are_refused():
    import ctypes
    import torch
    from pyemma_gb300 import _lib as L
    from pyemma_gb300.featurize import PairDistanceFrames
    xyz = torch.zeros((10, 4, 3), dtype=torch.float32, device="cuda")
    with pytest.raises(ValueError):
        PairDistanceFrames(xyz, [[0, 4]])
    # through the C ABI the pair table is checked on the host before any kernel runs
    pairs = torch.tensor([[0, 1], [2, 7]], dtype=torch.int32, device="cuda")
    C = torch.zeros((2, 2), dtype=torch.float32, device="cuda")
    with pytest.raises(L.KmError) as ei:
        L.assign_pairs(xyz, pairs, C)
    assert ei.value.status == L.KM_ERR_BAD_SHAPE
    out = torch.empty((10, 2), dtype=torch.float32, device="cuda")
    rc = L.load().km_pair_distances(ctypes.c_void_p(xyz.data_ptr()), 10, 4, ctypes.c_void_p(pairs.data_ptr()), 2,
                                    ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == L.KM_ERR_BAD_SHAPE
