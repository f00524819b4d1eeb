"""GPU: Lloyd on host frames (km_lloyd_host) against Lloyd on device frames.

The host frames are copied into the device buffer chunk by chunk while the
first iteration assigns the chunks already copied.  Bars: the device copy
equals the host frames bit for bit; the labels of a one-iteration run equal
km_lloyd's; centers and inertias agree to the rounding of the float64
centroid sums (their atomics add in a varying order).
"""
import numpy as np
import pytest

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


def _parts(rng, sizes, d):
    return [rng.normal(size=(m, d)).astype(np.float32) for m in sizes]


@pytest.mark.parametrize("prec", ["fp32", "fp16", "bf16"])
@pytest.mark.parametrize("sizes", [[50000], [1], [7000, 0, 23001, 16384, 3, 40000], [16384, 16384]])
def test_host_equals_device(torch, L, prec, sizes):
    rng = np.random.default_rng(sum(sizes) + len(sizes))
    d, k = 64, 300
    parts = _parts(rng, sizes, d)
    Xh = np.concatenate(parts)
    k = min(k, len(Xh))
    C0 = Xh[rng.choice(len(Xh), k, replace=False)] + 0.01
    C0 = torch.from_numpy(C0.astype(np.float32)).cuda()
    for iters in (1, 3):
        Ca, Cb = C0.clone(), C0.clone()
        ra = L.lloyd_host(parts, Ca, iters, -1.0, precision=prec)
        assert torch.equal(ra["X"].cpu(), torch.from_numpy(Xh))
        rb = L.lloyd(torch.from_numpy(Xh).cuda(), Cb, iters, -1.0, precision=prec)
        assert ra["n_iter"] == rb["n_iter"] == iters
        if iters == 1:
            assert torch.equal(ra["labels"], rb["labels"])
        torch.testing.assert_close(Ca, Cb, rtol=1e-5, atol=1e-5)
        np.testing.assert_allclose(ra["inertias"], rb["inertias"], rtol=1e-5)


def test_host_zero_iterations_copies(torch, L):
    rng = np.random.default_rng(3)
    parts = _parts(rng, [100, 50], 8)
    C = torch.from_numpy(parts[0][:4].copy()).cuda()
    C0 = C.clone()
    r = L.lloyd_host(parts, C, 0, -1.0, precision="fp32")
    assert r["n_iter"] == 0
    assert torch.equal(r["X"].cpu(), torch.from_numpy(np.concatenate(parts)))
    assert torch.equal(C, C0)


def test_host_pinned_wide(torch, L, oracle):
    """528 features, k = 2000, 300,000 frames from pinned memory: one iteration's
    labels equal the oracle's on a sample."""
    from pyemma_gb300 import datasets
    Xd = datasets.calpha_distances(300_000, seed=5, device="cuda")
    Xp = torch.empty(Xd.shape, dtype=torch.float32, pin_memory=True)
    Xp.copy_(Xd)
    rng = np.random.default_rng(5)
    C = Xd[torch.from_numpy(rng.choice(Xd.shape[0], 2000, replace=False)).cuda()].contiguous()
    C0 = C.clone()
    r = L.lloyd_host([Xp.numpy()], C, 1, -1.0, precision="fp16")
    lab_dev, _ = L.assign(Xd, C0, precision="fp32")
    assert torch.equal(r["labels"], lab_dev)
    sample = rng.choice(Xd.shape[0], 1000, replace=False)
    np.testing.assert_array_equal(r["labels"].cpu().numpy()[sample],
                                  oracle.assign(Xp.numpy()[sample], C0.cpu().numpy()))


def test_api_host_input_matches_device_input(torch):
    from pyemma_gb300 import coordinates as coor
    rng = np.random.default_rng(11)
    trajs = [rng.normal(size=(m, 20)).astype(np.float32) + 3.0 * (i % 3) for i, m in enumerate((9000, 21000, 500))]
    init = np.concatenate(trajs)[rng.choice(30500, 40, replace=False)]
    km_h = coor.cluster_kmeans(trajs, k=40, clustercenters=init, max_iter=20, tolerance=-1.0)
    km_d = coor.cluster_kmeans([torch.from_numpy(t).cuda() for t in trajs], k=40, clustercenters=init,
                               max_iter=20, tolerance=-1.0)
    assert km_h.n_iter == km_d.n_iter == 20
    np.testing.assert_allclose(km_h.clustercenters, km_d.clustercenters, rtol=1e-5, atol=1e-5)


@pytest.mark.parametrize("d", [333, 528])
def test_host_pageable_staged_many_blocks(torch, L, d):
    # Ordinary numpy parts (pageable) are staged through page-locked buffers
    # by worker threads in 16 MiB blocks; here about 80 blocks over several
    # chunks, parts of uneven size, one of them pinned.  The device copy is
    # bit-exact and the run equals km_lloyd on the same frames.
    rng = np.random.default_rng(d)
    sizes = [250_000, 1, 130_001, 0, 220_000]
    parts = _parts(rng, sizes, d)
    pinned = torch.empty((sizes[2], d), dtype=torch.float32, pin_memory=True)
    pinned.numpy()[...] = parts[2]
    parts[2] = pinned.numpy()
    Xh = np.concatenate(parts)
    C0 = torch.from_numpy(Xh[rng.choice(len(Xh), 500, replace=False)] + 0.01).cuda()
    Ca, Cb = C0.clone(), C0.clone()
    ra = L.lloyd_host(parts, Ca, 2, -1.0, precision="fp16")
    assert torch.equal(ra["X"].cpu(), torch.from_numpy(Xh))
    rb = L.lloyd(torch.from_numpy(Xh).cuda(), Cb, 2, -1.0, precision="fp16")
    assert ra["n_iter"] == rb["n_iter"] == 2
    torch.testing.assert_close(Ca, Cb, rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(ra["inertias"], rb["inertias"], rtol=1e-5)
    r0 = L.lloyd_host(parts, C0.clone(), 0, -1.0, precision="fp16")  # copy only
    assert torch.equal(r0["X"].cpu(), torch.from_numpy(Xh))
