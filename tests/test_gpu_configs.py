"""GPU parity at the sizes of the measured workloads, against the CPU oracle.

The small-case parity tests live in test_gpu_parity.py; these run the
workloads that bench.py measures, at their full sizes where the oracle
finishes in seconds, and through a sample or a float64 reference where it
does not.  Bars (as in test_gpu_parity.py):

  * labels bit-exact against the oracle (float32 distances in feature order,
    lowest index on ties) -- every precision, after the exact re-check;
  * one Lloyd iteration: centers within 1e-5 relative (1e-5 absolute for
    elements near zero) of the oracle's, inertia within 1e-6 relative;
  * centers after an iteration at 2,000,000 x 528 against the float64 NumPy
    member means of the same labels: within 1e-5 relative; the inertia
    against the float64 inertia of those labels and means: within 1e-6.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL_CENTERS = 1e-5
ATOL_CENTERS = 1e-5
RTOL_INERTIA = 1e-6
SEED = 2026  # the seed bench.py draws its workloads with


@pytest.fixture(scope="module")
def torch():
    import torch as _t
    return _t


@pytest.fixture(scope="module")
def L():
    from pyemma_gb300 import _lib
    _lib.load()
    return _lib


# ---------------------------------------------------------------------------
# 20 uneven AR(1) trajectories, d=10, k=1000 (4.28M frames, packed)
# ---------------------------------------------------------------------------
def test_c2_full_batch_assign_and_lloyd_iteration_vs_oracle(torch, L, oracle):
    from pyemma_gb300 import datasets
    trajs = datasets.metastable_trajectories(n_traj=20, d=10, seed=SEED)
    X = np.concatenate(trajs)
    n = len(X)
    assert n > 3_000_000
    offsets = np.concatenate([[0], np.cumsum([len(t) for t in trajs])]).astype(np.int64)
    rng = np.random.default_rng(SEED)
    C0 = X[rng.choice(n, 1000, replace=False)].copy()
    Xd = torch.from_numpy(X).cuda()
    Cd = torch.from_numpy(C0).cuda()
    want = oracle.assign(X, C0)
    for prec in ("auto", "fp16", "fp32"):
        lab, _ = L.batch_assign(Xd, offsets, Cd, precision=prec)
        np.testing.assert_array_equal(lab.cpu().numpy(), want, err_msg=prec)
    ref = oracle.lloyd(X, C0, 1, -1.0)
    np.testing.assert_array_equal(ref["labels"], want)
    for prec in ("auto", "fp32"):
        C = Cd.clone()
        r = L.lloyd(Xd, C, 1, -1.0, precision=prec)
        np.testing.assert_array_equal(r["labels"].cpu().numpy(), want, err_msg=prec)
        # atol as in the other Lloyd tests: an element near zero (C2's means
        # straddle 0) has no meaningful relative error
        np.testing.assert_allclose(C.cpu().numpy(), ref["centers"], rtol=RTOL_CENTERS, atol=ATOL_CENTERS,
                                   err_msg=prec)
        np.testing.assert_allclose(r["inertias"], ref["inertias"], rtol=RTOL_INERTIA, err_msg=prec)


# ---------------------------------------------------------------------------
# 2,000,000 x 528 C-alpha distances, k=2000
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def c3(torch):
    from pyemma_gb300 import datasets
    X = datasets.calpha_distances(2_000_000, seed=SEED, device="cuda")
    rng = np.random.default_rng(SEED)
    C0 = X[torch.from_numpy(rng.choice(X.shape[0], 2000, replace=False)).cuda()].contiguous()
    yield X, C0
    del X, C0
    torch.cuda.empty_cache()


def test_c3_labels_equal_fp32_kernel_and_oracle_on_200k(torch, L, oracle, c3):
    X, C = c3
    lab32, _ = L.assign(X, C, precision="fp32")
    lab16, stats = L.assign(X, C, precision="fp16")
    assert torch.equal(lab32, lab16)
    assert stats["n_recheck"] > 0  # the exact re-check did run
    rng = np.random.default_rng(SEED + 1)
    sample = np.sort(rng.choice(X.shape[0], 200_000, replace=False))
    Xs = X[torch.from_numpy(sample).cuda()].cpu().numpy()
    np.testing.assert_array_equal(lab16.cpu().numpy()[sample], oracle.assign(Xs, C.cpu().numpy()))


def test_c3_lloyd_centers_and_inertia_vs_fp64_reference(torch, L, oracle, c3):
    X, C0 = c3
    C = C0.clone()
    L.lloyd(X, C, 3, -1.0, precision="fp16")
    C_prev = C.clone()
    r = L.lloyd(X, C, 1, -1.0, precision="fp16")
    labels = r["labels"]
    lab32, _ = L.assign(X, C_prev, precision="fp32")
    assert torch.equal(labels, lab32)
    Xh = X.cpu().numpy()
    lab = labels.cpu().numpy()
    mu, cnt = oracle.centers_fp64(Xh, lab, C_prev.cpu().numpy())
    got = C.cpu().numpy().astype(np.float64)
    rel = np.abs(got - mu) / np.maximum(np.abs(mu), 1e-30)
    assert rel.max() <= RTOL_CENTERS, rel.max()
    inertia = oracle.inertia_fp64(Xh, lab, mu)
    assert abs(r["inertias"][0] - inertia) <= RTOL_INERTIA * inertia


def test_c3_kmpp_draws_equal_oracle_on_500k(torch, L, oracle):
    # kmeans++ on 500,000 C-alpha distance frames (d = 528): the pruned
    # device pass must draw the oracle's frames in every round.
    from pyemma_gb300 import datasets
    X = datasets.calpha_distances(500_000, seed=SEED)
    k = 300
    _, idx_ref = oracle.kmpp(X, k, 42)
    C0, idx = L.kmpp(torch.from_numpy(X).cuda(), k, 42)
    np.testing.assert_array_equal(idx.cpu().numpy(), idx_ref)
    np.testing.assert_array_equal(C0.cpu().numpy(), X[idx_ref])


# ---------------------------------------------------------------------------
# precision sweep: 1M frames, 4k Gaussian clusters, d x k grid
# ---------------------------------------------------------------------------
def _sweep_data(torch, d, k, n=1_000_000):
    # The bench's generator for this grid (seeded on the device).
    g = torch.Generator(device="cuda")
    g.manual_seed(SEED + 31 * d + k)
    means = torch.rand((4 * k, d), device="cuda", generator=g) * 10.0 - 5.0
    comp = torch.randint(0, 4 * k, (n,), device="cuda", generator=g)
    X = (means[comp] + 0.3 * torch.randn((n, d), device="cuda", generator=g)).contiguous()
    del means, comp
    C0 = X[torch.randperm(n, device="cuda", generator=g)[:k]].contiguous()
    return X, C0


@pytest.mark.parametrize("k", [100, 1000, 5000])
@pytest.mark.parametrize("d", [16, 64, 256, 1024])
def test_c4_grid_tensor_core_labels_equal_fp32_and_oracle(torch, L, oracle, d, k):
    X, C = _sweep_data(torch, d, k)
    lab32, _ = L.assign(X, C, precision="fp32")
    for prec in ("fp16", "bf16", "fp8"):
        lab, _ = L.assign(X, C, precision=prec)
        assert torch.equal(lab, lab32), prec
    rng = np.random.default_rng(SEED + d + k)
    sample = np.sort(rng.choice(X.shape[0], 20_000, replace=False))
    Xs = X[torch.from_numpy(sample).cuda()].cpu().numpy()
    np.testing.assert_array_equal(lab32.cpu().numpy()[sample], oracle.assign(Xs, C.cpu().numpy()))
    del X, C, lab32
    torch.cuda.empty_cache()
