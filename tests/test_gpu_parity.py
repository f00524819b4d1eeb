"""GPU parity: libkmgpu (through its C ABI) against the CPU oracle.

Bars:
  * labels (assign, batch assign, the tensor-core path after its recheck):
    bit-exact against the oracle;
  * kmeans++ chosen frames: identical;
  * one centroid update: centers within 1e-6 relative (float64 sums in a
    different order may move a center by one float32 ulp), counts exact,
    inertia within 1e-6 relative (the kernel rounds each deviation x - c once
    to float32 before its compensated sums; the oracle keeps it exact in
    float64);
  * Lloyd runs: same number of iterations and convergence flag, centers
    within 1e-5 relative, inertias within 1e-6 relative.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL_CENTER_STEP = 1e-6
RTOL_COST_STEP = 1e-6
RTOL_CENTERS = 1e-5
RTOL_INERTIA = 1e-6


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


def gpu_assign(torch, L, X, C, precision):
    lab, stats = L.assign(dev(torch, X), dev(torch, C), precision=precision)
    return lab.cpu().numpy(), stats


PRECS = ["fp32", "fp16", "bf16", "fp8"]


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("case", ["assign", "wide", "tie", "blobs"])
def test_golden_labels(torch, L, golden, case, prec):
    X, C, want = golden[case + "_X"], golden[case + "_C"], golden[case + "_labels"]
    got, stats = gpu_assign(torch, L, X, C, prec)
    np.testing.assert_array_equal(got, want)
    assert stats["precision"] == prec


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("d", [1, 2, 3, 7, 10, 16, 31, 32, 33, 64, 100, 128, 200, 257, 528, 576, 640, 1024, 2050])
def test_random_shapes(torch, L, oracle, d, prec):
    rng = np.random.default_rng(1000 + d)
    for n, k in [(1, 1), (127, 5), (1000, 33), (4097, 257), (3000, 1000)]:
        X = rng.normal(size=(n, d)).astype(np.float32)
        C = (X[rng.integers(0, n, size=k)] + 0.1 * rng.normal(size=(k, d))).astype(np.float32)
        got, _ = gpu_assign(torch, L, X, C, prec)
        np.testing.assert_array_equal(got, oracle.assign(X, C), err_msg="n=%d k=%d d=%d" % (n, k, d))


@pytest.mark.parametrize("prec", PRECS)
def test_duplicate_centers_ties(torch, L, oracle, prec):
    rng = np.random.default_rng(7)
    d = 64
    base = rng.normal(size=(100, d)).astype(np.float32)
    C = np.concatenate([base, base, base[::-1]])  # every center three times
    X = np.concatenate([base, base + 0.01 * rng.normal(size=base.shape).astype(np.float32)])
    got, stats = gpu_assign(torch, L, X, C, prec)
    np.testing.assert_array_equal(got, oracle.assign(X, C))
    assert got[:100].tolist() == list(range(100))  # exact hits go to the lowest duplicate


@pytest.mark.parametrize("groups,reps", [(90, 30), (40, 0), (90, 0)])
def test_full_recheck_across_center_blocks(torch, L, oracle, groups, reps):
    # Groups of 26 nearly equal centers overflow the candidate list of the
    # tensor-core pass (at most 16 entries); the exact copies of each group sit
    # 26 * groups apart, so the exact re-check must pick the lowest index
    # across center blocks.  40 listed frames take the short-list kernel, the
    # longer lists the tiled one.
    rng = np.random.default_rng(21)
    d = 96
    base = rng.normal(size=(groups, d)).astype(np.float32)
    near = [base + 1e-4 * rng.normal(size=base.shape).astype(np.float32) for _ in range(24)]
    C = np.concatenate([base] + near + [base]).astype(np.float32)  # k = 26 * groups
    X = [base + 1e-3 * rng.normal(size=base.shape).astype(np.float32) for _ in range(reps)]
    X = np.concatenate(X + [base]).astype(np.float32)
    got, stats = gpu_assign(torch, L, X, C, "fp16")
    assert stats["n_full"] >= groups
    np.testing.assert_array_equal(got, oracle.assign(X, C))
    assert got[-groups:].tolist() == list(range(groups))


@pytest.mark.parametrize("prec", PRECS)
def test_offset_data_bound(torch, L, oracle, prec):
    # Large common offset with small spread: the stress case of the tensor-core bound.
    rng = np.random.default_rng(11)
    X = (1.0e4 + 1e-2 * rng.normal(size=(5000, 128))).astype(np.float32)
    C = X[rng.choice(5000, 300, replace=False)].copy()
    got, stats = gpu_assign(torch, L, X, C, prec)
    np.testing.assert_array_equal(got, oracle.assign(X, C))


@pytest.mark.parametrize("prec", PRECS)
def test_non_finite_frames(torch, L, oracle, prec):
    rng = np.random.default_rng(12)
    X = rng.normal(size=(300, 96)).astype(np.float32)
    X[5, 3] = np.nan
    X[17, :] = np.nan
    X[40, 0] = np.inf
    X[41, 7] = -np.inf
    C = rng.normal(size=(20, 96)).astype(np.float32)
    got, _ = gpu_assign(torch, L, X, C, prec)
    np.testing.assert_array_equal(got, oracle.assign(X, C))


def test_empty_input(torch, L):
    X = torch.empty((0, 8), dtype=torch.float32, device="cuda")
    C = torch.ones((3, 8), dtype=torch.float32, device="cuda")
    for prec in PRECS:
        lab, stats = L.assign(X, C, precision=prec)
        assert lab.numel() == 0 and stats["n_frames"] == 0


def test_bad_shapes_raise(torch, L):
    X = torch.ones((10, 4), dtype=torch.float32, device="cuda")
    with pytest.raises(ValueError):
        L.assign(X, torch.ones((3, 5), dtype=torch.float32, device="cuda"))
    with pytest.raises(L.KmError):
        L.assign(X, torch.ones((0, 4), dtype=torch.float32, device="cuda"))


@pytest.mark.parametrize("prec", PRECS)
def test_batch_assign_uneven(torch, L, oracle, prec):
    rng = np.random.default_rng(13)
    lengths = [0, 1, 1000, 37, 5000, 0, 129]
    trajs = [rng.normal(size=(t, 72)).astype(np.float32) for t in lengths]
    C = rng.normal(size=(64, 72)).astype(np.float32)
    Xp = np.concatenate(trajs)
    offsets = np.concatenate([[0], np.cumsum(lengths)])
    lab, stats = L.batch_assign(dev(torch, Xp), offsets, dev(torch, C), precision=prec)
    np.testing.assert_array_equal(lab.cpu().numpy(), oracle.assign(Xp, C))


def test_update_matches_oracle(torch, L, oracle, golden):
    X, C, lab = golden["assign_X"], golden["assign_C"], golden["assign_labels"]
    Cn, counts, cost = L.update(dev(torch, X), torch.from_numpy(lab).cuda(), dev(torch, C))
    np.testing.assert_allclose(Cn.cpu().numpy(), golden["update_C"], rtol=RTOL_CENTER_STEP, atol=0)
    np.testing.assert_array_equal(counts.cpu().numpy(), golden["update_counts"])
    assert abs(cost - golden["update_cost"][0]) <= RTOL_COST_STEP * golden["update_cost"][0]


@pytest.mark.parametrize("d", [1, 2, 10, 31, 32, 100, 528])
def test_update_shapes(torch, L, oracle, d):
    rng = np.random.default_rng(50 + d)
    n, k = 20000, 97
    X = (5.0 + rng.normal(size=(n, d))).astype(np.float32)
    C = X[:k].copy()
    C[3] = 1e6  # an empty cluster keeps its center
    lab = oracle.assign(X, C)
    Cn_ref, cnt_ref, cost_ref, _ = oracle.update(X, lab, C)
    Cn, counts, cost = L.update(dev(torch, X), torch.from_numpy(lab).cuda(), dev(torch, C))
    np.testing.assert_allclose(Cn.cpu().numpy(), Cn_ref, rtol=RTOL_CENTER_STEP, atol=0)
    np.testing.assert_array_equal(Cn.cpu().numpy()[3], C[3])
    np.testing.assert_array_equal(counts.cpu().numpy(), cnt_ref)
    assert abs(cost - cost_ref) <= RTOL_COST_STEP * cost_ref


@pytest.mark.parametrize("d,n", [(d, 30011) for d in (1, 2, 3, 4, 5, 8, 9, 16, 17)] + [(2, 1000003), (16, 1000003)])
@pytest.mark.parametrize("k_kind", ["one", "max"])
def test_update_one_pass_shapes(torch, L, oracle, d, n, k_kind):
    # d <= 16 and few centers take the one-pass shared-memory sums: "max" is
    # the largest k whose sums (k x (d + 1) doubles and k counts) fit in
    # 48 KB, "one" puts every frame in one cluster; the larger n gives each
    # thread a run of several frames.  d = 17 is the segment path.
    k = 1 if k_kind == "one" else 49152 // (8 * (d + 1) + 4)
    rng = np.random.default_rng(300 + d)
    X = (3.0 + rng.normal(size=(n, d))).astype(np.float32)
    C = (3.0 + rng.normal(size=(k, d))).astype(np.float32)
    lab = rng.integers(0, k, size=n).astype(np.int32)
    if n > 100000:
        lab[: n // 2] = np.repeat(lab[: n // 2: 7], 7)[: n // 2]  # runs of equal labels
    if k > 2:
        lab[lab == 1] = 0  # an empty cluster keeps its center
    Cn_ref, cnt_ref, cost_ref, _ = oracle.update(X, lab, C)
    Cn, counts, cost = L.update(dev(torch, X), torch.from_numpy(lab).cuda(), dev(torch, C))
    np.testing.assert_allclose(Cn.cpu().numpy(), Cn_ref, rtol=RTOL_CENTER_STEP, atol=0)
    np.testing.assert_array_equal(counts.cpu().numpy(), cnt_ref)
    if k > 2:
        np.testing.assert_array_equal(Cn.cpu().numpy()[1], C[1])
    assert abs(cost - cost_ref) <= RTOL_COST_STEP * cost_ref


def test_update_sorted_labels_long_runs(torch, L, oracle):
    # Long runs of equal labels (time-correlated trajectories) stress the run flushes.
    rng = np.random.default_rng(77)
    n, d, k = 200000, 10, 50
    lab = np.repeat(rng.integers(0, k, size=n // 5000), 5000).astype(np.int32)
    X = rng.normal(size=(n, d)).astype(np.float32)
    C = rng.normal(size=(k, d)).astype(np.float32)
    Cn_ref, cnt_ref, cost_ref, _ = oracle.update(X, lab, C)
    Cn, counts, cost = L.update(dev(torch, X), torch.from_numpy(lab).cuda(), dev(torch, C))
    np.testing.assert_allclose(Cn.cpu().numpy(), Cn_ref, rtol=RTOL_CENTER_STEP, atol=1e-7)
    np.testing.assert_array_equal(counts.cpu().numpy(), cnt_ref)
    assert abs(cost - cost_ref) <= RTOL_COST_STEP * cost_ref


def test_update_bad_label_raises(torch, L):
    X = torch.ones((10, 3), dtype=torch.float32, device="cuda")
    C = torch.zeros((2, 3), dtype=torch.float32, device="cuda")
    lab = torch.zeros(10, dtype=torch.int32, device="cuda")
    lab[4] = 2
    with pytest.raises(L.KmError) as e:
        L.update(X, lab, C)
    assert e.value.status == L.KM_ERR_BAD_LABEL


def test_kmpp_golden(torch, L, golden):
    X = golden["kmpp_X"]
    C0, idx = L.kmpp(dev(torch, X), 20, int(golden["kmpp_seed"][0]))
    np.testing.assert_array_equal(idx.cpu().numpy(), golden["kmpp_idx"])
    np.testing.assert_array_equal(C0.cpu().numpy(), X[golden["kmpp_idx"]])


@pytest.mark.parametrize("n,d,k,seed", [(1, 3, 1, 0), (5, 2, 5, 1), (3000, 2, 50, 42), (10000, 10, 200, 7),
                                        (4100, 528, 30, 3), (2049, 7, 64, 2 ** 32 - 1), (600000, 2, 20, 11),
                                        (1100001, 3, 8, 5), (20000, 33, 40, 9), (7001, 64, 25, 4)])
def test_kmpp_matches_oracle(torch, L, oracle, n, d, k, seed, kmpp_prune):
    rng = np.random.default_rng(seed % 1000)
    X = rng.normal(size=(n, d)).astype(np.float32)
    _, idx_ref = oracle.kmpp(X, k, seed)
    calls = []
    C0, idx = L.kmpp(dev(torch, X), k, seed, callback=lambda: calls.append(1))
    np.testing.assert_array_equal(idx.cpu().numpy(), idx_ref)
    assert len(calls) == k


def test_kmpp_sparse_weights_many_tiles(torch, L, oracle, kmpp_prune):
    # 700,000 frames (342 weight tiles, more than one per thread of the draw):
    # all but 30 frames equal, so after a few rounds most tiles weigh 0 and
    # the last rounds find no weight at all (uniform fallback).
    rng = np.random.default_rng(4)
    X = np.zeros((700000, 2), dtype=np.float32)
    X[rng.choice(700000, 30, replace=False)] = rng.normal(size=(30, 2)).astype(np.float32) * 10
    _, idx_ref = oracle.kmpp(X, 40, 17)
    _, idx = L.kmpp(dev(torch, X), 40, 17)
    np.testing.assert_array_equal(idx.cpu().numpy(), idx_ref)


@pytest.fixture(params=["0", "1"], ids=["unpruned", "pruned"])
def kmpp_prune(request, monkeypatch):
    # KM_KMPP_PRUNE forces the pruned (bound, list, evaluation) or the plain
    # kmeans++ round; both must draw the oracle's frames.
    monkeypatch.setenv("KM_KMPP_PRUNE", request.param)
    return request.param


@pytest.mark.parametrize("case", ["mixture", "mixture_wide", "lattice", "collinear"])
def test_kmpp_pruned_pass_matches_oracle(torch, L, oracle, case, kmpp_prune):
    # Data on which the bound ||c_new - c_a||^2 >= 4 D^2 skips most frames
    # (well separated clusters), and data with exact boundary cases: integer
    # lattice points and points on a line, where a new center often sits at
    # exactly twice a frame's distance from its nearest center, and many
    # distances tie.  The running minima and so the draws must stay the
    # oracle's, which evaluates every frame in every round.
    rng = np.random.default_rng(31)
    if case == "mixture":
        from pyemma_gb300 import datasets
        X = datasets.gaussian_mixture(200000, 16, 50, 0.3, 5.0, seed=31)
        k = 300
    elif case == "mixture_wide":
        # 100 features: the listed frames are evaluated 32 to a warp, with a
        # partial last run of features and partial groups of frames.
        from pyemma_gb300 import datasets
        X = datasets.gaussian_mixture(100000, 100, 40, 0.3, 5.0, seed=32)
        k = 150
    elif case == "lattice":
        X = rng.integers(0, 8, size=(60000, 3)).astype(np.float32)
        k = 120
    else:
        X = np.zeros((50000, 4), dtype=np.float32)
        X[:, 0] = rng.integers(-64, 65, size=50000).astype(np.float32) * 0.5
        k = 60
    _, idx_ref = oracle.kmpp(X, k, 13)
    _, idx = L.kmpp(dev(torch, X), k, 13)
    np.testing.assert_array_equal(idx.cpu().numpy(), idx_ref)


def test_kmpp_duplicates(torch, L, oracle, kmpp_prune):
    X = np.ones((100, 4), dtype=np.float32)
    X[50:] = 2.0
    _, idx_ref = oracle.kmpp(X, 6, 5)
    _, idx = L.kmpp(dev(torch, X), 6, 5)
    np.testing.assert_array_equal(idx.cpu().numpy(), idx_ref)


@pytest.mark.parametrize("prec", PRECS)
def test_lloyd_golden(torch, L, golden, prec):
    X, C0 = golden["lloyd_X"], golden["lloyd_C0"]
    C = dev(torch, C0)
    calls = []
    r = L.lloyd(dev(torch, X), C, 100, 1e-5, precision=prec if X.shape[1] >= 2 else "fp32",
                callback=lambda: calls.append(1))
    assert r["n_iter"] == golden["lloyd_n_iter"][0]
    assert int(r["converged"]) == golden["lloyd_converged"][0]
    assert len(calls) == r["n_iter"]
    np.testing.assert_allclose(C.cpu().numpy(), golden["lloyd_C"], rtol=RTOL_CENTERS, atol=1e-6)
    np.testing.assert_allclose(r["inertias"], golden["lloyd_inertias"], rtol=RTOL_INERTIA)


@pytest.mark.parametrize("prec", PRECS)
@pytest.mark.parametrize("d,k", [(10, 100), (64, 64), (528, 40), (12, 2100)])
def test_lloyd_matches_oracle(torch, L, oracle, prec, d, k):
    from pyemma_gb300 import datasets
    X = datasets.gaussian_mixture(20000, d, 2 * k, 0.3, 5.0, seed=d)
    C0, _ = oracle.kmpp(X, k, 9)
    ref = oracle.lloyd(X, C0, 30, 1e-5)
    C = dev(torch, C0)
    r = L.lloyd(dev(torch, X), C, 30, 1e-5, precision=prec)
    assert r["n_iter"] == ref["n_iter"] and r["converged"] == ref["converged"]
    np.testing.assert_allclose(C.cpu().numpy(), ref["centers"], rtol=RTOL_CENTERS, atol=1e-5)
    np.testing.assert_allclose(r["inertias"], ref["inertias"], rtol=RTOL_INERTIA)
    np.testing.assert_array_equal(r["labels"].cpu().numpy(), ref["labels"])


@pytest.mark.parametrize("prec", ["fp16", "bf16"])
@pytest.mark.parametrize("fill", ["exact", "random", "shifted", "out_of_range"])
def test_tc_seed_from_label_array(torch, L, oracle, monkeypatch, prec, fill):
    # With short operand rows and many centers (KM_TC_SEED=1 here, for 700
    # centers; by default from 2048) the tensor-core pass starts each
    # frame's running best at a lower bound of the accumulator of the center
    # that the label array already names (the previous iteration's label in
    # a Lloyd run).  Whatever the array holds, the labels must be the
    # oracle's: half-integer lattice frames with many exact ties, centers a
    # hair off lattice points.
    monkeypatch.setenv("KM_TC_SEED", "1")
    rng = np.random.default_rng(71)
    n, d, k = 40000, 6, 700
    X = (rng.integers(0, 6, size=(n, d)) * 0.5).astype(np.float32)
    C = (X[rng.choice(n, k, replace=False)] + rng.normal(scale=1e-3, size=(k, d))).astype(np.float32)
    ref = oracle.assign(X, C)
    if fill == "exact":
        pre = ref.astype(np.int32)
    elif fill == "random":
        pre = rng.integers(0, k, size=n).astype(np.int32)
    elif fill == "shifted":
        pre = ((ref + 1) % k).astype(np.int32)
    else:
        pre = rng.choice(np.array([-1, -7, k, k + 5, 2 ** 31 - 1], dtype=np.int64), size=n).astype(np.int32)
    labels = torch.from_numpy(pre).cuda()
    out, _ = L.assign(dev(torch, X), dev(torch, C), precision=prec, labels=labels)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


def test_tc_seed_forced_on_long_rows(torch, L, oracle, monkeypatch):
    # KM_TC_SEED=1 seeds rows of any length (here kp = 320 and 64 centers,
    # where the default leaves the seed off); the labels stay the oracle's.
    monkeypatch.setenv("KM_TC_SEED", "1")
    from pyemma_gb300 import datasets
    X = datasets.gaussian_mixture(6000, 300, 80, 0.3, 5.0, seed=5)
    rng = np.random.default_rng(5)
    C = X[rng.choice(len(X), 64, replace=False)]
    ref = oracle.assign(X, C)
    labels = torch.from_numpy(((ref + 3) % 64).astype(np.int32)).cuda()
    out, _ = L.assign(dev(torch, X), dev(torch, C), precision="fp16", labels=labels)
    np.testing.assert_array_equal(out.cpu().numpy(), ref)


@pytest.mark.parametrize("prec", ["fp16", "bf16"])
def test_lloyd_chunked_pass_equals_one_launch(torch, L, oracle, monkeypatch, prec):
    # From 2^19 frames a Lloyd iteration runs its tensor-core pass in up to 4
    # launches over consecutive frame ranges (KM_TC_CHUNKS), each chunk with
    # its own candidate lists and counters and its exact re-check beside the
    # next launch.  Labels must not depend on the chunking; centers only to
    # the rounding of the float64 sums (the flips of different chunks arrive
    # in another order).  An odd frame count puts a partial unit in the last
    # chunk.
    from pyemma_gb300 import datasets
    n = (1 << 20) + 12345
    X = dev(torch, datasets.gaussian_mixture(n, 48, 400, 0.3, 5.0, seed=77))
    rng = np.random.default_rng(77)
    C0 = X[torch.from_numpy(rng.choice(n, 300, replace=False)).cuda()].contiguous()
    out = {}
    for chunks in ("1", "2", "3", "4", "8"):
        monkeypatch.setenv("KM_TC_CHUNKS", chunks)
        C = C0.clone()
        r = L.lloyd(X, C, 1, -1.0, precision=prec)  # labels of C0: exact, whatever the chunking
        r2 = L.lloyd(X, C, 2, -1.0, precision=prec)
        out[chunks] = (C, r, r2)
    C1, r1, r21 = out["1"]
    for chunks, (C, r, r2) in out.items():
        assert torch.equal(r["labels"], r1["labels"]), chunks
        np.testing.assert_allclose(r["inertias"], r1["inertias"], rtol=1e-9)
        torch.testing.assert_close(C, C1, rtol=1e-6, atol=1e-6)
        np.testing.assert_allclose(r2["inertias"], r21["inertias"], rtol=1e-6)
    # the last iteration's labels against the oracle on a sample
    monkeypatch.setenv("KM_TC_CHUNKS", "4")
    C = C0.clone()
    L.lloyd(X, C, 2, -1.0, precision=prec)
    lab, _ = L.assign(X, C, precision=prec)
    sample = np.sort(rng.choice(n, 20000, replace=False))
    Xs = X[torch.from_numpy(sample).cuda()].cpu().numpy()
    np.testing.assert_array_equal(lab.cpu().numpy()[sample], oracle.assign(Xs, C.cpu().numpy()))


def test_lloyd_zero_iterations(torch, L):
    X = torch.ones((10, 3), dtype=torch.float32, device="cuda")
    C = torch.zeros((2, 3), dtype=torch.float32, device="cuda")
    r = L.lloyd(X, C, 0, 1e-5)
    assert r["n_iter"] == 0 and not r["converged"]
    assert float(C.abs().sum()) == 0.0


def test_profile_counts_graph_replays(torch, L):
    rng = np.random.default_rng(21)
    X = dev(torch, rng.normal(size=(20000, 96)))
    C0 = X[:40].clone()
    L.profile_enable(True)
    try:
        C = C0.clone()
        L.lloyd(X, C, 6, -1.0, precision="fp16")
        C = C0.clone()
        L.lloyd(X, C, 4, -1.0, precision="fp32")
        prof = L.profile_read()
    finally:
        L.profile_enable(False)
    assert prof["tc"][1] == 6 and prof["tc"][0] > 0
    assert prof["fp32"][1] == 4 and prof["fp32"][0] > 0
    assert prof["update"][1] == 10
    lab, _ = L.assign(X, C0, precision="fp16")  # no error left behind by the timing
    assert lab.shape[0] == 20000


@pytest.mark.parametrize("prec,k", [("fp32", 40), ("fp16", 40), ("fp16", 300)])
def test_lloyd_device_loop_equals_host_loop(torch, L, prec, k):
    # Without a callback (and without profiling) the iterations after the first
    # run as a device-side CUDA graph WHILE loop; with a callback the host loop
    # runs them.  Both apply the same stopping rule.  k = 300 runs the CTA-pair
    # (cluster) launch inside the loop's body.
    rng = np.random.default_rng(77)
    X = dev(torch, rng.normal(size=(30000, 64)))
    C0 = X[:k].clone()
    calls = []
    for max_iter, tol in ((100, 1e-5), (150, -1.0)):
        Ca, Cb = C0.clone(), C0.clone()
        ra = L.lloyd(X, Ca, max_iter, tol, precision=prec)
        rb = L.lloyd(X, Cb, max_iter, tol, precision=prec, callback=lambda: calls.append(1))
        assert ra["n_iter"] == rb["n_iter"] and ra["converged"] == rb["converged"]
        assert len(calls) == rb["n_iter"]
        calls.clear()
        if tol < 0:
            assert ra["n_iter"] == max_iter  # crosses the 64-iteration launches
        np.testing.assert_allclose(ra["inertias"], rb["inertias"], rtol=1e-6)
        torch.testing.assert_close(Ca, Cb, rtol=1e-5, atol=1e-5)
