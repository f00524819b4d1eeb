"""CPU checks of the C ABI library and of the host layer (no GPU needed).

libkmgpu.so must load, export every entry point include/kmgpu.h declares,
size workspaces and reject bad arguments before touching a device.  The
host layer must keep PyEMMA's conventions (input normalisation, lengths,
seed and n_jobs rules) and fail loudly without a CUDA device.
"""
import ctypes
import os
import re
from unittest import mock

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            with open(os.path.join(ROOT, "include", fn)) as fh:
                text = fh.read()
            names += re.findall(r"^\s*(?:int|size_t|const char \*)\s*(km_\w+)\s*\(", text, re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_symbols()
    for required in ("km_assign", "km_batch_assign", "km_update", "km_kmpp", "km_lloyd"):
        assert required in names


def test_library_exports_every_declared_symbol(kmlib):
    for name in declared_symbols():
        assert hasattr(kmlib, name), name


def test_binding_lists_every_declared_symbol():
    from pyemma_gb300 import _lib
    assert sorted(_lib.EXPORTED) == [n for n in declared_symbols() if n in _lib.EXPORTED]
    assert set(declared_symbols()) <= set(_lib.EXPORTED)


def test_version_and_status_strings(kmlib):
    assert kmlib.km_version() >= 1
    for s in range(8):
        assert len(kmlib.km_status_string(s)) > 0


def test_workspace_sizes_are_host_only(kmlib):
    assert kmlib.km_assign_workspace_size(1000, 2, 50, 0) == 0  # exact FP32 kernel needs none
    tc = kmlib.km_assign_workspace_size(2_000_000, 528, 2000, 1)
    assert tc >= 2_000_000 * 576 * 2  # the FP16 frame copy
    assert kmlib.km_assign_workspace_size(2_000_000, 528, 2000, 2) == tc  # auto picks the tensor cores for wide d
    assert kmlib.km_assign_workspace_size(1000, 10, 50, 2) == 0  # auto picks FP32 for narrow d
    assert kmlib.km_update_workspace_size(100, 3, 7) > 0
    assert kmlib.km_kmpp_workspace_size(100, 3, 7) > 0
    assert kmlib.km_lloyd_workspace_size(100, 3, 7, 0) >= kmlib.km_update_workspace_size(100, 3, 7)
    # out-of-range shapes give 0
    assert kmlib.km_assign_workspace_size(-1, 3, 7, 0) == 0
    assert kmlib.km_assign_workspace_size(10, 0, 7, 0) == 0
    assert kmlib.km_assign_workspace_size(10, 3, 0, 0) == 0


def test_bad_arguments_rejected_before_device(kmlib):
    from pyemma_gb300 import _lib
    stats = _lib.AssignStats()
    rc = kmlib.km_assign(None, -5, 3, None, 2, 0, None, None, 0, ctypes.byref(stats), None)
    assert rc == _lib.KM_ERR_BAD_SHAPE
    assert b"out of range" in kmlib.km_last_error()
    rc = kmlib.km_assign(None, 10, 3, None, 2, 0, None, None, 0, ctypes.byref(stats), None)
    assert rc == _lib.KM_ERR_BAD_SHAPE
    offs = np.array([0, 5, 3], dtype=np.int64)
    rc = kmlib.km_batch_assign(ctypes.c_void_p(16), offs.ctypes.data_as(ctypes.c_void_p), 2, 3,
                               ctypes.c_void_p(16), 2, 0, ctypes.c_void_p(16), None, 0, None, None)
    assert rc == _lib.KM_ERR_BAD_SHAPE
    rc = kmlib.km_update(ctypes.c_void_p(16), 10, 3, ctypes.c_void_p(16), 2, ctypes.c_void_p(32),
                         ctypes.c_void_p(32), None, ctypes.c_void_p(64), None, 0, None)
    assert rc == _lib.KM_ERR_BAD_SHAPE  # C_new aliases C_old
    rc = kmlib.km_update(ctypes.c_void_p(16), 10, 3, ctypes.c_void_p(16), 2, ctypes.c_void_p(32),
                         ctypes.c_void_p(48), None, ctypes.c_void_p(64), None, 0, None)
    assert rc == _lib.KM_ERR_WORKSPACE
    n_iter, conv = ctypes.c_int32(), ctypes.c_int32()
    rc = kmlib.km_lloyd(None, 10, 3, 2, None, 5, 1e-5, 0, None, None, ctypes.byref(n_iter), ctypes.byref(conv),
                        _lib.CALLBACK(0), None, None, 0, None)
    assert rc == _lib.KM_ERR_BAD_SHAPE
    rc = kmlib.km_lloyd_host(None, None, -1, ctypes.c_void_p(16), 10, 3, 2, ctypes.c_void_p(32), 5, 1e-5, 0,
                             ctypes.c_void_p(48), None, ctypes.byref(n_iter), ctypes.byref(conv), _lib.CALLBACK(0),
                             None, None, 0, None)
    assert rc == _lib.KM_ERR_BAD_SHAPE
    # parts that do not add up to n are refused before any device work
    rows = np.array([4, 5], dtype=np.int64)
    ptrs = (ctypes.c_void_p * 2)(16, 32)
    need = kmlib.km_lloyd_workspace_size(10, 3, 2, 0)
    rc = kmlib.km_lloyd_host(ptrs, rows.ctypes.data_as(ctypes.c_void_p), 2, ctypes.c_void_p(16), 10, 3, 2,
                             ctypes.c_void_p(32), 5, 1e-5, 0, ctypes.c_void_p(48), None, ctypes.byref(n_iter),
                             ctypes.byref(conv), _lib.CALLBACK(0), None, ctypes.c_void_p(64), need, None)
    assert rc == _lib.KM_ERR_BAD_SHAPE
    assert b"host parts" in kmlib.km_last_error()


# ---------------------------------------------------------------------------
# host layer
# ---------------------------------------------------------------------------
def test_ensure_traj_list_conventions():
    from pyemma_gb300.coordinates.data import InMemorySource, ensure_traj_list
    assert ensure_traj_list(np.zeros(7))[0].shape == (7, 1)
    assert ensure_traj_list([1.0, 2.0, 3.0])[0].shape == (3, 1)
    assert [t.shape for t in ensure_traj_list([np.zeros((4, 2)), np.zeros((5, 2))])] == [(4, 2), (5, 2)]
    assert ensure_traj_list(np.zeros((3, 2, 4)))[0].shape == (3, 8)
    with pytest.raises(ValueError):
        InMemorySource([np.zeros((4, 2)), np.zeros((4, 3))])
    with pytest.raises(ValueError):
        ensure_traj_list("not data")


def test_strided_lengths():
    from pyemma_gb300.coordinates.data import InMemorySource
    src = InMemorySource([np.zeros((100, 3)), np.zeros((10, 3)), np.zeros((3, 3))])
    for stride in (1, 2, 3, 7):
        for skip in (0, 1, 5, 42):
            want = [len(t[skip::stride]) for t in src.data]
            assert list(src.trajectory_lengths(stride=stride, skip=skip)) == want
            assert [len(f) for f in src.frames(stride=stride, skip=skip)] == want
    with pytest.raises(IndexError):
        src.trajectory_length(3)
    assert src.default_chunksize == 256 * 1024 * 1024 // (8 * 3)


def test_fixed_seed_rules():
    from pyemma_gb300.coordinates import KmeansClustering
    km = KmeansClustering(5, fixed_seed=True)
    assert km.fixed_seed == 42
    assert KmeansClustering(5, fixed_seed=463498).fixed_seed == 463498
    for bad in (-1, 2 ** 32):
        s = KmeansClustering(5, fixed_seed=bad).fixed_seed
        assert 0 <= s <= 2 ** 32 - 1
    assert 0 <= KmeansClustering(5, fixed_seed=False).fixed_seed <= 2 ** 32 - 1
    with pytest.raises(ValueError):
        KmeansClustering(5, fixed_seed="x")
    with pytest.raises(ValueError):
        KmeansClustering(5, init_strategy="random")


def test_n_jobs_resolution():
    from pyemma_gb300.coordinates import AssignCenters
    C = np.zeros((3, 2))
    with mock.patch.dict(os.environ, {"PYEMMA_NJOBS": "0"}):
        assert AssignCenters(C, n_jobs=2).n_jobs == 2
    with mock.patch.dict(os.environ, {"PYEMMA_NJOBS": "3"}):
        assert AssignCenters(C, n_jobs=None).n_jobs == 3
    env = {k: v for k, v in os.environ.items() if k not in ("PYEMMA_NJOBS", "SLURM_CPUS_ON_NODE")}
    with mock.patch.dict(os.environ, env, clear=True), mock.patch("psutil.cpu_count", lambda *a, **k: 5):
        assert AssignCenters(C).n_jobs == 5
    env["PYEMMA_NJOBS"] = "this is not right"
    with mock.patch.dict(os.environ, env, clear=True), mock.patch("psutil.cpu_count", lambda *a, **k: 3):
        assert AssignCenters(C).n_jobs == 3
    with pytest.raises(ValueError):
        AssignCenters(C, n_jobs=0)


def test_assign_centers_shape_errors():
    from pyemma_gb300.coordinates import assign_to_centers
    with pytest.raises(ValueError):
        assign_to_centers(np.empty((100, 3)), np.empty((5, 4)))
    with pytest.raises(ValueError):
        assign_to_centers(np.empty((100, 3)), np.empty(1))
    with pytest.raises(ValueError):
        assign_to_centers(np.empty((100, 3)), None)


def test_uniform_init_follows_reference_rule():
    # kmeans.py:299-324: seeded random.sample per trajectory, frames taken in
    # iteration order until n_clusters.
    import math
    import random
    from pyemma_gb300.coordinates import KmeansClustering
    trajs = [np.arange(40, dtype=np.float32)[:, None], 100 + np.arange(60, dtype=np.float32)[:, None]]
    km = KmeansClustering(7, init_strategy="uniform", fixed_seed=11)
    lengths = [40, 60]
    idx = km._uniform_indices(lengths, 100)
    state = random.getstate()
    random.seed(11)
    want = {i: random.sample(list(range(L)), int(math.ceil(L / 100.0 * 7))) for i, L in enumerate(lengths)}
    random.setstate(state)
    assert idx == want
    centers = km._uniform_centers(trajs, idx)
    expect = [trajs[0][t] for t in sorted(want[0])] + [trajs[1][t] for t in sorted(want[1])]
    np.testing.assert_array_equal(centers, np.asarray(expect[:7]).reshape(-1, 1))


def test_minrmsd_dimension_rule():
    # clustering_module.cpp:13-15: the metric needs d divisible by 3
    from pyemma_gb300.coordinates.clustering.kmeans import KmeansClustering
    from pyemma_gb300.coordinates.clustering.regspace import RegularSpaceClustering
    km = KmeansClustering(n_clusters=3, metric="minRMSD")
    assert km.metric == "minRMSD"
    with pytest.raises(ValueError):
        km.estimate(np.zeros((10, 4), dtype=np.float32))
    with pytest.raises(ValueError):
        RegularSpaceClustering(dmin=1.0, metric="minRMSD").estimate(np.zeros((10, 4), dtype=np.float32))
    with pytest.raises(ValueError):
        KmeansClustering(n_clusters=3, metric="manhattan")


def test_gpu_path_fails_loudly_without_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    from pyemma_gb300.coordinates import assign_to_centers, cluster_kmeans
    with pytest.raises(RuntimeError):
        assign_to_centers(np.zeros((10, 2)), np.zeros((3, 2)))
    with pytest.raises(RuntimeError):
        cluster_kmeans(np.zeros((10, 2)), k=2)


def test_serving_and_resident_sets_need_a_device():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    from pyemma_gb300 import _lib
    with pytest.raises(_lib.KmError) as e:
        _lib.Server()
    assert e.value.status == _lib.KM_ERR_CUDA
    L = _lib.load()
    import ctypes
    # argument checks run before any device call
    assert L.km_serve_submit(None, 0, None, 0, 1, None, None) == _lib.KM_ERR_BAD_SHAPE
    assert L.km_serve_poll(None, 1, 0, None) == _lib.KM_ERR_BAD_SHAPE
    assert L.km_serve_shutdown(None) == _lib.KM_OK
    assert L.km_centers_destroy(None) == _lib.KM_OK
    out = ctypes.c_void_p()
    assert L.km_centers_create(None, 4, 2, 0, None, ctypes.byref(out)) == _lib.KM_ERR_BAD_SHAPE
    assert L.km_assign_centers_workspace_size(100, None) == 0


def test_plan_batches_covers_every_frame_in_order():
    from pyemma_gb300.coordinates._device import plan_batches
    rng = np.random.default_rng(0)
    for lengths in ([0], [5], [0, 3, 0, 7, 1], list(rng.integers(0, 50, size=30))):
        for budget in (1, 4, 7, 1000):
            batches = plan_batches(lengths, budget)
            sizes = [sum(b - a for _, a, b in batch) for batch in batches]
            assert all(0 < s <= budget for s in sizes)
            assert all(s == budget for s in sizes[:-1])
            seen = {i: [] for i in range(len(lengths))}
            for batch in batches:
                for i, a, b in batch:
                    assert 0 <= a < b <= lengths[i]
                    seen[i].append((a, b))
            for i, length in enumerate(lengths):
                spans = seen[i]
                assert (spans[0][0] if spans else 0) == 0
                assert all(spans[j][1] == spans[j + 1][0] for j in range(len(spans) - 1))
                assert (spans[-1][1] if spans else 0) == length
    with pytest.raises(ValueError):
        plan_batches([3], 0)



def test_minrmsd_leader_walk_equals_sequential_walk(oracle, monkeypatch):
    # The batched walk over km_assign_minrmsd, driven here by a stand-in that
    # returns the oracle's labels and float32 rmsd (the values the kernel
    # returns bit for bit), equals the oracle's sequential walk for any block
    # size, including the max_centers stop and a frame that is not finite.
    import torch
    from pyemma_gb300 import _lib
    from pyemma_gb300.coordinates.clustering import regspace

    def fake_assign_minrmsd(X, C, labels=None, return_rmsd=False):
        lab, msd = oracle.assign_minrmsd(X.numpy(), C.numpy(), return_msd=True)
        return torch.from_numpy(lab), torch.from_numpy(np.sqrt(msd).astype(np.float32))

    monkeypatch.setattr(_lib, "assign_minrmsd", fake_assign_minrmsd)
    from test_oracle_pins import rotated_clusters
    rng = np.random.default_rng(22)
    X = np.concatenate([rotated_clusters(rng, n_clusters=4, n_particles=4, per_cluster=30),
                        rng.uniform(-2, 2, size=(60, 12)).astype(np.float32)])
    X[7, 2] = np.nan
    Xt = torch.from_numpy(X)
    for dmin, max_centers in ((0.9, 1000), (0.5, 1000), (0.5, 7), (0.5, 1)):
        want, conv = oracle.regspace_minrmsd(X, dmin, max_centers)
        for block in (1, 5, 64, 8192):
            idx, done = regspace.minrmsd_leader_walk(Xt, dmin, max_centers, block=block)
            np.testing.assert_array_equal(X[idx], want)
            assert done == conv
    Xn = X.copy()
    Xn[0, 0] = np.nan  # a first frame that is not finite is the only center
    want, conv = oracle.regspace_minrmsd(Xn, 0.5, 1000)
    idx, done = regspace.minrmsd_leader_walk(torch.from_numpy(Xn), 0.5, 1000, block=16)
    assert idx == [0] and len(want) == 1 and done == conv


def test_index_clusters_and_samples():
    # test_cluster_samples.py:30-73: the catalogue of (trajectory, time)
    # indexes per cluster and samples drawn from it, on dtrajs set directly
    # (these helpers are host-only; the assignment that makes the dtrajs is
    # tested on the GPU)
    from pyemma_gb300.coordinates import AssignCenters
    trajs = [[0, 1, 2], [3, 4, 5], [6, 7, 8], [0, 1, 2], [3, 4, 5], [6, 7, 8]]
    obj = AssignCenters(np.arange(9, dtype=np.float32).reshape(-1, 1))
    obj._dtrajs = [np.asarray(t, dtype=np.int32) for t in trajs]
    ref = [[[i // 3, i % 3], [i // 3 + 3, i % 3]] for i in range(9)]
    for cc in range(9):
        np.testing.assert_array_equal(obj.index_clusters[cc], ref[cc])
    samples = obj.sample_indexes_by_cluster(np.arange(9), 10)
    for ii, isample in enumerate(samples):
        assert isample.shape == (10, 2)
        assert all(obj.dtrajs[a][b] == ii for a, b in isample)
    distinct = obj.sample_indexes_by_cluster([4], 10, replace=False)[0]
    assert len(distinct) == 2 and len({tuple(p) for p in distinct}) == 2


def test_save_dtrajs_formats(tmp_path):
    # interface.py:233-302 (test_cluster.py:137-150, test_assign.py:157-166):
    # file names from the prefix and trajectory index or from trajfiles, ascii
    # and npy output, no silent overwrite
    from pyemma_gb300.coordinates import AssignCenters
    obj = AssignCenters(np.arange(4, dtype=np.float32).reshape(-1, 1))
    obj._dtrajs = [np.array([0, 3, 3, 1], dtype=np.int32), np.array([2], dtype=np.int32)]
    out = str(tmp_path)
    obj.save_dtrajs(prefix="run", output_dir=out, extension="dtraj")
    for i, d in enumerate(obj._dtrajs):
        np.testing.assert_array_equal(np.atleast_1d(np.loadtxt(os.path.join(out, "run_%i.dtraj" % i), dtype=int)), d)
    obj.save_dtrajs(output_dir=out, output_format="npy", extension=".npy")
    for i, d in enumerate(obj._dtrajs):
        np.testing.assert_array_equal(np.load(os.path.join(out, "%i.npy" % i)), d)
    obj.save_dtrajs(trajfiles=["/data/a.xtc", "/data/b.xtc"], output_dir=out)
    assert os.path.exists(os.path.join(out, "a.dtraj")) and os.path.exists(os.path.join(out, "b.dtraj"))
    obj._dtrajs = [np.array([1, 1], dtype=np.int32), np.array([0], dtype=np.int32)]
    obj.save_dtrajs(prefix="run", output_dir=out, extension=".dtraj")  # exists: kept, error logged
    np.testing.assert_array_equal(np.loadtxt(os.path.join(out, "run_0.dtraj"), dtype=int), [0, 3, 3, 1])
    obj.overwrite_dtrajs = True
    obj.save_dtrajs(prefix="run", output_dir=out, extension=".dtraj")
    np.testing.assert_array_equal(np.loadtxt(os.path.join(out, "run_0.dtraj"), dtype=int), [1, 1])


def test_save_and_load_estimators(tmp_path):
    # test_serialization.py:73-90: a saved estimator comes back with its
    # parameters and model fields; several models share a file
    import pyemma_gb300
    from pyemma_gb300.coordinates import (AssignCenters, KmeansClustering, MiniBatchKmeansClustering,
                                          RegularSpaceClustering, UniformTimeClustering)
    fn = str(tmp_path / "models.pyemma")
    rng = np.random.default_rng(0)
    km = KmeansClustering(n_clusters=10, init_strategy="uniform", max_iter=42, metric="minRMSD", stride=1,
                          fixed_seed=463498, precision="fp16")
    km.clustercenters = rng.random((10, 3))
    km.initial_centers_ = rng.random((10, 3)).astype(np.float32)
    km._converged = True
    km.inertias = np.array([3.0, 2.5, 2.4])
    km.n_iter = 3
    km._dtrajs = [np.array([0, 3, 9], dtype=np.int32), np.array([], dtype=np.int32)]
    km.save(fn)
    back = pyemma_gb300.load(fn)
    assert type(back) is KmeansClustering
    for k in ("n_clusters", "init_strategy", "max_iter", "metric", "stride", "fixed_seed", "precision", "tolerance"):
        assert getattr(back, k) == getattr(km, k), k
    np.testing.assert_array_equal(back.clustercenters, km.clustercenters)
    np.testing.assert_array_equal(back.initial_centers_, km.initial_centers_)
    assert back.converged and back.n_iter == 3
    np.testing.assert_array_equal(back.inertias, km.inertias)
    assert [d.tolist() for d in back.dtrajs] == [[0, 3, 9], []]
    others = {"regspace": RegularSpaceClustering(dmin=0.1, max_centers=100, metric="minRMSD", n_jobs=4, stride=2),
              "uniform": UniformTimeClustering(n_clusters=3, metric="minRMSD", n_jobs=4),
              "mini": MiniBatchKmeansClustering(n_clusters=5, batch_size=0.3, max_iter=7),
              "assign": AssignCenters(rng.random((4, 6)), metric="minRMSD", skip=2)}
    for name, obj in others.items():
        obj.save(fn, model_name=name)
    assert pyemma_gb300.list_models(fn) == ["assign", "default", "mini", "regspace", "uniform"]
    for name, obj in others.items():
        back = type(obj).load(fn, model_name=name)
        for k, v in obj.get_params().items():
            if isinstance(v, np.ndarray):
                np.testing.assert_array_equal(getattr(back, k), v)
            else:
                assert getattr(back, k) == v, (name, k)
    with pytest.raises(RuntimeError):
        km.save(fn)
    km.max_iter = 7
    km.save(fn, overwrite=True)
    assert pyemma_gb300.load(fn).max_iter == 7
    with pytest.raises(KeyError):
        pyemma_gb300.load(fn, model_name="missing")
    with pytest.raises(TypeError):
        KmeansClustering.load(fn, model_name="regspace")


def test_synthetic_workloads_are_seeded():
    # the benchmark inputs: deterministic per seed, with the stated shapes
    # and value ranges (c1 mixture, c2 trajectories, c3 C-alpha distances)
    from pyemma_gb300 import datasets
    a, b = datasets.small_mixture(seed=3), datasets.small_mixture(seed=3)
    assert a.shape == (100000, 2) and a.dtype == np.float32
    np.testing.assert_array_equal(a, b)
    assert not np.array_equal(a, datasets.small_mixture(seed=4))
    trajs = datasets.metastable_trajectories(n_traj=5, d=10, lmin=500, lmax=5000, seed=1)
    assert len(trajs) == 5 and all(t.shape[1] == 10 and t.dtype == np.float32 for t in trajs)
    assert all(500 <= len(t) <= 5000 for t in trajs)
    again = datasets.metastable_trajectories(n_traj=5, d=10, lmin=500, lmax=5000, seed=1)
    assert all(np.array_equal(x, y) for x, y in zip(trajs, again))
    D = datasets.calpha_distances(n_frames=3000, seed=2)
    assert D.shape == (3000, 528) and D.dtype == np.float32
    assert 0.0 < D.min() and D.max() < 12.0 and np.isfinite(D).all()
    np.testing.assert_array_equal(D, datasets.calpha_distances(n_frames=3000, seed=2))
