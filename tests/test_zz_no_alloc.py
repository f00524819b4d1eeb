"""The allocation-free centroid update (km_update_noalloc) on the GPU.

Callers such as plugins inside programs that own every device allocation
cannot pass a workspace; km_update_noalloc serves them from a fixed scratch
array inside the library.  These tests call it through the C ABI and check
it against km_update (which takes a caller workspace) with the tolerances of
the other update tests: centers within 1e-6 relative, counts exact, inertia
within 1e-9 relative.  Two calls run back to back with different shapes, so
that stale contents of the shared scratch array would show up.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL_CENTER_STEP = 1e-6
RTOL_INERTIA = 1e-9


def _call_noalloc(L, torch, X, labels, C_old):
    lib = L.load()
    n, d = X.shape
    k = C_old.shape[0]
    C_new = torch.empty_like(C_old)
    counts = torch.empty(k, dtype=torch.int64, device=X.device)
    cost = torch.empty(1, dtype=torch.float64, device=X.device)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib.km_update_noalloc(ctypes.c_void_p(X.data_ptr()), n, d, ctypes.c_void_p(labels.data_ptr()), k,
                               ctypes.c_void_p(C_old.data_ptr()), ctypes.c_void_p(C_new.data_ptr()),
                               ctypes.c_void_p(counts.data_ptr()), ctypes.c_void_p(cost.data_ptr()), stream)
    return rc, C_new, counts, float(cost.item())


def _case(torch, seed, n, d, k):
    rng = np.random.default_rng(seed)
    X = (3.0 + rng.normal(size=(n, d))).astype(np.float32)
    C = X[rng.choice(n, k, replace=False)].copy()
    C[k // 2] = 1e6  # an empty cluster keeps its center
    from oracle import oracle
    labels = oracle.assign(X, C)
    t = lambda a: torch.from_numpy(a).cuda()
    return t(X), t(labels), t(C)


def test_noalloc_matches_workspace_update_twice():
    import torch
    from pyemma_gb300 import _lib as L
    for seed, (n, d, k) in enumerate([(50000, 528, 300), (7000, 10, 1000), (30000, 3, 20)]):
        X, labels, C = _case(torch, seed, n, d, k)
        rc, C_na, cnt_na, cost_na = _call_noalloc(L, torch, X, labels, C)
        assert rc == L.KM_OK, L.load().km_last_error()
        C_ws, cnt_ws, cost_ws = L.update(X, labels, C)
        np.testing.assert_allclose(C_na.cpu().numpy(), C_ws.cpu().numpy(), rtol=RTOL_CENTER_STEP, atol=0)
        np.testing.assert_array_equal(cnt_na.cpu().numpy(), cnt_ws.cpu().numpy())
        assert abs(cost_na - cost_ws) <= RTOL_INERTIA * abs(cost_ws)
        np.testing.assert_array_equal(C_na.cpu().numpy()[k // 2], C.cpu().numpy()[k // 2])


def test_noalloc_rejects_oversized_shapes_and_bad_labels():
    import torch
    from pyemma_gb300 import _lib as L
    lib = L.load()
    limit = lib.km_update_noalloc_max_bytes()
    assert limit == 32 << 20
    # 20 M frames need 80 MB of sorted indices: beyond the fixed array.
    dummy = ctypes.c_void_p(256)
    rc = lib.km_update_noalloc(dummy, 20_000_000, 4, dummy, 8, dummy, ctypes.c_void_p(512), None,
                               ctypes.c_void_p(768), None)
    assert rc == L.KM_ERR_WORKSPACE
    assert b"fixed array" in lib.km_last_error()
    X, labels, C = _case(torch, 5, 1000, 6, 10)
    labels[17] = 10
    rc, _, _, _ = _call_noalloc(L, torch, X, labels, C)
    assert rc == L.KM_ERR_BAD_LABEL
    labels[17] = 0
    rc, C_na, _, _ = _call_noalloc(L, torch, X, labels, C)  # the error word does not stick
    assert rc == L.KM_OK


def test_noalloc_concurrent_threads_and_streams():
    # Two host threads, each on its own stream, call km_update_noalloc with
    # different shapes; the library runs the calls one at a time, so every
    # result equals the workspace update's.
    import threading
    import torch
    from pyemma_gb300 import _lib as L
    cases = [_case(torch, 10 + i, n, d, k) for i, (n, d, k) in enumerate([(40000, 64, 200), (25000, 5, 30)])]
    want = [L.update(X, labels, C) for X, labels, C in cases]
    torch.cuda.synchronize()
    failures = []

    def worker(i):
        X, labels, C = cases[i]
        C_ws, cnt_ws, cost_ws = want[i]
        with torch.cuda.stream(torch.cuda.Stream()):
            for _ in range(15):
                rc, C_na, cnt_na, cost_na = _call_noalloc(L, torch, X, labels, C)
                if rc != L.KM_OK:
                    failures.append((i, "rc", rc))
                    return
                if not np.allclose(C_na.cpu().numpy(), C_ws.cpu().numpy(), rtol=RTOL_CENTER_STEP, atol=0):
                    failures.append((i, "centers"))
                if not np.array_equal(cnt_na.cpu().numpy(), cnt_ws.cpu().numpy()):
                    failures.append((i, "counts"))
                if abs(cost_na - cost_ws) > RTOL_INERTIA * abs(cost_ws):
                    failures.append((i, "cost"))

    threads = [threading.Thread(target=worker, args=(i,)) for i in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join(timeout=120)
    assert not any(t.is_alive() for t in threads)
    assert not failures, failures
