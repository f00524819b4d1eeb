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
    # 20 M frames need 160 MB (two int32 arrays of n: the sorted indices and
    # their labels): beyond the fixed array.
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


def test_noalloc_maps_every_device_error_bit_like_km_update():
    # The error word of a call carries a bit per failure site.  A wait of the
    # segment sums that ran out (bit 1) must come back as KM_ERR_TIMEOUT, as
    # from km_update, not as KM_OK with stale outputs.  The bit is planted by
    # the library's test hook on the host side; no device wait is made to
    # run out.
    import torch
    from pyemma_gb300 import _lib as L
    lib = L.load()
    X, labels, C = _case(torch, 7, 2000, 8, 12)
    for bits, want in ((1, L.KM_ERR_TIMEOUT), (2, L.KM_ERR_TIMEOUT), (4, L.KM_ERR_TIMEOUT),
                       (8, L.KM_ERR_BAD_LABEL)):
        assert lib.km_debug_fake_device_error(bits) == L.KM_OK
        rc, _, _, _ = _call_noalloc(L, torch, X, labels, C)
        assert rc == want, (bits, rc, lib.km_last_error())
        assert lib.km_debug_fake_device_error(bits) == L.KM_OK
        with pytest.raises(L.KmError) as ei:
            L.update(X, labels, C)
        assert ei.value.status == want
    rc, _, _, _ = _call_noalloc(L, torch, X, labels, C)  # the planted bits are used up
    assert rc == L.KM_OK


def test_noalloc_refuses_a_capturing_stream():
    # Each call reads its error word back and synchronises its stream, which
    # a stream capture cannot hold: the call refuses before enqueuing work,
    # and the capture stays valid.
    import torch
    from pyemma_gb300 import _lib as L
    lib = L.load()
    X, labels, C = _case(torch, 8, 1000, 4, 6)
    C_new = torch.empty_like(C)
    cost = torch.empty(1, dtype=torch.float64, device="cuda")
    s = torch.cuda.Stream()
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        g.capture_begin()
        try:
            rc = lib.km_update_noalloc(ctypes.c_void_p(X.data_ptr()), X.shape[0], X.shape[1],
                                       ctypes.c_void_p(labels.data_ptr()), C.shape[0], ctypes.c_void_p(C.data_ptr()),
                                       ctypes.c_void_p(C_new.data_ptr()), None, ctypes.c_void_p(cost.data_ptr()),
                                       ctypes.c_void_p(s.cuda_stream))
            C_new.add_(1.0)  # the capture still records work
        finally:
            g.capture_end()
    assert rc == L.KM_ERR_UNSUPPORTED
    assert b"captured" in lib.km_last_error()
    rc, C_na, _, _ = _call_noalloc(L, torch, X, labels, C)
    assert rc == L.KM_OK
