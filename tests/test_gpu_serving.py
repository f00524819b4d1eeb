"""Resident center sets (km_centers_*) and the serving loop (km_serve_*).

A request's labels must not depend on what else is in flight: every request
served in a mixed stream of center sets, lengths and batch splits is checked
against the same trajectory assigned alone (and against the oracle).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch
    return torch


@pytest.fixture(scope="module")
def L():
    from pyemma_gb300 import _lib
    _lib.load()
    return _lib


def _mixture(rng, n, d, k):
    C = rng.normal(size=(k, d)).astype(np.float32)
    X = (C[rng.integers(0, k, size=n)] + 0.3 * rng.normal(size=(n, d))).astype(np.float32)
    return X, C


@pytest.mark.parametrize("d,k,prec", [(10, 50, "fp32"), (64, 300, "fp16"), (528, 257, "fp16"), (3, 7, "auto")])
def test_resident_centers_match_assign(torch, L, oracle, d, k, prec):
    rng = np.random.default_rng(d * 1000 + k)
    X, C = _mixture(rng, 4000, d, k)
    Cd = torch.from_numpy(C).cuda()
    Xd = torch.from_numpy(X).cuda()
    cs = L.Centers(Cd, precision=prec)
    assert (cs.k, cs.d) == (k, d)
    assert cs.device_bytes >= k * d * 4
    Cd.zero_()  # the set holds its own copy
    lab, stats = cs.assign(Xd)
    np.testing.assert_array_equal(lab.cpu().numpy(), oracle.assign(X, C))
    assert stats["n_frames"] == 4000
    lab0, _ = cs.assign(Xd[:0])
    assert lab0.numel() == 0
    cs.close()


def test_resident_centers_reject_dim_mismatch(torch, L):
    C = torch.zeros((5, 8), dtype=torch.float32, device="cuda")
    cs = L.Centers(C, precision="fp32")
    with pytest.raises(L.KmError):
        cs.assign(torch.zeros((3, 9), dtype=torch.float32, device="cuda"))
    cs.close()


def _pinned(torch, a):
    t = torch.empty(a.shape, dtype=torch.float32, pin_memory=True)
    t.numpy()[...] = a
    return t


def test_server_mixed_requests_equal_alone(torch, L, oracle):
    rng = np.random.default_rng(77)
    specs = [(2, 20, "fp32"), (10, 100, "auto"), (64, 300, "fp16"), (528, 130, "fp16")]
    sets, data = [], []
    srv = L.Server(hbm_budget_bytes=1 << 30, max_batch_frames=7000)
    for d, k, prec in specs:
        X, C = _mixture(rng, 30000, d, k)
        cs = L.Centers(torch.from_numpy(C).cuda(), precision=prec)
        sets.append((srv.add_centers(cs), cs, C))
        data.append(X)
    reqs = []
    for r in range(40):
        s = int(rng.integers(0, len(specs)))
        n = int(rng.integers(1, 12000)) if r % 10 else 0
        a = int(rng.integers(0, 30000 - n)) if n else 0
        Xr = data[s][a:a + n]
        buf = _pinned(torch, Xr) if r % 2 else np.ascontiguousarray(Xr)
        ticket, lab = srv.submit(sets[s][0], buf)
        reqs.append((ticket, s, Xr, lab))
    for ticket, s, Xr, lab in reqs:
        info = srv.poll(ticket, timeout_ms=60000)
        assert info is not None and info["status"] == 0
        assert info["n_frames"] == len(Xr)
        lab = lab.numpy() if hasattr(lab, "numpy") else lab
        if len(Xr):
            alone, _ = sets[s][1].assign(torch.from_numpy(Xr).cuda())
            np.testing.assert_array_equal(lab, alone.cpu().numpy())
            np.testing.assert_array_equal(lab, oracle.assign(Xr, sets[s][2]))
            assert info["total_ms"] >= info["queue_ms"] >= 0.0
    st = srv.stats()
    assert st["requests"] == 40
    assert st["batch_cap_frames"] == 7000
    assert st["frames"] == sum(len(x) for _, _, x, _ in reqs)
    with pytest.raises(L.KmError):
        srv.poll(reqs[0][0], timeout_ms=0)  # released after its completion
    srv.shutdown()


def test_server_splits_long_requests(torch, L, oracle):
    rng = np.random.default_rng(78)
    X, C = _mixture(rng, 50000, 64, 200)
    srv = L.Server(hbm_budget_bytes=1 << 30, max_batch_frames=4096)
    cs = L.Centers(torch.from_numpy(C).cuda(), precision="fp16")
    sid = srv.add_centers(cs)
    t, lab = srv.submit(sid, _pinned(torch, X))
    info = srv.poll(t)
    assert info["status"] == 0 and info["batch_frames"] == 4096
    np.testing.assert_array_equal(lab.numpy() if hasattr(lab, "numpy") else lab, oracle.assign(X, C))
    assert srv.stats()["batches"] >= 50000 // 4096
    srv.shutdown()


def test_server_argument_errors(torch, L):
    srv = L.Server(hbm_budget_bytes=1 << 28)
    cs = L.Centers(torch.zeros((4, 6), dtype=torch.float32, device="cuda"), precision="fp32")
    sid = srv.add_centers(cs)
    with pytest.raises(L.KmError):
        srv.submit(sid, np.zeros((3, 7), dtype=np.float32))  # d mismatch
    with pytest.raises(L.KmError):
        srv.submit(sid + 5, np.zeros((3, 6), dtype=np.float32))  # unknown set
    with pytest.raises(L.KmError):
        srv.poll(12345, timeout_ms=0)
    srv.shutdown()


def test_server_budget_too_small_fails_requests(torch, L):
    srv = L.Server(hbm_budget_bytes=512)
    cs = L.Centers(torch.zeros((4, 6), dtype=torch.float32, device="cuda"), precision="fp32")
    sid = srv.add_centers(cs)
    t, _ = srv.submit(sid, np.zeros((100, 6), dtype=np.float32))
    with pytest.raises(L.KmError) as e:
        srv.poll(t, timeout_ms=30000)
    assert e.value.status == L.KM_ERR_WORKSPACE
    srv.shutdown()
