"""GPU parity of the two forms of the tensor-core assignment kernel.

Full-width center tiles (k >= 256) with a resident frame tile (d <= 638) run
on CTA pairs (tcgen05 cta_group::2, 256 frames per pair); KM_TC_PAIR=0 in the
environment selects the one-CTA form (128 frames per CTA).  Both must give the
oracle's labels bit for bit, including frame counts that leave the second CTA
of the last pair partly or wholly past the end of the data.
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


def dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()


@pytest.mark.parametrize("form", ["0", "1"])
@pytest.mark.parametrize("prec", ["fp16", "bf16"])
@pytest.mark.parametrize("n", [1, 100, 128, 129, 255, 256, 257, 383, 5000])
def test_pair_edges(torch, L, oracle, monkeypatch, form, prec, n):
    monkeypatch.setenv("KM_TC_PAIR", form)
    rng = np.random.default_rng(n)
    d, k = 96, 600
    X = rng.normal(size=(n, d)).astype(np.float32)
    C = rng.normal(size=(k, d)).astype(np.float32)
    C[: min(n, k)] = X[: min(n, k)] + 0.05 * rng.normal(size=(min(n, k), d)).astype(np.float32)
    lab, stats = L.assign(dev(torch, X), dev(torch, C), precision=prec)
    assert stats["precision"] == prec
    np.testing.assert_array_equal(lab.cpu().numpy(), oracle.assign(X, C))


@pytest.mark.parametrize("d", [16, 64, 200, 528, 630, 640])
def test_forms_agree(torch, L, oracle, monkeypatch, d):
    rng = np.random.default_rng(d)
    n, k = 20000, 1000
    X = rng.normal(size=(n, d)).astype(np.float32)
    C = (X[rng.integers(0, n, size=k)] + 0.1 * rng.normal(size=(k, d))).astype(np.float32)
    Xd, Cd = dev(torch, X), dev(torch, C)
    out = {}
    for form in ("0", "1"):
        monkeypatch.setenv("KM_TC_PAIR", form)
        out[form], _ = L.assign(Xd, Cd, precision="fp16")
    assert torch.equal(out["0"], out["1"])
    np.testing.assert_array_equal(out["1"].cpu().numpy(), oracle.assign(X, C))


def test_pair_lloyd_matches_single(torch, L, monkeypatch):
    rng = np.random.default_rng(5)
    X = dev(torch, rng.normal(size=(50000, 128)))
    C0 = X[:512].clone()
    res = {}
    for form in ("0", "1"):
        monkeypatch.setenv("KM_TC_PAIR", form)
        C = C0.clone()
        r = L.lloyd(X, C, 5, -1.0, precision="fp16")
        res[form] = (C, r)
    # The centroid sums use float64 atomics, whose order varies run to run.
    torch.testing.assert_close(res["0"][0], res["1"][0], rtol=1e-5, atol=1e-6)
    assert res["0"][1]["n_iter"] == res["1"][1]["n_iter"] == 5
