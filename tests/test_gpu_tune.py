"""km_tune: measured precision choice for (d, k), consulted by 'auto'."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_tune_sets_the_auto_choice(oracle):
    import torch
    from pyemma_gb300 import _lib as L
    L.load()
    rng = np.random.default_rng(31)
    X = rng.normal(size=(20000, 64)).astype(np.float32)
    C = X[rng.choice(20000, 500, replace=False)].copy()
    Xd, Cd = torch.from_numpy(X).cuda(), torch.from_numpy(C).cuda()
    L.tune_clear()
    r = L.tune(Xd, Cd)
    assert r["chosen"] in ("fp32", "fp16")
    assert r["ms_fp32"] > 0 and r["ms_fp16"] > 0
    assert r["chosen"] == ("fp16" if r["ms_fp16"] < r["ms_fp32"] else "fp32")
    lab, st = L.assign(Xd, Cd, precision="auto")
    assert st["precision"] == r["chosen"]
    np.testing.assert_array_equal(lab.cpu().numpy(), oracle.assign(X, C))
    L.tune_clear()
    # without a table entry the rule applies: d=64 takes the tensor cores
    _, st = L.assign(Xd, Cd, precision="auto")
    assert st["precision"] == "fp16"


def test_auto_rule_small_d():
    import torch
    from pyemma_gb300 import _lib as L
    L.load()
    L.tune_clear()
    rng = np.random.default_rng(32)
    X = torch.from_numpy(rng.normal(size=(5000, 16)).astype(np.float32)).cuda()
    for k, want in ((100, "fp32"), (1000, "fp16")):
        C = X[:k].contiguous()
        _, st = L.assign(X, C, precision="auto")
        assert st["precision"] == want, (k, st)
    # d = 8..15 picks the tensor cores once k >= 1000, the exact kernel below
    X10 = torch.from_numpy(rng.normal(size=(5000, 10)).astype(np.float32)).cuda()
    _, st = L.assign(X10, X10[:2000].contiguous(), precision="auto")
    assert st["precision"] == "fp16"
    _, st = L.assign(X10, X10[:500].contiguous(), precision="auto")
    assert st["precision"] == "fp32"
    X4 = torch.from_numpy(rng.normal(size=(5000, 4)).astype(np.float32)).cuda()
    _, st = L.assign(X4, X4[:2000].contiguous(), precision="auto")
    assert st["precision"] == "fp32"
