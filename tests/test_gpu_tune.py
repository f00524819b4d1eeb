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


@pytest.mark.parametrize("d,k", [(10, 1000), (64, 300), (528, 600), (200, 100)])
def test_every_tile_shape_gives_the_oracle_labels(oracle, d, k):
    # km_tune_tiles may pick any shape that fits; each one (center tile
    # width, CTA pair or single CTA, ring depth, 8 or 16 candidates per
    # frame) must give the exact labels.
    import torch
    from pyemma_gb300 import _lib as L
    L.load()
    L.tune_clear()
    rng = np.random.default_rng(d + k)
    X = (rng.normal(size=(6000, d)) + 4.0 * rng.integers(0, 6, size=(6000, 1))).astype(np.float32)
    C = (X[rng.choice(6000, k, replace=False)] + 0.05 * rng.normal(size=(k, d))).astype(np.float32)
    want = oracle.assign(X, C)
    Xd, Cd = torch.from_numpy(X).cuda(), torch.from_numpy(C).cuda()
    r = L.tune_tiles(Xd, Cd)
    assert len(r["tried"]) >= 2
    assert r["best"]["ms"] == min(t["ms"] for t in r["tried"])
    try:
        for plan in r["tried"]:
            L.force_tile_plan(plan)
            for prec in ("fp16", "bf16"):
                lab, _ = L.assign(Xd, Cd, precision=prec)
                np.testing.assert_array_equal(lab.cpu().numpy(), want, err_msg="%s %s" % (plan, prec))
    finally:
        L.force_tile_plan(None)
    cur = L.tile_plan(d, k)
    assert cur["tuned"] and all(cur[key] == r["best"][key] for key in ("bn", "pair", "stages", "list_len"))
    lab, _ = L.assign(Xd, Cd, precision="fp16")  # the tuned shape
    np.testing.assert_array_equal(lab.cpu().numpy(), want)
    L.tune_clear()
    assert not L.tile_plan(d, k)["tuned"]


def test_forced_shape_that_does_not_fit_is_refused():
    import torch
    from pyemma_gb300 import _lib as L
    X = torch.randn(1000, 32, device="cuda")
    try:
        L.force_tile_plan(dict(bn=128, pair=1, stages=4, list_len=16))  # pairs need 256 columns
        with pytest.raises(L.KmError) as ei:
            L.assign(X, X[:300].contiguous(), precision="fp16")
        assert ei.value.status == L.KM_ERR_UNSUPPORTED
    finally:
        L.force_tile_plan(None)
    L.assign(X, X[:300].contiguous(), precision="fp16")
