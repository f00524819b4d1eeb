"""The error bound of the tensor-core assignment, checked pair by pair.

km_debug_tc_distances returns the tensor-core value v of every squared
distance.  For every (frame, center) pair the exact float32 distance D of the
oracle must lie in [lo(v), hi(v)] as the kernel computes them (formulas in
pyemma_gb300/csrc/assign_tc.cu).  The test also measures how much of the
accumulation allowance E the hardware uses: the exact distance of the
FP16-rounded operands is evaluated here in float64 and compared with v.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

U = 2.0 ** -24


def bound_terms(X, C):
    n, d = X.shape
    k = C.shape[0]
    kp = 64 * math.ceil((d + 2) / 64)
    shift = (C.astype(np.float64).sum(0) / k).astype(np.float32)
    xp = (X - shift).astype(np.float32)
    cp = (C - shift).astype(np.float32)
    sx = np.sqrt((xp.astype(np.float64) ** 2).sum(1)) * (1 + 1e-6)
    sc = np.sqrt((cp.astype(np.float64) ** 2).sum(1)) * (1 + 1e-6)
    e = math.frexp(float(np.sqrt((cp.astype(np.float64) ** 2).sum(1)).max()))[1] if sc.max() > 0 else 7
    scale = 2.0 ** (7 - e)
    # exact norms of the FP16 rounding errors, as the prep kernels measure them
    hx = np.sqrt(((((xp * scale).astype(np.float16).astype(np.float64)) / scale - xp) ** 2).sum(1)) * (1 + 1e-6)
    hc = np.sqrt(((((cp * scale).astype(np.float16).astype(np.float64)) / scale - cp) ** 2).sum(1)) * (1 + 1e-6)
    e_coef = ((kp // 16 + 1) * 2.0 ** -21 * 1.003 + 2.0 ** -21 + 8 * U) * 1.01
    g = (d + 2) * U / (1 - (d + 2) * U) * 1.01
    S = sx[:, None] + sc[None, :]
    R = hx[:, None] + hc[None, :] + 2.0 ** -23 * S
    return dict(R=R, E=e_coef * S ** 2, g=g, xp=xp, cp=cp, scale=scale)


def check_pairs(L, torch, oracle, X, C):
    Xd = torch.from_numpy(X).cuda()
    Cd = torch.from_numpy(C).cuda()
    labels, V, _ = L.debug_tc_distances(Xd, Cd)
    V = V.cpu().numpy().astype(np.float64)
    t = bound_terms(X, C)
    R, E, g = t["R"], t["E"], t["g"]
    lo = (1 - g) * np.maximum(np.sqrt(np.maximum(V - E, 0)) - R, 0) ** 2
    hi = (1 + g) * (np.sqrt(np.maximum(V + E, 0)) + R) ** 2
    D = oracle.sqdist_fp32_sequential(X, C).astype(np.float64)
    bad = (D < lo * (1 - 1e-6) - 1e-30) | (D > hi * (1 + 1e-6) + 1e-30)
    assert not bad.any(), "bound violated for %d pairs" % bad.sum()
    # Accumulation: v against the exact distance of the rounded operands.
    s = t["scale"]
    xh = (t["xp"] * s).astype(np.float16).astype(np.float64)
    ch = (t["cp"] * s).astype(np.float16).astype(np.float64)
    Dh = ((xh[:, None, :] - ch[None, :, :]) ** 2).sum(-1) / s ** 2
    acc_use = float(np.max(np.abs(V - Dh) / E))
    assert acc_use <= 1.0
    np.testing.assert_array_equal(labels.cpu().numpy(), oracle.assign(X, C))
    return acc_use


def test_bound_holds_on_varied_data(oracle):
    import torch
    from pyemma_gb300 import _lib as L, datasets
    L.load()
    rng = np.random.default_rng(5)
    cases = []
    X = rng.normal(size=(1500, 528)).astype(np.float32)
    cases.append((X, X[rng.choice(1500, 300, replace=False)] + 0.05 * rng.normal(size=(300, 528)).astype(np.float32)))
    X = datasets.calpha_distances(n_frames=1500, seed=2)
    cases.append((X, X[rng.choice(1500, 200, replace=False)]))
    X = (1e3 + rng.normal(size=(1000, 200))).astype(np.float32)
    cases.append((X, X[rng.choice(1000, 100, replace=False)]))
    # cancellation: alternating large components with small differences
    base = rng.choice([-50.0, 50.0], size=(1, 128)) * rng.uniform(0.5, 1.5, size=(1, 128))
    X = (base + rng.normal(scale=0.1, size=(1200, 128))).astype(np.float32)
    cases.append((X, X[rng.choice(1200, 64, replace=False)]))
    uses = []
    for X, C in cases:
        uses.append(check_pairs(L, torch, oracle, np.ascontiguousarray(X, np.float32),
                                np.ascontiguousarray(C, np.float32)))
    print("largest share of the accumulation allowance used:", uses)


# ---------------------------------------------------------------------------
# FP8 (e4m3): per-frame power-of-two scales, one for the centers, the center
# norms applied in the epilogue, the accumulation allowance of assign_tc.cu's
# FP8 form.
# ---------------------------------------------------------------------------
def e4m3(v):
    """Round float64 values to e4m3 (round to nearest even, saturating at 448)."""
    v = np.asarray(v, dtype=np.float64)
    a = np.abs(v)
    e = np.floor(np.log2(np.maximum(a, 2.0 ** -6)))  # subnormals share the 2^-6 binade's step
    step = 2.0 ** (e - 3)
    q = np.rint(v / step) * step
    return np.clip(q, -448.0, 448.0)


def fp8_scale(m):
    m = np.asarray(m, dtype=np.float64)
    e = np.frexp(m)[1]
    return np.where(m > 0, 2.0 ** (8 - e), 1.0)


def bound_terms_fp8(X, C):
    n, d = X.shape
    k = C.shape[0]
    shift = (C.astype(np.float64).sum(0) / k).astype(np.float32)
    xp = (X - shift).astype(np.float32).astype(np.float64)
    cp = (C - shift).astype(np.float32).astype(np.float64)
    si = fp8_scale(np.abs(xp).max(1))[:, None]
    t = float(fp8_scale(np.abs(cp).max()))
    xt = e4m3(xp * si) / si
    ct = e4m3(cp * t) / t
    infl = 1 + 1e-6
    sx = np.sqrt((xp ** 2).sum(1)) * infl
    sc = np.sqrt((cp ** 2).sum(1)) * infl
    hx = np.sqrt(((xt - xp) ** 2).sum(1)) * infl
    hc = np.sqrt(((ct - cp) ** 2).sum(1)) * infl
    ksteps = math.ceil(d / 32)
    e_coef = (2.0 * ksteps * 2.0 ** -18 + 16 * U) * 1.25
    g = (d + 2) * U / (1 - (d + 2) * U) * 1.01
    S = sx[:, None] + sc[None, :]
    R = hx[:, None] + hc[None, :] + 2.0 ** -23 * S
    return dict(R=R, E=e_coef * S ** 2, g=g, xt=xt, ct=ct)


def check_pairs_fp8(L, torch, oracle, X, C):
    Xd = torch.from_numpy(X).cuda()
    Cd = torch.from_numpy(C).cuda()
    labels, V, _ = L.debug_tc_distances(Xd, Cd, precision="fp8")
    V = V.cpu().numpy().astype(np.float64)
    t = bound_terms_fp8(X, C)
    R, E, g = t["R"], t["E"], t["g"]
    lo = (1 - g) * np.maximum(np.sqrt(np.maximum(V - E, 0)) - R, 0) ** 2
    hi = (1 + g) * (np.sqrt(np.maximum(V + E, 0)) + R) ** 2
    D = oracle.sqdist_fp32_sequential(X, C).astype(np.float64)
    bad = (D < lo * (1 - 1e-6) - 1e-30) | (D > hi * (1 + 1e-6) + 1e-30)
    assert not bad.any(), "bound violated for %d pairs" % bad.sum()
    # Accumulation: v against the exact distance of the rounded operands.
    Dh = ((t["xt"][:, None, :] - t["ct"][None, :, :]) ** 2).sum(-1)
    acc_use = float(np.max(np.abs(V - Dh) / E))
    assert acc_use <= 1.0
    np.testing.assert_array_equal(labels.cpu().numpy(), oracle.assign(X, C))
    return acc_use


def test_fp8_bound_holds_on_varied_data(oracle):
    import torch
    from pyemma_gb300 import _lib as L, datasets
    L.load()
    rng = np.random.default_rng(6)
    cases = []
    X = rng.normal(size=(1200, 528)).astype(np.float32)
    cases.append((X, X[rng.choice(1200, 260, replace=False)] + 0.05 * rng.normal(size=(260, 528)).astype(np.float32)))
    X = datasets.calpha_distances(n_frames=1200, seed=3)
    cases.append((X, X[rng.choice(1200, 200, replace=False)]))
    X = (1e3 + rng.normal(size=(1000, 200))).astype(np.float32)
    cases.append((X, X[rng.choice(1000, 100, replace=False)]))
    # rows of very different magnitude (per-row scales) and a zero row
    X = (rng.normal(size=(900, 96)) * 10.0 ** rng.uniform(-3, 3, size=(900, 1))).astype(np.float32)
    X[5] = 0.0
    cases.append((X, X[rng.choice(900, 90, replace=False)]))
    uses = []
    for X, C in cases:
        uses.append(check_pairs_fp8(L, torch, oracle, np.ascontiguousarray(X, np.float32),
                                    np.ascontiguousarray(C, np.float32)))
    print("FP8: largest share of the accumulation allowance used:", uses)
