"""Generates tests/golden/golden_small.npz: seeded inputs with oracle outputs.

The reference's own arithmetic (deeptime) cannot run here, so the vectors
come from the CPU oracle (oracle/kmeans_oracle.c).  Before they are written,
every output is cross-checked against implementations that share no code with
the oracle:

* labels: scikit-learn pairwise_distances_argmin (float64) agrees except on
  frames whose two nearest float64 distances are within 1e-5 relative;
* centers and inertia: a float64 NumPy evaluation (oracle.centers_fp64,
  oracle.inertia_fp64);
* the reference's known answers (5 separated blobs -> dtraj[i] == i // 1000,
  test_assign.py:50-109) hold for the stored blob case.

Run:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402


def _mixture(rng, n, d, ncomp, sigma, box):
    means = rng.uniform(-box, box, size=(ncomp, d))
    comp = rng.integers(0, ncomp, size=n)
    return (means[comp] + sigma * rng.normal(size=(n, d))).astype(np.float32)


def _check_labels(X, C, labels):
    from sklearn.metrics import pairwise_distances_argmin
    ref = pairwise_distances_argmin(X.astype(np.float64), C.astype(np.float64))
    D = ((X.astype(np.float64)[:, None, :] - C.astype(np.float64)[None]) ** 2).sum(-1)
    Ds = np.sort(D, axis=1)
    near_tie = (Ds[:, 1] - Ds[:, 0]) <= 1e-5 * np.maximum(Ds[:, 0], 1e-30) if C.shape[0] > 1 else np.zeros(len(X), bool)
    bad = (ref != labels) & ~near_tie
    assert not bad.any(), "oracle labels disagree with scikit-learn on %d clear frames" % bad.sum()


def main():
    rng = np.random.default_rng(20261203)
    out = {}

    # assignment, moderate d
    X = _mixture(rng, 3000, 7, 12, 0.7, 4.0)
    C = X[rng.choice(len(X), 37, replace=False)].copy()
    lab, dist = O.assign(X, C, return_dist=True)
    _check_labels(X, C, lab)
    out.update(assign_X=X, assign_C=C, assign_labels=lab, assign_dist=dist)

    # assignment, wide d (Calpha-distance-like values 0.3..6)
    Xw = rng.uniform(0.3, 6.0, size=(160, 528)).astype(np.float32)
    Cw = Xw[rng.choice(len(Xw), 24, replace=False)] + rng.normal(scale=0.05, size=(24, 528)).astype(np.float32)
    Cw = Cw.astype(np.float32)
    labw = O.assign(Xw, Cw)
    _check_labels(Xw, Cw, labw)
    out.update(wide_X=Xw, wide_C=Cw, wide_labels=labw)

    # exact ties: duplicated centers and frames equidistant from two centers
    Ct = np.array([[0, 0], [2, 0], [2, 0], [0, 2], [1, 1]], dtype=np.float32)
    Xt = np.array([[1, 0], [1, 1], [2, 0], [0, 1], [1, 2], [3, 0], [-1, -1], [1, 0.5]], dtype=np.float32)
    out.update(tie_X=Xt, tie_C=Ct, tie_labels=O.assign(Xt, Ct))

    # five separated blobs with the exact answer of test_assign.py:50-109
    means = np.array([[-3, 0], [-1, 1], [0, 0], [1, -1], [4, 2]], dtype=np.float64)
    Xb = np.zeros((5000, 2))
    for i in range(5):
        Xb[i * 1000:(i + 1) * 1000] = 0.1 * rng.normal(size=2) + means[i]
    Xb = Xb.astype(np.float32)
    labb = O.assign(Xb, means.astype(np.float32))
    assert np.array_equal(labb, np.arange(5000) // 1000)
    out.update(blobs_X=Xb, blobs_C=means.astype(np.float32), blobs_labels=labb)

    # one centroid update
    Cn, cnt, cost, _ = O.update(X, lab, C)
    C64, _ = O.centers_fp64(X, lab, C)
    assert np.allclose(Cn, C64, rtol=1e-6, atol=1e-6)
    assert abs(cost - O.inertia_fp64(X, lab, Cn)) <= 1e-9 * cost
    out.update(update_C=Cn, update_counts=cnt, update_cost=np.array([cost]))

    # Lloyd from given centers
    Xl = _mixture(rng, 5000, 2, 10, 0.5, 5.0)
    C0 = Xl[:20].copy()
    r = O.lloyd(Xl, C0, 100, 1e-5)
    C64, _ = O.centers_fp64(Xl, O.assign(Xl, C0 if r["n_iter"] == 0 else r["centers"]), r["centers"])
    out.update(lloyd_X=Xl, lloyd_C0=C0, lloyd_C=r["centers"], lloyd_labels=r["labels"],
               lloyd_inertias=r["inertias"], lloyd_n_iter=np.array([r["n_iter"]]),
               lloyd_converged=np.array([int(r["converged"])]))

    # kmeans++
    Xk = _mixture(rng, 3000, 3, 8, 0.4, 3.0)
    Ck, idx = O.kmpp(Xk, 20, 42)
    assert np.array_equal(Ck, Xk[idx])
    assert len(np.unique(idx)) == 20
    out.update(kmpp_X=Xk, kmpp_seed=np.array([42]), kmpp_idx=idx)

    # Philox4x32-10 known-answer vectors (Random123 distribution)
    out.update(philox_ctr=np.array([[0, 0, 0, 0], [0xFFFFFFFF] * 4,
                                    [0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344]], dtype=np.uint32),
               philox_key=np.array([[0, 0], [0xFFFFFFFF] * 2, [0xA4093822, 0x299F31D0]], dtype=np.uint32),
               philox_out=np.array([[0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8],
                                    [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD],
                                    [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]], dtype=np.uint32))
    for c, k, o in zip(out["philox_ctr"], out["philox_key"], out["philox_out"]):
        assert O.philox4x32_10(list(c), list(k)) == list(o)

    path = os.path.join(HERE, "golden_small.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
