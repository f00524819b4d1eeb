"""Python access to the CPU oracle (test infrastructure only).

The oracle restates PyEMMA's k-means discretization path on the CPU
(``oracle/kmeans_oracle.c``; semantics and reference citations are in that
file's header).  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs
of ``bench.py`` import this module: it checks the product and is never part of it.

Besides the ctypes bindings this module holds a float64 NumPy reference for
centers and inertia, which is independent of the C code.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libkmoracle.so")
_lib = None


def build():
    """Compile ``libkmoracle.so`` next to this file."""
    subprocess.check_call(["sh", os.path.join(_HERE, "build.sh")])


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        i64, i32, u32, f64 = ctypes.c_int64, ctypes.c_int32, ctypes.c_uint32, ctypes.c_double
        L.kmo_philox4x32_10.argtypes = [P, P, P]
        L.kmo_kmpp_draw.argtypes = [u32, u32]
        L.kmo_kmpp_draw.restype = ctypes.c_uint64
        L.kmo_quant_exponent.argtypes = [ctypes.c_float, i64]
        L.kmo_quant_exponent.restype = i32
        L.kmo_sqdist.argtypes = [P, P, i32]
        L.kmo_sqdist.restype = ctypes.c_float
        L.kmo_assign.argtypes = [P, i64, i32, P, i32, P, P, i32]
        L.kmo_update.argtypes = [P, i64, i32, P, i32, P, P, P, P, P]
        L.kmo_lloyd.argtypes = [P, i64, i32, i32, P, i32, f64, P, P, P, P, i32]
        L.kmo_kmpp.argtypes = [P, i64, i32, i32, u32, P, P, i32]
        L.kmo_regspace.argtypes = [P, i64, i32, f64, i32, P, P, P]
        L.kmo_rmsd_center.argtypes = [P, i32, P]
        L.kmo_rmsd_center.restype = f64
        L.kmo_rmsd_msd.argtypes = [P, P, f64, f64, i32]
        L.kmo_rmsd_msd.restype = f64
        L.kmo_assign_minrmsd.argtypes = [P, i64, i32, P, i32, P, P, i32]
        L.kmo_minrmsd_rows.argtypes = [P, P, i64, i32, P]
        L.kmo_lloyd_minrmsd.argtypes = [P, i64, i32, i32, P, i32, f64, P, P, P, P, i32]
        L.kmo_kmpp_minrmsd.argtypes = [P, i64, i32, i32, u32, P, P, i32]
        L.kmo_regspace_minrmsd.argtypes = [P, i64, i32, f64, i32, P, P, P]
        for name in ("kmo_assign", "kmo_update", "kmo_lloyd", "kmo_kmpp", "kmo_assign_minrmsd", "kmo_minrmsd_rows",
                     "kmo_lloyd_minrmsd", "kmo_kmpp_minrmsd", "kmo_regspace_minrmsd"):
            getattr(L, name).restype = ctypes.c_int
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def default_threads():
    return max(1, len(os.sched_getaffinity(0)))


def _check(rc, what):
    if rc != 0:
        raise RuntimeError("oracle %s failed with status %d" % (what, rc))


def philox4x32_10(ctr, key):
    c = (ctypes.c_uint32 * 4)(*ctr)
    k = (ctypes.c_uint32 * 2)(*key)
    o = (ctypes.c_uint32 * 4)()
    lib().kmo_philox4x32_10(c, k, o)
    return list(o)


def kmpp_draw(seed, rnd):
    return int(lib().kmo_kmpp_draw(seed, rnd))


def quant_exponent(max_weight, n):
    return int(lib().kmo_quant_exponent(max_weight, n))


def assign(X, C, n_threads=None, return_dist=False):
    """int32 labels of the nearest center (float32 sequential distances)."""
    X = _f32(X)
    C = _f32(C)
    n, d = X.shape
    k = C.shape[0]
    labels = np.empty(n, dtype=np.int32)
    dist = np.empty(n, dtype=np.float32) if return_dist else None
    rc = lib().kmo_assign(_ptr(X), n, d, _ptr(C), k, _ptr(labels), _ptr(dist),
                          n_threads or default_threads())
    _check(rc, "assign")
    return (labels, dist) if return_dist else labels


def update(X, labels, C_old):
    """One centroid update; returns (new centers, counts, inertia, per-cluster inertia)."""
    X = _f32(X)
    C_old = _f32(C_old)
    labels = np.ascontiguousarray(labels, dtype=np.int32)
    n, d = X.shape
    k = C_old.shape[0]
    C_new = np.empty_like(C_old)
    counts = np.empty(k, dtype=np.int64)
    cost = np.zeros(1, dtype=np.float64)
    ccost = np.empty(k, dtype=np.float64)
    rc = lib().kmo_update(_ptr(X), n, d, _ptr(labels), k, _ptr(C_old), _ptr(C_new),
                          _ptr(counts), _ptr(cost), _ptr(ccost))
    _check(rc, "update")
    return C_new, counts, float(cost[0]), ccost


def lloyd(X, C0, max_iter, tol, n_threads=None):
    """Lloyd iterations from C0; returns dict(centers, labels, inertias, n_iter, converged)."""
    X = _f32(X)
    C = _f32(C0).copy()
    n, d = X.shape
    k = C.shape[0]
    labels = np.zeros(n, dtype=np.int32)
    inertias = np.zeros(max(1, max_iter), dtype=np.float64)
    n_iter = np.zeros(1, dtype=np.int32)
    conv = np.zeros(1, dtype=np.int32)
    rc = lib().kmo_lloyd(_ptr(X), n, d, k, _ptr(C), max_iter, float(tol), _ptr(labels),
                         _ptr(inertias), _ptr(n_iter), _ptr(conv), n_threads or default_threads())
    _check(rc, "lloyd")
    it = int(n_iter[0])
    return dict(centers=C, labels=labels, inertias=inertias[:it].copy(), n_iter=it,
                converged=bool(conv[0]))


def kmpp(X, k, seed, n_threads=None):
    """kmeans++ initial centers; returns (centers (k,d) float32, frame indices)."""
    X = _f32(X)
    n, d = X.shape
    C0 = np.empty((k, d), dtype=np.float32)
    idx = np.empty(k, dtype=np.int64)
    rc = lib().kmo_kmpp(_ptr(X), n, d, k, int(seed) & 0xFFFFFFFF, _ptr(C0), _ptr(idx),
                        n_threads or default_threads())
    _check(rc, "kmpp")
    return C0, idx


def regspace(X, dmin, max_centers):
    """Regular space centers in frame order; returns (centers, converged)."""
    X = _f32(X)
    n, d = X.shape
    C = np.empty((max(1, max_centers), d), dtype=np.float32)
    nc = np.zeros(1, dtype=np.int32)
    conv = np.zeros(1, dtype=np.int32)
    rc = lib().kmo_regspace(_ptr(X), n, d, float(dmin), int(max_centers), _ptr(C), _ptr(nc), _ptr(conv))
    _check(rc, "regspace")
    return C[:int(nc[0])].copy(), bool(conv[0])


def regspace_minrmsd(X, dmin, max_centers):
    """Regular space centers under the minRMSD metric; returns (centers, converged)."""
    X = _f32(X)
    n, d = X.shape
    C = np.empty((max(1, max_centers), d), dtype=np.float32)
    nc = np.zeros(1, dtype=np.int32)
    conv = np.zeros(1, dtype=np.int32)
    rc = lib().kmo_regspace_minrmsd(_ptr(X), n, d, float(dmin), int(max_centers), _ptr(C), _ptr(nc), _ptr(conv))
    _check(rc, "regspace_minrmsd")
    return C[:int(nc[0])].copy(), bool(conv[0])


def count_matrix(dtrajs, lag, sliding=True, nstates=None):
    """Dense lag-`lag` transition counts, as deeptime's count_matrix builds
    them (rows dtraj[0:-lag] or dtraj[0:-lag:lag], columns dtraj[lag:] or
    dtraj[lag::lag]; pairs with a negative state dropped)."""
    dtrajs = [np.asarray(d, dtype=np.int64) for d in dtrajs]
    if nstates is None:
        nstates = max((int(d.max()) for d in dtrajs if len(d)), default=-1) + 1
    C = np.zeros((nstates, nstates), dtype=np.int64)
    for d in dtrajs:
        if len(d) <= lag:
            continue
        if sliding:
            row, col = d[:-lag], d[lag:]
        else:
            row, col = d[0:-lag:lag], d[lag::lag]
        keep = (row >= 0) & (col >= 0) & (row < nstates) & (col < nstates)
        np.add.at(C, (row[keep], col[keep]), 1)
    return C


def assign_minrmsd(X, C, n_threads=None, return_msd=False):
    """int32 labels of the nearest center under the minRMSD metric (d = 3 n_atoms, atom-major)."""
    X = _f32(X)
    C = _f32(C)
    n, d = X.shape
    labels = np.empty(n, dtype=np.int32)
    msd = np.empty(n, dtype=np.float64) if return_msd else None
    _check(lib().kmo_assign_minrmsd(_ptr(X), n, d, _ptr(C), C.shape[0], _ptr(labels), _ptr(msd),
                                    n_threads or default_threads()), "assign_minrmsd")
    return (labels, msd) if return_msd else labels


def minrmsd_rows(X, Y):
    """float32 minRMSD of the row pairs (X[i], Y[i]) (compute_metric)."""
    X = _f32(np.atleast_2d(X))
    Y = _f32(np.atleast_2d(Y))
    out = np.empty(X.shape[0], dtype=np.float32)
    _check(lib().kmo_minrmsd_rows(_ptr(X), _ptr(Y), X.shape[0], X.shape[1], _ptr(out)), "minrmsd_rows")
    return out


def rmsd_center(x):
    """(centered float32 row, trace G) of one atom-major row."""
    x = _f32(x).ravel()
    a = np.empty_like(x)
    g = lib().kmo_rmsd_center(_ptr(x), x.size // 3, _ptr(a))
    return a, g


def lloyd_minrmsd(X, C0, max_iter, tol, n_threads=None):
    """Lloyd iterations under the minRMSD metric (mean update); as lloyd()."""
    X = _f32(X)
    C = _f32(C0).copy()
    n, d = X.shape
    k = C.shape[0]
    labels = np.zeros(n, dtype=np.int32)
    inertias = np.zeros(max(1, max_iter), dtype=np.float64)
    n_iter = np.zeros(1, dtype=np.int32)
    conv = np.zeros(1, dtype=np.int32)
    _check(lib().kmo_lloyd_minrmsd(_ptr(X), n, d, k, _ptr(C), max_iter, float(tol), _ptr(labels), _ptr(inertias),
                                   _ptr(n_iter), _ptr(conv), n_threads or default_threads()), "lloyd_minrmsd")
    it = int(n_iter[0])
    return dict(centers=C, labels=labels, inertias=inertias[:it].copy(), n_iter=it, converged=bool(conv[0]))


def kmpp_minrmsd(X, k, seed, n_threads=None):
    """kmeans++ under the minRMSD metric; returns (centers, frame indices)."""
    X = _f32(X)
    n, d = X.shape
    C0 = np.empty((k, d), dtype=np.float32)
    idx = np.empty(k, dtype=np.int64)
    _check(lib().kmo_kmpp_minrmsd(_ptr(X), n, d, k, int(seed) & 0xFFFFFFFF, _ptr(C0), _ptr(idx),
                                  n_threads or default_threads()), "kmpp_minrmsd")
    return C0, idx


def kabsch_rmsd_fp64(x, y):
    """Independent float64 check of minRMSD: optimal rotation by SVD (Kabsch)."""
    a = np.asarray(x, dtype=np.float64).reshape(-1, 3)
    b = np.asarray(y, dtype=np.float64).reshape(-1, 3)
    a = a - a.mean(axis=0)
    b = b - b.mean(axis=0)
    u, s, vt = np.linalg.svd(a.T @ b)
    sign = np.sign(np.linalg.det(u @ vt))
    s[-1] *= sign
    msd = (np.sum(a * a) + np.sum(b * b) - 2.0 * np.sum(s)) / a.shape[0]
    return float(np.sqrt(max(msd, 0.0)))


def pair_distances(xyz, pairs):
    """Atom-pair distances in float32 with each operation rounded on its own:
    sqrt((dx*dx + dy*dy) + dz*dz), d = xyz[:, j] - xyz[:, i]
    (mdtraj.compute_distances without a unit cell, as called from
    pyemma/coordinates/data/featurization/distances.py:53-54)."""
    xyz = np.asarray(xyz, dtype=np.float32)
    pairs = np.asarray(pairs, dtype=np.int64).reshape(-1, 2)
    d = xyz[:, pairs[:, 1], :] - xyz[:, pairs[:, 0], :]
    r2 = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]
    return np.sqrt(r2).astype(np.float32)


# ---------------------------------------------------------------------------
# float64 NumPy reference (independent of the C code)
# ---------------------------------------------------------------------------
_CHUNK_FP64 = 1 << 16


def _chunks_fp64(n, fn, n_threads=None):
    """fn(a, b) over the row chunks [a, b) of n rows on a thread pool (NumPy
    releases the interpreter lock inside its array loops); returns the
    results in chunk order."""
    from concurrent.futures import ThreadPoolExecutor
    bounds = [(a, min(n, a + _CHUNK_FP64)) for a in range(0, n, _CHUNK_FP64)]
    workers = max(1, min(len(bounds), n_threads or default_threads()))
    if workers == 1:
        return [fn(a, b) for a, b in bounds]
    with ThreadPoolExecutor(max_workers=workers) as ex:
        return list(ex.map(lambda ab: fn(*ab), bounds))


def centers_fp64(X, labels, C_old, n_threads=None):
    """Member means in float64; empty clusters keep their previous center.

    Works through X in chunks of 65,536 rows (each converted to float64 on
    its own), so that a 2,000,000 x 528 float32 X needs no float64 copy of
    the whole array.  Within a chunk the rows are summed cluster by cluster
    in frame order (np.add.reduceat over the rows sorted by label); the
    chunk sums are added in chunk order."""
    labels = np.asarray(labels).astype(np.int64, copy=False)
    k, d = C_old.shape
    cnt = np.bincount(labels, minlength=k).astype(np.float64)[:k]

    def part(a, b):
        lab = labels[a:b]
        order = np.argsort(lab, kind="stable")
        ls = lab[order]
        starts = np.flatnonzero(np.r_[True, ls[1:] != ls[:-1]])
        return ls[starts], np.add.reduceat(np.asarray(X[a:b], dtype=np.float64)[order], starts, axis=0)

    S = np.zeros((k, d))
    for rows, sums in _chunks_fp64(len(labels), part, n_threads):
        S[rows] += sums
    out = np.asarray(C_old, dtype=np.float64).copy()
    nz = cnt > 0
    out[nz] = S[nz] / cnt[nz, None]
    return out, cnt


def inertia_fp64(X, labels, C, n_threads=None):
    """sum_i ||x_i - c_{label_i}||^2 in float64 (chunks of 65,536 rows, added
    in chunk order)."""
    labels = np.asarray(labels).astype(np.int64, copy=False)
    C = np.asarray(C, dtype=np.float64)

    def part(a, b):
        diff = np.asarray(X[a:b], dtype=np.float64) - C[labels[a:b]]
        return float(np.einsum("ij,ij->", diff, diff))

    return float(sum(_chunks_fp64(len(labels), part, n_threads)))


def sqdist_fp32_sequential(X, C):
    """(n, k) float32 distances with the oracle's feature order (slow; small cases only)."""
    X = np.asarray(X, dtype=np.float32)
    C = np.asarray(C, dtype=np.float32)
    acc = np.zeros((X.shape[0], C.shape[0]), dtype=np.float32)
    for f in range(X.shape[1]):
        t = X[:, f][:, None] - C[:, f][None, :]
        acc = acc + t * t
    return acc
