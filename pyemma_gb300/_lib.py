"""ctypes binding of libkmgpu.so (the C ABI in include/kmgpu.h).

Device buffers are torch tensors; only raw pointers, sizes and the CUDA
stream handle cross the boundary.  There is no CPU implementation behind
these functions: without the library or without a CUDA device every call
raises.
"""
import ctypes
import os

import numpy as np

from . import _build

PRECISIONS = {"fp32": 0, "fp16": 1, "auto": 2, "bf16": 3, "fp8": 4}
PRECISION_NAMES = {v: k for k, v in PRECISIONS.items()}

KM_OK = 0
KM_ERR_BAD_SHAPE = 1
KM_ERR_WORKSPACE = 2
KM_ERR_NON_FINITE = 3
KM_ERR_TIMEOUT = 4
KM_ERR_CUDA = 5
KM_ERR_UNSUPPORTED = 6
KM_ERR_BAD_LABEL = 7
KM_PENDING = 8

EXPORTED = (
    "km_version", "km_status_string", "km_last_error", "km_profile_enable", "km_profile_read",
    "km_debug_fake_device_error",
    "km_assign_workspace_size", "km_assign", "km_batch_assign", "km_debug_tc_distances",
    "km_update_workspace_size", "km_update", "km_update_noalloc_max_bytes", "km_update_noalloc",
    "km_kmpp_workspace_size", "km_kmpp",
    "km_lloyd_workspace_size", "km_lloyd", "km_lloyd_host",
    "km_centers_create", "km_centers_destroy", "km_centers_info", "km_assign_centers_workspace_size",
    "km_assign_centers",
    "km_serve_create", "km_serve_add_centers", "km_serve_submit", "km_serve_poll", "km_serve_stats_read",
    "km_serve_shutdown", "km_tune_workspace_size", "km_tune", "km_tune_clear", "km_tune_tiles", "km_tile_plan_get",
    "km_debug_force_tile_plan",
    "km_regspace_workspace_size", "km_regspace", "km_count_matrix_workspace_size", "km_count_matrix",
    "km_pair_distances", "km_assign_pairs_workspace_size", "km_assign_pairs", "km_lloyd_pairs_workspace_size",
    "km_lloyd_pairs", "km_kmpp_pairs_workspace_size", "km_kmpp_pairs", "km_assign_minrmsd_workspace_size", "km_assign_minrmsd", "km_minrmsd_rows_workspace_size",
    "km_minrmsd_rows", "km_kmpp_minrmsd_workspace_size", "km_kmpp_minrmsd", "km_lloyd_minrmsd_workspace_size",
    "km_lloyd_minrmsd",
)


class KmError(RuntimeError):
    """A libkmgpu call returned a non-zero km_status."""

    def __init__(self, status, message):
        super().__init__(message)
        self.status = status


class AssignStats(ctypes.Structure):
    _fields_ = [("n_frames", ctypes.c_int64), ("n_recheck", ctypes.c_int64),
                ("n_full", ctypes.c_int64), ("n_flipped", ctypes.c_int64),
                ("precision", ctypes.c_int32), ("reserved", ctypes.c_int32), ("n_pairs", ctypes.c_int64)]

    def as_dict(self):
        return dict(n_frames=self.n_frames, n_recheck=self.n_recheck, n_full=self.n_full,
                    n_flipped=self.n_flipped, n_pairs=self.n_pairs,
                    precision=PRECISION_NAMES.get(self.precision, "?"))


CALLBACK = ctypes.CFUNCTYPE(None, ctypes.c_void_p)


class TilePlan(ctypes.Structure):
    _fields_ = [("bn", ctypes.c_int32), ("pair", ctypes.c_int32), ("stages", ctypes.c_int32),
                ("list_len", ctypes.c_int32), ("ms", ctypes.c_double)]

    def as_dict(self):
        return dict(bn=self.bn, pair=self.pair, stages=self.stages, list_len=self.list_len, ms=self.ms)


class ServeConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_int64), ("max_batch_frames", ctypes.c_int64),
                ("device", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class RequestInfo(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("set_id", ctypes.c_int32), ("n_frames", ctypes.c_int64),
                ("batch_frames", ctypes.c_int64), ("queue_ms", ctypes.c_double), ("total_ms", ctypes.c_double)]

    def as_dict(self):
        return dict(status=self.status, set_id=self.set_id, n_frames=self.n_frames,
                    batch_frames=self.batch_frames, queue_ms=self.queue_ms, total_ms=self.total_ms)


class ServeStats(ctypes.Structure):
    _fields_ = [("batches", ctypes.c_int64), ("frames", ctypes.c_int64), ("requests", ctypes.c_int64),
                ("batch_cap_frames", ctypes.c_int64), ("device_bytes", ctypes.c_int64)]

    def as_dict(self):
        return {name: getattr(self, name) for name, _ in self._fields_}

_lib = None


def library_path():
    return _build.LIB_PATH


def load(build_if_missing=False):
    """Loads libkmgpu.so and declares its signatures."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    if not os.path.exists(path):
        if build_if_missing:
            _build.build()
        else:
            raise ImportError("libkmgpu.so is not built (%s); run __graft_entry__.build()" % path)
    L = ctypes.CDLL(path)
    P, i64, i32, u32, f64 = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_uint32, ctypes.c_double
    sz = ctypes.c_size_t
    L.km_version.restype = ctypes.c_int
    L.km_status_string.argtypes = [ctypes.c_int]
    L.km_status_string.restype = ctypes.c_char_p
    L.km_last_error.restype = ctypes.c_char_p
    L.km_profile_enable.argtypes = [ctypes.c_int]
    L.km_profile_enable.restype = ctypes.c_int
    L.km_profile_read.argtypes = [i32, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64)]
    L.km_profile_read.restype = ctypes.c_int
    L.km_debug_fake_device_error.argtypes = [u32]
    L.km_debug_fake_device_error.restype = ctypes.c_int
    L.km_assign_workspace_size.argtypes = [i64, i32, i32, i32]
    L.km_assign_workspace_size.restype = sz
    L.km_assign.argtypes = [P, i64, i32, P, i32, i32, P, P, sz, ctypes.POINTER(AssignStats), P]
    L.km_debug_tc_distances.argtypes = [P, i64, i32, P, i32, i32, P, P, P, P, sz, P]
    L.km_debug_tc_distances.restype = ctypes.c_int
    L.km_batch_assign.argtypes = [P, P, i32, i32, P, i32, i32, P, P, sz, ctypes.POINTER(AssignStats), P]
    L.km_update_workspace_size.argtypes = [i64, i32, i32]
    L.km_update_workspace_size.restype = sz
    L.km_update.argtypes = [P, i64, i32, P, i32, P, P, P, P, P, sz, P]
    L.km_update_noalloc_max_bytes.restype = sz
    L.km_update_noalloc.argtypes = [P, i64, i32, P, i32, P, P, P, P, P]
    L.km_update_noalloc.restype = ctypes.c_int
    L.km_kmpp_workspace_size.argtypes = [i64, i32, i32]
    L.km_kmpp_workspace_size.restype = sz
    L.km_kmpp.argtypes = [P, i64, i32, i32, u32, P, P, CALLBACK, P, P, sz, P]
    L.km_lloyd_workspace_size.argtypes = [i64, i32, i32, i32]
    L.km_lloyd_workspace_size.restype = sz
    L.km_lloyd.argtypes = [P, i64, i32, i32, P, i32, f64, i32, P, P, P, P, CALLBACK, P, P, sz, P]
    L.km_lloyd_host.argtypes = [P, P, i32, P, i64, i32, i32, P, i32, f64, i32, P, P, P, P, CALLBACK, P, P, sz, P]
    for name, args in (("km_assign_minrmsd_workspace_size", [i64, i32, i32]),
                       ("km_minrmsd_rows_workspace_size", [i64, i32]),
                       ("km_kmpp_minrmsd_workspace_size", [i64, i32, i32]),
                       ("km_lloyd_minrmsd_workspace_size", [i64, i32, i32])):
        getattr(L, name).argtypes = args
        getattr(L, name).restype = sz
    L.km_assign_minrmsd.argtypes = [P, i64, i32, P, i32, P, P, P, sz, P]
    L.km_minrmsd_rows.argtypes = [P, P, i64, i32, P, P, sz, P]
    L.km_kmpp_minrmsd.argtypes = [P, i64, i32, i32, u32, P, P, CALLBACK, P, P, sz, P]
    L.km_lloyd_minrmsd.argtypes = [P, i64, i32, i32, P, i32, f64, P, P, P, P, CALLBACK, P, P, sz, P]
    pp = ctypes.POINTER(ctypes.c_void_p)
    L.km_centers_create.argtypes = [P, i32, i32, i32, P, pp]
    L.km_centers_destroy.argtypes = [P]
    L.km_centers_info.argtypes = [P, ctypes.POINTER(i32), ctypes.POINTER(i32), ctypes.POINTER(i32),
                                  ctypes.POINTER(i64)]
    L.km_assign_centers_workspace_size.argtypes = [i64, P]
    L.km_assign_centers_workspace_size.restype = sz
    L.km_assign_centers.argtypes = [P, i64, i32, P, P, P, sz, ctypes.POINTER(AssignStats), P]
    L.km_serve_create.argtypes = [ctypes.POINTER(ServeConfig), pp]
    L.km_serve_add_centers.argtypes = [P, P, ctypes.POINTER(i32)]
    L.km_serve_submit.argtypes = [P, i32, P, i64, i32, P, ctypes.POINTER(ctypes.c_uint64)]
    L.km_serve_poll.argtypes = [P, ctypes.c_uint64, i32, ctypes.POINTER(RequestInfo)]
    L.km_serve_stats_read.argtypes = [P, ctypes.POINTER(ServeStats)]
    L.km_serve_shutdown.argtypes = [P]
    L.km_tune_workspace_size.argtypes = [i64, i32, i32]
    L.km_tune_workspace_size.restype = sz
    L.km_tune.argtypes = [P, i64, i32, P, i32, P, sz, ctypes.POINTER(i32), ctypes.POINTER(f64),
                          ctypes.POINTER(f64), P]
    L.km_tune.restype = ctypes.c_int
    L.km_tune_clear.restype = ctypes.c_int
    L.km_assign_pairs_workspace_size.argtypes = [i64, i32, i32, i32]
    L.km_assign_pairs_workspace_size.restype = sz
    L.km_assign_pairs.argtypes = [P, i64, i32, P, i32, P, i32, i32, P, P, sz, ctypes.POINTER(AssignStats), P]
    L.km_assign_pairs.restype = ctypes.c_int
    L.km_lloyd_pairs_workspace_size.argtypes = [i64, i32, i32, i32]
    L.km_lloyd_pairs_workspace_size.restype = sz
    L.km_lloyd_pairs.argtypes = [P, i64, i32, P, i32, i32, P, i32, f64, i32, P, P, P, P, CALLBACK, P, P, sz, P]
    L.km_lloyd_pairs.restype = ctypes.c_int
    L.km_kmpp_pairs_workspace_size.argtypes = [i64, i32, i32]
    L.km_kmpp_pairs_workspace_size.restype = sz
    L.km_kmpp_pairs.argtypes = [P, i64, i32, P, i32, i32, u32, P, P, CALLBACK, P, P, sz, P]
    L.km_kmpp_pairs.restype = ctypes.c_int
    L.km_tune_tiles.argtypes = [P, i64, i32, P, i32, i32, P, sz, ctypes.POINTER(TilePlan), ctypes.POINTER(TilePlan),
                                i32, ctypes.POINTER(i32), P]
    L.km_tune_tiles.restype = ctypes.c_int
    L.km_tile_plan_get.argtypes = [i32, i32, ctypes.POINTER(TilePlan), ctypes.POINTER(i32)]
    L.km_tile_plan_get.restype = ctypes.c_int
    L.km_debug_force_tile_plan.argtypes = [ctypes.POINTER(TilePlan)]
    L.km_debug_force_tile_plan.restype = ctypes.c_int
    L.km_regspace_workspace_size.argtypes = [i32]
    L.km_regspace_workspace_size.restype = sz
    L.km_regspace.argtypes = [P, i64, i32, f64, i32, P, ctypes.POINTER(i32), ctypes.POINTER(i32), P, sz, P]
    L.km_regspace.restype = ctypes.c_int
    L.km_count_matrix_workspace_size.argtypes = [i32]
    L.km_count_matrix_workspace_size.restype = sz
    L.km_count_matrix.argtypes = [P, P, i32, i32, i32, i32, P, P, sz, P]
    L.km_count_matrix.restype = ctypes.c_int
    L.km_pair_distances.argtypes = [P, i64, i32, P, i32, P, P]
    L.km_pair_distances.restype = ctypes.c_int
    for name in ("km_assign", "km_batch_assign", "km_update", "km_kmpp", "km_lloyd", "km_lloyd_host",
                 "km_assign_minrmsd", "km_minrmsd_rows", "km_kmpp_minrmsd", "km_lloyd_minrmsd",
                 "km_centers_create",
                 "km_centers_destroy", "km_centers_info", "km_assign_centers", "km_serve_create",
                 "km_serve_add_centers", "km_serve_submit", "km_serve_poll", "km_serve_stats_read",
                 "km_serve_shutdown"):
        getattr(L, name).restype = ctypes.c_int
    _lib = L
    return L


PROFILE_KINDS = {"tc": 0, "fp32": 1, "recheck": 2, "update": 3, "full_recheck": 4}


def profile_enable(on=True):
    """Starts (or stops) CUDA-event timing of the main kernels; resets the totals."""
    check(load().km_profile_enable(1 if on else 0))


def profile_read():
    """{kind: (total ms, launches)} since the last profile_enable."""
    L = load()
    out = {}
    for name, kind in PROFILE_KINDS.items():
        ms, n = ctypes.c_double(), ctypes.c_int64()
        check(L.km_profile_read(kind, ctypes.byref(ms), ctypes.byref(n)))
        out[name] = (ms.value, n.value)
    return out


def check(rc):
    if rc != KM_OK:
        L = load()
        raise KmError(rc, "libkmgpu: %s: %s" % (L.km_status_string(rc).decode(),
                                                L.km_last_error().decode()))


# ---------------------------------------------------------------------------
# torch-facing helpers
# ---------------------------------------------------------------------------
def _torch():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("pyemma_gb300 needs a CUDA device; none is available")
    return torch


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream(torch, device):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def _workspace(torch, nbytes, device):
    if nbytes == 0:
        return None
    return torch.empty(int(nbytes), dtype=torch.uint8, device=device)


def precision_code(precision):
    if isinstance(precision, str):
        try:
            return PRECISIONS[precision.lower()]
        except KeyError:
            raise ValueError("precision must be one of %s" % sorted(PRECISIONS))
    return int(precision)


def _check_frames(torch, X, name="X"):
    if X.device.type != "cuda" or X.dtype != torch.float32 or X.dim() != 2 or not X.is_contiguous():
        raise ValueError("%s must be a contiguous float32 (n, d) CUDA tensor" % name)


def assign(X, C, precision="auto", labels=None):
    """Labels (int32 CUDA tensor) of the nearest center for every row of X."""
    torch = _torch()
    L = load()
    _check_frames(torch, X)
    _check_frames(torch, C, "C")
    n, d = X.shape
    k = C.shape[0]
    if C.shape[1] != d:
        raise ValueError("centers have dimension %d, frames %d" % (C.shape[1], d))
    p = precision_code(precision)
    if labels is None:
        labels = torch.empty(n, dtype=torch.int32, device=X.device)
    ws_bytes = L.km_assign_workspace_size(n, d, k, p)
    ws = _workspace(torch, ws_bytes, X.device)
    stats = AssignStats()
    check(L.km_assign(_ptr(X), n, d, _ptr(C), k, p, _ptr(labels), _ptr(ws), ws_bytes, ctypes.byref(stats),
                      _stream(torch, X.device)))
    return labels, stats.as_dict()


WAIT_SLOTS = ("producer_b", "producer_a", "mma_b", "mma_a", "mma_acc", "epilogue_acc", "epilogue_total",
              "mma_total")


def debug_tc_distances(X, C, distances=True, precision="fp16"):
    """(labels, V or None, wait cycles): the tensor-core assignment in the
    given precision (fp16, bf16 or fp8), its n x k approximate distances and
    the cycles each kernel role spent waiting."""
    torch = _torch()
    L = load()
    _check_frames(torch, X)
    _check_frames(torch, C, "C")
    n, d = X.shape
    k = C.shape[0]
    V = torch.empty((n, k), dtype=torch.float32, device=X.device) if distances else None
    labels = torch.empty(n, dtype=torch.int32, device=X.device)
    ws_bytes = L.km_assign_workspace_size(n, d, k, PRECISIONS["fp16"])
    ws = _workspace(torch, ws_bytes, X.device)
    wait = (ctypes.c_uint64 * 8)()
    check(L.km_debug_tc_distances(_ptr(X), n, d, _ptr(C), k, precision_code(precision), _ptr(V), _ptr(labels), wait,
                                  _ptr(ws), ws_bytes, _stream(torch, X.device)))
    return labels, V, dict(zip(WAIT_SLOTS, list(wait)))


def batch_assign(X_packed, offsets, C, precision="auto", labels=None):
    """Assignment of trajectories packed back to back; offsets has n_traj+1 entries."""
    torch = _torch()
    L = load()
    _check_frames(torch, X_packed)
    _check_frames(torch, C, "C")
    offs = np.ascontiguousarray(offsets, dtype=np.int64)
    n_traj = len(offs) - 1
    n, d = X_packed.shape
    if n_traj < 0 or (n_traj >= 0 and offs[-1] != n):
        raise ValueError("offsets must end at the number of packed frames")
    k = C.shape[0]
    p = precision_code(precision)
    if labels is None:
        labels = torch.empty(n, dtype=torch.int32, device=X_packed.device)
    ws_bytes = L.km_assign_workspace_size(n, d, k, p)
    ws = _workspace(torch, ws_bytes, X_packed.device)
    stats = AssignStats()
    check(L.km_batch_assign(_ptr(X_packed), offs.ctypes.data_as(ctypes.c_void_p), n_traj, d, _ptr(C), k, p,
                            _ptr(labels), _ptr(ws), ws_bytes, ctypes.byref(stats),
                            _stream(torch, X_packed.device)))
    return labels, stats.as_dict()


def update(X, labels, C_old):
    """One centroid update; returns (C_new, counts int64, inertia float)."""
    torch = _torch()
    L = load()
    _check_frames(torch, X)
    n, d = X.shape
    k = C_old.shape[0]
    C_new = torch.empty_like(C_old)
    counts = torch.empty(k, dtype=torch.int64, device=X.device)
    cost = torch.empty(1, dtype=torch.float64, device=X.device)
    ws_bytes = L.km_update_workspace_size(n, d, k)
    ws = _workspace(torch, ws_bytes, X.device)
    check(L.km_update(_ptr(X), n, d, _ptr(labels), k, _ptr(C_old), _ptr(C_new), _ptr(counts), _ptr(cost),
                      _ptr(ws), ws_bytes, _stream(torch, X.device)))
    return C_new, counts, float(cost.item())


def _callback(fn):
    if fn is None:
        return CALLBACK(0), None
    cb = CALLBACK(lambda _user: fn())
    return cb, cb


def kmpp(X, k, seed, callback=None):
    """kmeans++ initial centers (k, d) and chosen frame indices."""
    torch = _torch()
    L = load()
    _check_frames(torch, X)
    n, d = X.shape
    C0 = torch.empty((k, d), dtype=torch.float32, device=X.device)
    idx = torch.empty(k, dtype=torch.int64, device=X.device)
    ws_bytes = L.km_kmpp_workspace_size(n, d, k)
    ws = _workspace(torch, ws_bytes, X.device)
    cb, keep = _callback(callback)
    check(L.km_kmpp(_ptr(X), n, d, k, int(seed) & 0xFFFFFFFF, _ptr(C0), _ptr(idx), cb, None, _ptr(ws),
                    ws_bytes, _stream(torch, X.device)))
    del keep
    return C0, idx


def lloyd(X, C, max_iter, tolerance, precision="auto", callback=None, labels=None):
    """Lloyd iterations in place on C; returns dict(labels, inertias, n_iter, converged)."""
    torch = _torch()
    L = load()
    _check_frames(torch, X)
    _check_frames(torch, C, "C")
    n, d = X.shape
    k = C.shape[0]
    p = precision_code(precision)
    if labels is None:
        labels = torch.empty(n, dtype=torch.int32, device=X.device)
    inertias = np.zeros(max(1, max_iter), dtype=np.float64)
    n_iter = ctypes.c_int32(0)
    conv = ctypes.c_int32(0)
    ws_bytes = L.km_lloyd_workspace_size(n, d, k, p)
    ws = _workspace(torch, ws_bytes, X.device)
    cb, keep = _callback(callback)
    check(L.km_lloyd(_ptr(X), n, d, k, _ptr(C), int(max_iter), float(tolerance), p, _ptr(labels),
                     inertias.ctypes.data_as(ctypes.c_void_p), ctypes.byref(n_iter), ctypes.byref(conv), cb,
                     None, _ptr(ws), ws_bytes, _stream(torch, X.device)))
    del keep
    return dict(labels=labels, inertias=inertias[:n_iter.value].copy(), n_iter=n_iter.value,
                converged=bool(conv.value))


def lloyd_host(parts, C, max_iter, tolerance, precision="auto", callback=None, X=None, labels=None):
    """Lloyd iterations on frames in host memory, in place on C.

    ``parts`` is a list of (T_i, d) float32 C-contiguous numpy arrays (pinned
    memory gives an overlapped copy).  They are copied into the device tensor
    ``X`` (allocated when None) while the first iteration assigns the frames
    already copied.  Returns dict(X, labels, inertias, n_iter, converged).
    """
    torch = _torch()
    L = load()
    _check_frames(torch, C, "C")
    d = C.shape[1]
    k = C.shape[0]
    arrs = []
    for a in parts:
        if not (isinstance(a, np.ndarray) and a.dtype == np.float32 and a.flags["C_CONTIGUOUS"] and a.ndim == 2
                and a.shape[1] == d):
            raise ValueError("host parts must be C-contiguous float32 arrays of shape (T, %d)" % d)
        if len(a):
            arrs.append(a)
    n = int(sum(len(a) for a in arrs))
    if X is None:
        X = torch.empty((n, d), dtype=torch.float32, device=C.device)
    _check_frames(torch, X)
    if X.shape[0] != n or X.shape[1] != d:
        raise ValueError("X must have shape (%d, %d)" % (n, d))
    p = precision_code(precision)
    if labels is None:
        labels = torch.empty(n, dtype=torch.int32, device=C.device)
    ptrs = (ctypes.c_void_p * max(1, len(arrs)))(*[a.ctypes.data for a in arrs])
    rows = np.array([len(a) for a in arrs] or [0], dtype=np.int64)
    inertias = np.zeros(max(1, max_iter), dtype=np.float64)
    n_iter = ctypes.c_int32(0)
    conv = ctypes.c_int32(0)
    ws_bytes = L.km_lloyd_workspace_size(n, d, k, p)
    ws = _workspace(torch, ws_bytes, C.device)
    cb, keep = _callback(callback)
    check(L.km_lloyd_host(ptrs, rows.ctypes.data_as(ctypes.c_void_p), len(arrs), _ptr(X), n, d, k, _ptr(C),
                          int(max_iter), float(tolerance), p, _ptr(labels),
                          inertias.ctypes.data_as(ctypes.c_void_p), ctypes.byref(n_iter), ctypes.byref(conv), cb,
                          None, _ptr(ws), ws_bytes, _stream(torch, C.device)))
    del keep
    return dict(X=X, labels=labels, inertias=inertias[:n_iter.value].copy(), n_iter=n_iter.value,
                converged=bool(conv.value))


# ---------------------------------------------------------------------------
# the minRMSD metric (atom-major rows, d = 3 n_atoms)
# ---------------------------------------------------------------------------
def assign_minrmsd(X, C, labels=None, return_rmsd=False):
    """Labels of the nearest center under the minRMSD metric (and, when asked,
    the metric value to it)."""
    torch = _torch()
    L = load()
    _check_frames(torch, X)
    _check_frames(torch, C, "C")
    n, d = X.shape
    k = C.shape[0]
    if labels is None:
        labels = torch.empty(n, dtype=torch.int32, device=X.device)
    rmsd = torch.empty(n, dtype=torch.float32, device=X.device) if return_rmsd else None
    ws_bytes = L.km_assign_minrmsd_workspace_size(n, d, k)
    ws = _workspace(torch, ws_bytes, X.device)
    check(L.km_assign_minrmsd(_ptr(X), n, d, _ptr(C), k, _ptr(labels), _ptr(rmsd), _ptr(ws), ws_bytes,
                              _stream(torch, X.device)))
    return (labels, rmsd) if return_rmsd else labels


def minrmsd_rows(X, Y):
    """float32 minRMSD of the row pairs (X[i], Y[i])."""
    torch = _torch()
    L = load()
    _check_frames(torch, X)
    _check_frames(torch, Y, "Y")
    n, d = X.shape
    if tuple(Y.shape) != (n, d):
        raise ValueError("X and Y must have the same shape")
    out = torch.empty(n, dtype=torch.float32, device=X.device)
    ws_bytes = L.km_minrmsd_rows_workspace_size(n, d)
    ws = _workspace(torch, ws_bytes, X.device)
    check(L.km_minrmsd_rows(_ptr(X), _ptr(Y), n, d, _ptr(out), _ptr(ws), ws_bytes, _stream(torch, X.device)))
    return out


def kmpp_minrmsd(X, k, seed, callback=None):
    """kmeans++ initial centers under the minRMSD metric and the chosen frame indices."""
    torch = _torch()
    L = load()
    _check_frames(torch, X)
    n, d = X.shape
    C0 = torch.empty((k, d), dtype=torch.float32, device=X.device)
    idx = torch.empty(k, dtype=torch.int64, device=X.device)
    ws_bytes = L.km_kmpp_minrmsd_workspace_size(n, d, k)
    ws = _workspace(torch, ws_bytes, X.device)
    cb, keep = _callback(callback)
    check(L.km_kmpp_minrmsd(_ptr(X), n, d, k, int(seed) & 0xFFFFFFFF, _ptr(C0), _ptr(idx), cb, None, _ptr(ws),
                            ws_bytes, _stream(torch, X.device)))
    del keep
    return C0, idx


def lloyd_minrmsd(X, C, max_iter, tolerance, callback=None, labels=None):
    """Lloyd iterations under the minRMSD metric, in place on C."""
    torch = _torch()
    L = load()
    _check_frames(torch, X)
    _check_frames(torch, C, "C")
    n, d = X.shape
    k = C.shape[0]
    if labels is None:
        labels = torch.empty(n, dtype=torch.int32, device=X.device)
    inertias = np.zeros(max(1, max_iter), dtype=np.float64)
    n_iter = ctypes.c_int32(0)
    conv = ctypes.c_int32(0)
    ws_bytes = L.km_lloyd_minrmsd_workspace_size(n, d, k)
    ws = _workspace(torch, ws_bytes, X.device)
    cb, keep = _callback(callback)
    check(L.km_lloyd_minrmsd(_ptr(X), n, d, k, _ptr(C), int(max_iter), float(tolerance), _ptr(labels),
                             inertias.ctypes.data_as(ctypes.c_void_p), ctypes.byref(n_iter), ctypes.byref(conv),
                             cb, None, _ptr(ws), ws_bytes, _stream(torch, X.device)))
    del keep
    return dict(labels=labels, inertias=inertias[:n_iter.value].copy(), n_iter=n_iter.value,
                converged=bool(conv.value))


class Centers(object):
    """A resident center set (km_centers): centers copied to the device and,
    for the tensor-core path, prepared once for every later assignment."""

    def __init__(self, C, precision="auto"):
        torch = _torch()
        L = load()
        _check_frames(torch, C, "C")
        self._L = L
        self._h = ctypes.c_void_p()
        self.device = C.device
        check(L.km_centers_create(_ptr(C), C.shape[0], C.shape[1], precision_code(precision),
                                  _stream(torch, C.device), ctypes.byref(self._h)))
        k, d, p, nb = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int64()
        check(L.km_centers_info(self._h, ctypes.byref(k), ctypes.byref(d), ctypes.byref(p), ctypes.byref(nb)))
        self.k, self.d, self.precision, self.device_bytes = k.value, d.value, PRECISION_NAMES[p.value], nb.value

    @property
    def handle(self):
        if not self._h:
            raise ValueError("the center set was released")
        return self._h

    def assign(self, X, labels=None):
        """Labels (int32 CUDA tensor) of the nearest resident center for every row of X."""
        torch = _torch()
        _check_frames(torch, X)
        n, d = X.shape
        if labels is None:
            labels = torch.empty(n, dtype=torch.int32, device=X.device)
        ws_bytes = self._L.km_assign_centers_workspace_size(n, self.handle)
        ws = _workspace(torch, ws_bytes, X.device)
        stats = AssignStats()
        check(self._L.km_assign_centers(_ptr(X), n, d, self.handle, _ptr(labels), _ptr(ws), ws_bytes,
                                        ctypes.byref(stats), _stream(torch, X.device)))
        return labels, stats.as_dict()

    def close(self):
        if self._h:
            torch = _torch()
            torch.cuda.synchronize(self.device)
            check(self._L.km_centers_destroy(self._h))
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server(object):
    """The native serving loop (km_serve_*): trajectories submitted from host
    memory are batched per resident center set and assigned on the GPU."""

    def __init__(self, hbm_budget_bytes=40 << 30, max_batch_frames=0, device=0):
        L = load()
        self._L = L
        cfg = ServeConfig(int(hbm_budget_bytes), int(max_batch_frames), int(device), 0)
        self._h = ctypes.c_void_p()
        check(L.km_serve_create(ctypes.byref(cfg), ctypes.byref(self._h)))
        self._sets = []
        self._inflight = {}

    def add_centers(self, centers):
        """Registers a Centers object; returns its set id."""
        sid = ctypes.c_int32()
        check(self._L.km_serve_add_centers(self._h, centers.handle, ctypes.byref(sid)))
        self._sets.append(centers)
        return sid.value

    def submit(self, set_id, X_host, labels_host=None):
        """Queues X_host (C-contiguous float32 (n, d) numpy array or CPU tensor,
        page-locked for asynchronous copies); returns (ticket, labels array)."""
        if hasattr(X_host, "numpy"):
            X_np = X_host.numpy()
        else:
            X_np = X_host
        if X_np.dtype != np.float32 or X_np.ndim != 2 or not X_np.flags["C_CONTIGUOUS"]:
            raise ValueError("X_host must be a C-contiguous float32 (n, d) host array")
        n, d = X_np.shape
        if labels_host is None:
            labels_host = np.empty(n, dtype=np.int32)
        lab_np = labels_host.numpy() if hasattr(labels_host, "numpy") else labels_host
        if lab_np.dtype != np.int32 or lab_np.shape != (n,) or not lab_np.flags["C_CONTIGUOUS"]:
            raise ValueError("labels_host must be a contiguous int32 array of n entries")
        t = ctypes.c_uint64()
        check(self._L.km_serve_submit(self._h, int(set_id), X_np.ctypes.data_as(ctypes.c_void_p), n, d,
                                      lab_np.ctypes.data_as(ctypes.c_void_p), ctypes.byref(t)))
        self._inflight[t.value] = (X_host, labels_host)  # keep the buffers alive
        return t.value, labels_host

    def poll(self, ticket, timeout_ms=-1):
        """Request info dict once the request completed, None while pending."""
        info = RequestInfo()
        rc = self._L.km_serve_poll(self._h, ctypes.c_uint64(ticket), int(timeout_ms), ctypes.byref(info))
        if rc == KM_PENDING:
            return None
        self._inflight.pop(ticket, None)
        check(rc)
        return info.as_dict()

    def stats(self):
        st = ServeStats()
        check(self._L.km_serve_stats_read(self._h, ctypes.byref(st)))
        return st.as_dict()

    def shutdown(self):
        if self._h:
            check(self._L.km_serve_shutdown(self._h))
            self._h = ctypes.c_void_p()
            self._inflight.clear()

    def __del__(self):
        try:
            self.shutdown()
        except Exception:
            pass


def tune(X, C):
    """Times both precisions on X (a representative sample) against C and
    stores the faster for (d, k); 'auto' then uses it.  Returns
    dict(chosen, ms_fp32, ms_fp16)."""
    torch = _torch()
    L = load()
    _check_frames(torch, X)
    _check_frames(torch, C, "C")
    n, d = X.shape
    k = C.shape[0]
    ws_bytes = L.km_tune_workspace_size(n, d, k)
    ws = _workspace(torch, ws_bytes, X.device)
    chosen, t32, t16 = ctypes.c_int32(), ctypes.c_double(), ctypes.c_double()
    check(L.km_tune(_ptr(X), n, d, _ptr(C), k, _ptr(ws), ws_bytes, ctypes.byref(chosen), ctypes.byref(t32),
                    ctypes.byref(t16), _stream(torch, X.device)))
    return dict(chosen=PRECISION_NAMES[chosen.value], ms_fp32=t32.value,
                ms_fp16=t16.value if t16.value >= 0 else None)


def _pair_args(torch, xyz, pairs):
    if not (isinstance(xyz, torch.Tensor) and xyz.device.type == "cuda" and xyz.dtype == torch.float32
            and xyz.is_contiguous() and xyz.dim() == 3 and xyz.shape[2] == 3):
        raise ValueError("xyz must be a contiguous float32 CUDA tensor of shape (n, n_atoms, 3)")
    if not (isinstance(pairs, torch.Tensor) and pairs.device == xyz.device and pairs.dtype == torch.int32
            and pairs.is_contiguous() and pairs.dim() == 2 and pairs.shape[1] == 2):
        raise ValueError("pairs must be a contiguous int32 tensor of shape (d, 2) on the device of xyz")
    return int(xyz.shape[0]), int(xyz.shape[1]), int(pairs.shape[0])


def assign_pairs(xyz, pairs, C, precision="auto", labels=None):
    """Labels of the pair-distance features of coordinate frames, the
    features computed where the kernels read them (no feature matrix)."""
    torch = _torch()
    L = load()
    n, n_atoms, d = _pair_args(torch, xyz, pairs)
    _check_frames(torch, C, "C")
    if C.shape[1] != d:
        raise ValueError("centers have dimension %d, the pairs %d" % (C.shape[1], d))
    k = C.shape[0]
    p = precision_code(precision)
    if labels is None:
        labels = torch.empty(n, dtype=torch.int32, device=xyz.device)
    ws_bytes = L.km_assign_pairs_workspace_size(n, d, k, p)
    ws = _workspace(torch, ws_bytes, xyz.device)
    stats = AssignStats()
    check(L.km_assign_pairs(_ptr(xyz), n, n_atoms, _ptr(pairs), d, _ptr(C), k, p, _ptr(labels), _ptr(ws), ws_bytes,
                            ctypes.byref(stats), _stream(torch, xyz.device)))
    return labels, stats.as_dict()


def lloyd_pairs(xyz, pairs, C, max_iter, tolerance, precision="auto", callback=None, labels=None):
    """Lloyd iterations (in place on C) on the pair-distance features of
    coordinate frames; returns dict(labels, inertias, n_iter, converged)."""
    torch = _torch()
    L = load()
    n, n_atoms, d = _pair_args(torch, xyz, pairs)
    _check_frames(torch, C, "C")
    k = C.shape[0]
    p = precision_code(precision)
    if labels is None:
        labels = torch.empty(n, dtype=torch.int32, device=xyz.device)
    inertias = np.zeros(max(1, max_iter), dtype=np.float64)
    n_iter = ctypes.c_int32(0)
    conv = ctypes.c_int32(0)
    ws_bytes = L.km_lloyd_pairs_workspace_size(n, d, k, p)
    ws = _workspace(torch, ws_bytes, xyz.device)
    cb, keep = _callback(callback)
    check(L.km_lloyd_pairs(_ptr(xyz), n, n_atoms, _ptr(pairs), d, k, _ptr(C), int(max_iter), float(tolerance), p,
                           _ptr(labels), inertias.ctypes.data_as(ctypes.c_void_p), ctypes.byref(n_iter),
                           ctypes.byref(conv), cb, None, _ptr(ws), ws_bytes, _stream(torch, xyz.device)))
    del keep
    return dict(labels=labels, inertias=inertias[:n_iter.value].copy(), n_iter=n_iter.value,
                converged=bool(conv.value))


def kmpp_pairs(xyz, pairs, k, seed, callback=None):
    """kmeans++ initial centers (k, d) and chosen frame indices for the
    pair-distance features of coordinate frames."""
    torch = _torch()
    L = load()
    n, n_atoms, d = _pair_args(torch, xyz, pairs)
    C0 = torch.empty((k, d), dtype=torch.float32, device=xyz.device)
    idx = torch.empty(k, dtype=torch.int64, device=xyz.device)
    ws_bytes = L.km_kmpp_pairs_workspace_size(n, d, k)
    ws = _workspace(torch, ws_bytes, xyz.device)
    cb, keep = _callback(callback)
    check(L.km_kmpp_pairs(_ptr(xyz), n, n_atoms, _ptr(pairs), d, k, int(seed) & 0xFFFFFFFF, _ptr(C0), _ptr(idx), cb,
                          None, _ptr(ws), ws_bytes, _stream(torch, xyz.device)))
    del keep
    return C0, idx


def tune_clear():
    check(load().km_tune_clear())


def tune_tiles(X, C, precision="fp16"):
    """Times every tensor-core tile shape that fits (d, k) on X against C and
    stores the fastest for (d, k).  Returns dict(best, tried) of plan dicts
    (bn, pair, stages, list_len, ms)."""
    torch = _torch()
    L = load()
    _check_frames(torch, X)
    _check_frames(torch, C, "C")
    n, d = X.shape
    k = C.shape[0]
    ws_bytes = L.km_tune_workspace_size(n, d, k)
    ws = _workspace(torch, ws_bytes, X.device)
    best = TilePlan()
    tried = (TilePlan * 64)()
    n_tried = ctypes.c_int32(0)
    check(L.km_tune_tiles(_ptr(X), n, d, _ptr(C), k, precision_code(precision), _ptr(ws), ws_bytes,
                          ctypes.byref(best), tried, 64, ctypes.byref(n_tried), _stream(torch, X.device)))
    return dict(best=best.as_dict(), tried=[tried[i].as_dict() for i in range(n_tried.value)])


def tile_plan(d, k):
    """The tile shape tensor-core calls for (d, k) use now: dict(bn, pair,
    stages, list_len, tuned)."""
    plan = TilePlan()
    tuned = ctypes.c_int32(0)
    check(load().km_tile_plan_get(int(d), int(k), ctypes.byref(plan), ctypes.byref(tuned)))
    out = plan.as_dict()
    out.pop("ms")
    out["tuned"] = bool(tuned.value)
    return out


def force_tile_plan(plan):
    """Test hook: this thread's tensor-core calls use `plan` (a dict with bn,
    pair, stages, list_len) until force_tile_plan(None)."""
    L = load()
    if plan is None:
        check(L.km_debug_force_tile_plan(None))
        return
    tp = TilePlan(int(plan["bn"]), int(plan["pair"]), int(plan["stages"]), int(plan["list_len"]), 0.0)
    check(L.km_debug_force_tile_plan(ctypes.byref(tp)))


def regspace(X, dmin, max_centers):
    """Regular space centers of X in frame order: (centers (m, d) CUDA tensor, converged)."""
    torch = _torch()
    L = load()
    _check_frames(torch, X)
    n, d = X.shape
    C = torch.empty((max(1, int(max_centers)), d), dtype=torch.float32, device=X.device)
    ws_bytes = L.km_regspace_workspace_size(d)
    ws = _workspace(torch, ws_bytes, X.device)
    nc, conv = ctypes.c_int32(), ctypes.c_int32()
    check(L.km_regspace(_ptr(X), n, d, float(dmin), int(max_centers), _ptr(C), ctypes.byref(nc), ctypes.byref(conv),
                        _ptr(ws), ws_bytes, _stream(torch, X.device)))
    return C[:nc.value].clone(), bool(conv.value)


def count_matrix(dtrajs_packed, offsets, lag, nstates, sliding=True):
    """Dense (nstates, nstates) int64 CUDA tensor of lag-`lag` transition counts."""
    torch = _torch()
    L = load()
    if dtrajs_packed.device.type != "cuda" or dtrajs_packed.dtype != torch.int32 or not dtrajs_packed.is_contiguous():
        raise ValueError("dtrajs_packed must be a contiguous int32 CUDA tensor")
    offs = np.ascontiguousarray(offsets, dtype=np.int64)
    n_traj = len(offs) - 1
    counts = torch.empty((int(nstates), int(nstates)), dtype=torch.int64, device=dtrajs_packed.device)
    ws_bytes = L.km_count_matrix_workspace_size(n_traj)
    ws = _workspace(torch, ws_bytes, dtrajs_packed.device)
    check(L.km_count_matrix(_ptr(dtrajs_packed), offs.ctypes.data_as(ctypes.c_void_p), n_traj, int(lag),
                            1 if sliding else 0, int(nstates), _ptr(counts), _ptr(ws), ws_bytes,
                            _stream(torch, dtrajs_packed.device)))
    return counts


def pair_distances(xyz, pairs, out=None):
    """(n, npairs) float32 CUDA tensor of atom-pair distances of xyz (n, n_atoms, 3) CUDA float32."""
    torch = _torch()
    L = load()
    if xyz.device.type != "cuda" or xyz.dtype != torch.float32 or xyz.dim() != 3 or xyz.shape[2] != 3 \
            or not xyz.is_contiguous():
        raise ValueError("xyz must be a contiguous float32 (n, n_atoms, 3) CUDA tensor")
    n, n_atoms, _ = xyz.shape
    if pairs.device.type != "cuda" or pairs.dtype != torch.int32 or pairs.dim() != 2 or pairs.shape[1] != 2 \
            or not pairs.is_contiguous():
        raise ValueError("pairs must be a contiguous int32 (npairs, 2) CUDA tensor")
    if pairs.numel() and (int(pairs.min()) < 0 or int(pairs.max()) >= n_atoms):
        raise ValueError("pair indices out of range [0, %d)" % n_atoms)
    npairs = pairs.shape[0]
    if out is None:
        out = torch.empty((n, npairs), dtype=torch.float32, device=xyz.device)
    check(L.km_pair_distances(_ptr(xyz), n, n_atoms, _ptr(pairs), npairs, _ptr(out), _stream(torch, xyz.device)))
    return out
