"""Host <-> device movement of trajectories for the clustering kernels.

Frames of many trajectories are packed back to back into one pinned host
buffer (the float32 cast of interface.py:159 happens in that copy), moved to
the GPU with one asynchronous copy, assigned by one batched launch
(km_batch_assign) and copied back.  Inputs larger than the per-batch budget
are processed in several batches; a trajectory may be split across batches.
"""
import numpy as np

from .. import _lib

# Frames moved to the device per batch (bytes of float32 frames).
BATCH_BYTES = 8 << 30


def torch_module():
    import torch
    if not torch.cuda.is_available():
        raise RuntimeError("pyemma_gb300 needs a CUDA device; none is available")
    return torch


def device():
    torch = torch_module()
    return torch.device("cuda", torch.cuda.current_device())


def pack_to_device(trajs, dim):
    """Copies a list of (T_i, dim) arrays into one (sum T_i, dim) float32 CUDA tensor.

    Each trajectory goes to its slice of the device buffer with one copy
    (float32 cast first where needed, like np.require(X, float32) in
    interface.py:159); host arrays that live in pinned memory are read by DMA
    directly.
    """
    torch = torch_module()
    if len(trajs) > 0 and all(isinstance(t, torch.Tensor) and t.device.type == "cuda" for t in trajs):
        # frames already on the device: used as they are when they form one
        # contiguous float32 block, else gathered on the device
        ts = [t for t in trajs if len(t)]
        if len(ts) == 1 and ts[0].dtype == torch.float32 and ts[0].is_contiguous():
            return ts[0]
        if not ts:
            return torch.empty((0, dim), dtype=torch.float32, device=device())
        return torch.cat([t.float() for t in ts]).contiguous()
    n = int(sum(len(t) for t in trajs))
    dev = torch.empty((n, dim), dtype=torch.float32, device=device())
    pos = 0
    for t in trajs:
        if len(t) == 0:
            continue
        a = np.require(t, dtype=np.float32, requirements="C")
        dev[pos:pos + len(a)].copy_(torch.from_numpy(a))
        pos += len(a)
    torch.cuda.current_stream().synchronize()
    return dev


def host_parts(trajs):
    """The trajectories as float32 C-contiguous host arrays (cast where
    needed, as np.require in interface.py:159), or None when any of them is
    already on the device."""
    torch = torch_module()
    out = []
    for t in trajs:
        if isinstance(t, torch.Tensor):
            if t.device.type != "cpu":
                return None
            t = t.numpy()
        out.append(np.require(t, dtype=np.float32, requirements="C"))
    return out


def centers_to_device(centers):
    torch = torch_module()
    c = np.ascontiguousarray(centers, dtype=np.float32)
    return torch.from_numpy(c).to(device())


def check_minrmsd_dim(dim):
    if dim % 3 != 0:
        # clustering_module.cpp:13-15 raises the same condition
        raise ValueError("RMSDMetric is only implemented for input data with a dimension divisible by 3.")


def plan_batches(lengths, budget):
    """Batches of (traj, start, stop) pieces covering trajectories of the
    given lengths in order, at most ``budget`` frames per batch; every batch
    but the last is full, so a trajectory may be split across batches."""
    if budget < 1:
        raise ValueError("a batch must hold at least one frame")
    pieces, batch, size = [], [], 0
    for i, length in enumerate(lengths):
        start = 0
        while start < length:
            take = min(length - start, budget - size)
            batch.append((i, start, start + take))
            size += take
            start += take
            if size == budget:
                pieces.append(batch)
                batch, size = [], 0
    if batch:
        pieces.append(batch)
    return pieces


def assign_trajs(trajs, centers, precision="auto", batch_bytes=None, metric="euclidean"):
    """int32 labels for every frame of every trajectory; returns (list, stats)."""
    torch = torch_module()
    centers = np.ascontiguousarray(centers, dtype=np.float32)
    if centers.ndim != 2:
        raise ValueError("cluster centers have to be 2d")
    dim = centers.shape[1]
    for t in trajs:
        if t.ndim != 2 or t.shape[1] != dim:
            raise ValueError("cluster centers have wrong dimension. Have dim=%i, but input has %i"
                             % (dim, t.shape[1] if t.ndim == 2 else 1))
    if metric == "minRMSD":
        check_minrmsd_dim(dim)
    C = centers_to_device(centers)
    budget = max(1, int((batch_bytes or BATCH_BYTES) // (4 * dim)))
    outs = [np.empty(len(t), dtype=np.int32) for t in trajs]
    stats = dict(n_frames=0, n_recheck=0, n_full=0, n_flipped=0, precision=None)
    for batch in plan_batches([len(t) for t in trajs], budget):
        arrays = [trajs[i][a:b] for i, a, b in batch]
        X = pack_to_device(arrays, dim)
        offsets = np.zeros(len(arrays) + 1, dtype=np.int64)
        offsets[1:] = np.cumsum([len(a) for a in arrays])
        if metric == "minRMSD":
            labels = _lib.assign_minrmsd(X, C)
            st = dict(n_frames=int(X.shape[0]), n_recheck=0, n_full=0, n_flipped=0, precision="fp32")
        else:
            labels, st = _lib.batch_assign(X, offsets, C, precision=precision)
        host = labels.cpu().numpy()
        for (i, a, b), o0, o1 in zip(batch, offsets[:-1], offsets[1:]):
            outs[i][a:b] = host[o0:o1]
        for key in ("n_frames", "n_recheck", "n_full", "n_flipped"):
            stats[key] += st[key]
        stats["precision"] = st["precision"]
        del X, labels
    return outs, stats
