"""Regular space clustering on the GPU.

Mirrors RegularSpaceClustering of pyemma/coordinates/clustering/
regspace.py:36-185.  The first pass (the leader walk over the frames in
iteration order, deeptime RegularSpace.partial_fit at regspace.py:140-152)
runs as km_regspace for the Euclidean metric and as
:func:`minrmsd_leader_walk` over km_assign_minrmsd for minRMSD (the metric
regspace.py:89 registers); the second pass (Voronoi assignment) is the same
assignment path as every other estimator here.
"""
import warnings

import numpy as np

from ... import _lib
from .. import _device
from .interface import AbstractClustering

__all__ = ["RegularSpaceClustering", "NotConvergedWarning"]


MINRMSD_WALK_BLOCK = 8192


def minrmsd_leader_walk(X, dmin, max_centers, block=MINRMSD_WALK_BLOCK):
    """The regular space walk under the minRMSD metric.

    X is a contiguous float32 (n, 3 n_atoms) CUDA tensor.  Returns the frame
    indices of the centers in frame order and whether the walk finished
    (False when a (max_centers + 1)-th center would be added).

    The walk is the sequential one (a frame becomes a center when its float32
    rmsd to every center before it, compared in double, is at least dmin),
    batched: for a block of frames one km_assign_minrmsd call gives every
    frame's smallest rmsd to the centers found before the block, which
    settles the frames below dmin.  The others are resolved in frame order:
    the first is a center (no center of the block precedes it), the later
    ones stay candidates only if at least dmin from it (one more call), and
    so on.  A frame's rmsd to a center is the same value in both forms, so
    the result equals the sequential walk's.
    """
    import torch
    n = int(X.shape[0])
    idx = []
    C = None
    for pos in range(0, n, block):
        blk = X[pos:pos + block]
        if C is None:
            cand = np.arange(int(blk.shape[0]))
        else:
            _, r = _lib.assign_minrmsd(blk, C, return_rmsd=True)
            cand = np.nonzero(r.cpu().numpy().astype(np.float64) >= dmin)[0]
        while len(cand):
            if len(idx) == max_centers:
                return idx, False
            first = int(cand[0])
            idx.append(pos + first)
            c1 = blk[first:first + 1].contiguous()
            C = c1 if C is None else torch.cat([C, c1]).contiguous()
            rest = cand[1:]
            if not len(rest):
                break
            rows = blk[torch.from_numpy(rest).to(blk.device)].contiguous()
            _, r = _lib.assign_minrmsd(rows, c1, return_rmsd=True)
            cand = rest[r.cpu().numpy().astype(np.float64) >= dmin]
    return idx, True


class NotConvergedWarning(RuntimeWarning):
    """The estimation stopped early (pyemma/util/exceptions.py:44)."""


class RegularSpaceClustering(AbstractClustering):
    r"""Regular space clustering (regspace.py:36).

    Parameters
    ----------
    dmin : float
        Minimum distance between cluster centers.
    max_centers : int
        When this many centers are found and another frame qualifies, the
        walk stops with a warning and the centers found so far are kept.
    metric : str
        'euclidean' or 'minRMSD'.
    stride, skip : int
        Frames used for the center search: traj[skip::stride].
    n_jobs : int or None
        Accepted for compatibility.
    precision : {'auto', 'fp32', 'fp16', 'bf16'}
        Arithmetic of the assignment pass (labels are exact in all cases).
    """

    def __init__(self, dmin, max_centers=1000, metric="euclidean", stride=1, n_jobs=None, skip=0,
                 precision="auto"):
        super(RegularSpaceClustering, self).__init__(metric=metric, n_jobs=n_jobs, precision=precision)
        self._converged = False
        self.set_params(dmin=dmin, metric=metric, max_centers=max_centers, stride=stride, skip=skip)

    def _param_names(self):
        return ("dmin", "max_centers", "metric", "stride", "skip", "n_jobs", "precision")

    def describe(self):
        return "[RegularSpaceClustering dmin=%f, inp_dim=%i]" % (self._dmin, self.data_producer.dimension())

    @property
    def dmin(self):
        """Minimum distance between cluster centers."""
        return self._dmin

    @dmin.setter
    def dmin(self, d):
        d = float(d)
        if d < 0:
            raise ValueError("d has to be positive")
        self._dmin = d

    @property
    def max_centers(self):
        """Cutoff of the center search (regspace.py:112-122)."""
        return self._max_centers

    @max_centers.setter
    def max_centers(self, value):
        value = int(value)
        if value < 0:
            raise ValueError("max_centers has to be positive")
        self._max_centers = value

    @property
    def n_clusters(self):
        return self.max_centers

    @n_clusters.setter
    def n_clusters(self, val):
        self.max_centers = val

    @property
    def converged(self):
        return self._converged

    def _estimate(self, source):
        stride = self.stride if self.stride else 1
        trajs = source.frames(stride=stride, skip=self.skip)
        dim = source.dimension()
        if self.metric == "minRMSD":
            _device.check_minrmsd_dim(dim)
        used = int(sum(len(t) for t in trajs))
        X = _device.pack_to_device(trajs, dim)
        if self.metric == "minRMSD":
            import torch
            idx, converged = minrmsd_leader_walk(X, self.dmin, max(1, self.max_centers))
            C = X[torch.tensor(idx, dtype=torch.int64, device=X.device)]
        else:
            C, converged = _lib.regspace(X, self.dmin, max(1, self.max_centers))
        del X
        self.clustercenters = C.cpu().numpy()
        self._converged = converged
        if not converged:
            msg = ("Maximum number of cluster centers reached. Consider increasing max_centers or choose"
                   " a larger minimum distance, dmin.")
            self.logger.warning(msg)
            warnings.warn(msg)
            # regspace.py:162-163 raises NotConvergedWarning, which the
            # streaming estimator turns into an info message
            # (streaming_estimator.py:43-47).
            self.logger.info("Presumably finished estimation. Message: Used data for centers: %.2f%%"
                             % (100.0 * used / max(1, used)))
        if len(self.clustercenters) == 1:
            self.logger.warning("Have found only one center according to minimum distance requirement of %f"
                                % self.dmin)
        return self
