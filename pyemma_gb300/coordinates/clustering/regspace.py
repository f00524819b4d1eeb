"""Regular space clustering on the GPU.

Mirrors RegularSpaceClustering of pyemma/coordinates/clustering/
regspace.py:36-185.  The first pass (the leader walk over the frames in
iteration order, deeptime RegularSpace.partial_fit at regspace.py:140-152)
runs as km_regspace; the second pass (Voronoi assignment) is the same
assignment path as every other estimator here.
"""
import warnings

import numpy as np

from ... import _lib
from .. import _device
from .interface import AbstractClustering

__all__ = ["RegularSpaceClustering", "NotConvergedWarning"]


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
        'euclidean'.
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
        if self.metric == "minRMSD":
            raise NotImplementedError("regular space clustering has no minRMSD center search; "
                                      "the minRMSD metric is available for k-means and assignment")
        stride = self.stride if self.stride else 1
        trajs = source.frames(stride=stride, skip=self.skip)
        dim = source.dimension()
        used = int(sum(len(t) for t in trajs))
        X = _device.pack_to_device(trajs, dim)
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
