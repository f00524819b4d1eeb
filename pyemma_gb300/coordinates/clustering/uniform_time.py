"""Uniform time clustering.

Mirrors UniformTimeClustering of pyemma/coordinates/clustering/
uniform_time.py:31-110: k frames evenly spread over the concatenated
(strided, skipped) time axis become the centers; the assignment is the same
GPU path as every other estimator here.
"""
import math

import numpy as np

from .interface import AbstractClustering

__all__ = ["UniformTimeClustering"]


class UniformTimeClustering(AbstractClustering):
    r"""Uniform time clustering (uniform_time.py:31).

    Parameters
    ----------
    n_clusters : int or None
        Number of centers; None gives min(sqrt(N), 5000).
    metric : str
        'euclidean'.
    stride, skip : int
    n_jobs : int or None
        Accepted for compatibility.
    precision : {'auto', 'fp32', 'fp16', 'bf16'}
    """

    def __init__(self, n_clusters=2, metric="euclidean", stride=1, n_jobs=None, skip=0, precision="auto"):
        super(UniformTimeClustering, self).__init__(metric=metric, n_jobs=n_jobs, precision=precision)
        self.set_params(n_clusters=n_clusters, metric=metric, stride=stride, skip=skip)

    def _param_names(self):
        return ("n_clusters", "metric", "stride", "skip", "n_jobs", "precision")

    def describe(self):
        return "[Uniform time clustering, k = %i, inp_dim=%i]" % (self.n_clusters, self.data_producer.dimension())

    @staticmethod
    def _idx_to_traj_idx(idx, cumsum):
        prev_len = 0
        for traj_idx, length in enumerate(cumsum):
            if prev_len <= idx < length:
                return traj_idx, idx - prev_len
            prev_len = length
        raise ValueError("Requested index %s was out of bounds [0,%s)" % (idx, cumsum[-1]))

    def _estimate(self, source):
        stride = self.stride if self.stride else 1
        if self.n_clusters is None:
            total_length = int(sum(source.trajectory_lengths(stride=stride, skip=self.skip)))
            self.n_clusters = min(int(math.sqrt(total_length)), 5000)
            self.logger.info("The number of cluster centers was not specified, "
                             "using min(sqrt(N), 5000)=%s as n_clusters." % self.n_clusters)
        T = source.n_frames_total(stride=stride, skip=self.skip)
        if self.n_clusters > T:
            self.n_clusters = T
            self.logger.info("Requested more clusters (k = %i than there are total data points %i). "
                             "Will do clustering with k = %i" % (self.n_clusters, T, T))
        # uniform_time.py:92-100: the first frame in the middle of the first
        # segment, positions in units of the stride on the unstrided axis.
        next_t = (T // self.n_clusters) // 2
        cumsum = np.cumsum(source.trajectory_lengths(skip=self.skip))
        linspace = stride * np.arange(next_t, T - next_t + 1, (T - 2 * next_t + 1) // self.n_clusters)[:self.n_clusters]
        picks = [self._idx_to_traj_idx(x, cumsum) for x in linspace]
        frames = source.frames(stride=1, skip=self.skip)
        rows = [frames[i][t] for i, t in picks]
        self.clustercenters = np.asarray([r if isinstance(r, np.ndarray) else r.cpu().numpy() for r in rows],
                                         dtype=np.float32)
        assert len(self.clustercenters) == self.n_clusters
        return self
