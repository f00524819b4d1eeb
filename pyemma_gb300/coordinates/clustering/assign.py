"""Assignment to given centers (pyemma/coordinates/clustering/assign.py:33-108)."""
import numpy as np

from .interface import AbstractClustering

__all__ = ["AssignCenters"]


def _load_centers(path):
    if path.endswith(".npy"):
        return np.load(path)
    return np.loadtxt(path, ndmin=2)


class AssignCenters(AbstractClustering):
    r"""Assigns data to given (pre-calculated) cluster centers.

    Parameters
    ----------
    clustercenters : path to file (text or .npy) or ndarray (k, d)
    metric : str
        'euclidean'.
    stride : int
    n_jobs : int or None
        Accepted for compatibility.
    skip : int
        Skip the first n frames of each trajectory.
    precision : {'auto', 'fp32', 'fp16', 'bf16'}
    """

    def __init__(self, clustercenters, metric="euclidean", stride=1, n_jobs=None, skip=0, precision="auto"):
        super(AssignCenters, self).__init__(metric=metric, n_jobs=n_jobs, precision=precision)
        if isinstance(clustercenters, str):
            clustercenters = _load_centers(clustercenters)
        clustercenters = np.array(clustercenters, dtype=np.float32, order="C")
        if not clustercenters.ndim == 2:
            raise ValueError("cluster centers have to be 2d")
        self.clustercenters = clustercenters
        self.stride = stride
        self.skip = skip
        self._estimated = True

    def _param_names(self):
        return ("clustercenters", "metric", "stride", "n_jobs", "skip", "precision")

    def describe(self):
        return "[{name} centers shape={shape}]".format(name=type(self).__name__, shape=self.clustercenters.shape)

    @AbstractClustering.data_producer.setter
    def data_producer(self, dp):
        if dp is not None:
            dim = self.clustercenters.shape[1]
            if not dim == dp.dimension():
                raise ValueError("cluster centers have wrong dimension. Have dim=%i, but input has %i"
                                 % (dim, dp.dimension()))
        AbstractClustering.data_producer.fset(self, dp)

    def _estimate(self, source):
        self.assign(None, self.stride)
        return self
