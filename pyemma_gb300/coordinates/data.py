"""In-memory trajectory source and the small conventions around it.

Mirrors the parts of PyEMMA's streaming layer that decide which frames the
clustering kernels see:

* input normalisation: pyemma/util/types.py:473 (ensure_traj_list) and
  pyemma/coordinates/data/data_in_memory.py:96-108 (1-D -> (T, 1), >2-D
  flattened to (T, prod(rest)));
* strided/skipped lengths: pyemma/coordinates/data/_base/datasource.py:268
  (max((T - skip - 1) // stride + 1, 0));
* default chunk size: pyemma/coordinates/data/_base/iterable.py:43-62 with
  config.default_chunksize = 256m (pyemma/pyemma.cfg:40);
* n_jobs resolution: pyemma/_base/parallel.py:2-38.
"""
import functools
import logging
import numbers
import os
import warnings

import numpy as np

DEFAULT_CHUNKSIZE_BYTES = 256 * 1024 * 1024


def _as_2d(a):
    a = np.asarray(a)
    if a.ndim == 1:
        return np.atleast_2d(a).T
    if a.ndim == 2:
        return a
    return np.reshape(a, (a.shape[0], functools.reduce(lambda x, y: x * y, a.shape[1:])))


def ensure_traj_list(data):
    if isinstance(data, (list, tuple)):
        if len(data) > 0 and all(isinstance(x, numbers.Real) and not isinstance(x, np.ndarray) for x in data):
            return [np.asarray(data)[:, None]]
        out = []
        for t in data:
            if not isinstance(t, np.ndarray):
                raise ValueError("Please supply numpy.ndarray, or list/tuple of ndarray. Your input was %s"
                                 % type(t))
            out.append(_as_2d(t))
        return out
    if not isinstance(data, np.ndarray):
        raise ValueError("Please supply numpy.ndarray, or list/tuple of ndarray. Your input was %s"
                         % type(data))
    return [_as_2d(data)]


def default_chunksize(dim, itemsize):
    return max(1, int(np.floor(DEFAULT_CHUNKSIZE_BYTES / (itemsize * dim))))


class InMemorySource(object):
    """Trajectories held as NumPy arrays (the reference's DataInMemory)."""

    def __init__(self, data, chunksize=None):
        self._data = ensure_traj_list(data)
        if len(self._data) == 0:
            raise ValueError("no trajectories given")
        dims = {t.shape[1] for t in self._data}
        if len(dims) != 1:
            raise ValueError("trajectories have different dimensions: %s" % sorted(dims))
        self._dim = dims.pop()
        self.chunksize = chunksize

    @property
    def data(self):
        return self._data

    @property
    def ntraj(self):
        return len(self._data)

    @property
    def ndim(self):
        return self._dim

    def dimension(self):
        return self._dim

    def number_of_trajectories(self, stride=None):
        return len(self._data)

    def trajectory_length(self, itraj, stride=1, skip=0):
        if itraj >= self.ntraj:
            raise IndexError("given index (%s) exceeds number of data sets (%s). Zero based indexing!"
                             % (itraj, self.ntraj))
        return max((len(self._data[itraj]) - skip - 1) // int(stride) + 1, 0)

    def trajectory_lengths(self, stride=1, skip=0):
        return np.fromiter((self.trajectory_length(i, stride, skip) for i in range(self.ntraj)),
                           dtype=int, count=self.ntraj)

    def n_frames_total(self, stride=1, skip=0):
        return int(sum(self.trajectory_lengths(stride=stride, skip=skip)))

    def frames(self, stride=1, skip=0):
        """Per trajectory, the frames the iterator would yield (views)."""
        return [t[skip::stride] for t in self._data]

    @property
    def default_chunksize(self):
        itemsize = max(t.dtype.itemsize for t in self._data)
        return default_chunksize(self._dim, itemsize)


def is_device_data(data):
    """True for a CUDA torch tensor or a list/tuple of them (frames already on the GPU)."""
    try:
        import torch
    except ImportError:
        return False
    if isinstance(data, torch.Tensor):
        return data.device.type == "cuda"
    if isinstance(data, (list, tuple)) and len(data) > 0:
        return all(isinstance(t, torch.Tensor) and t.device.type == "cuda" for t in data)
    return False


class DeviceSource(InMemorySource):
    """Trajectories that already live in device memory (CUDA torch tensors),
    e.g. features computed on the GPU; they are used without a host copy."""

    def __init__(self, data, chunksize=None):
        import torch
        if isinstance(data, torch.Tensor):
            data = [data]
        out = []
        for t in data:
            if t.dim() == 1:
                t = t[:, None]
            elif t.dim() > 2:
                t = t.reshape(t.shape[0], -1)
            out.append(t)
        if len(out) == 0:
            raise ValueError("no trajectories given")
        dims = {int(t.shape[1]) for t in out}
        if len(dims) != 1:
            raise ValueError("trajectories have different dimensions: %s" % sorted(dims))
        self._data = out
        self._dim = dims.pop()
        self.chunksize = chunksize

    @property
    def default_chunksize(self):
        return default_chunksize(self._dim, 4)


def get_n_jobs(logger=None):
    """n_jobs from SLURM_CPUS_ON_NODE, PYEMMA_NJOBS or the logical CPU count."""

    def _from_hardware():
        try:
            import psutil
            count = psutil.cpu_count(logical=True)
        except ImportError:
            count = os.cpu_count()
        return count if count is not None else 1

    def _from_env(var):
        e = os.getenv(var, None)
        if e:
            try:
                return int(e)
            except ValueError as ve:
                if logger is not None:
                    logger.warning("could not parse env variable '%s'. Value='%s'. Error=%s." % (var, e, ve))
        return None

    slurm = _from_env("SLURM_CPUS_ON_NODE")
    pyemma = _from_env("PYEMMA_NJOBS")
    if slurm and pyemma:
        warnings.warn("two settings for n_jobs from environment: PYEMMA_NJOBS and SLURM_CPUS_ON_NODE. "
                      "Respecting the SLURM setting to avoid overprovisioning resources.")
    val = slurm or pyemma
    if not val:
        val = _from_hardware()
    return val


def make_logger(obj):
    return logging.getLogger("pyemma_gb300.%s" % type(obj).__name__)
