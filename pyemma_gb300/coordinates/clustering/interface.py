"""Shared clustering base: centers, dtrajs, assign/transform/get_output.

Mirrors pyemma/coordinates/clustering/interface.py (AbstractClustering,
:44-302).  The native call of the reference, ClusterModel(centers,
metric).transform(X) at interface.py:164-165, becomes a batched launch of the
GPU assignment kernel through libkmgpu (pyemma_gb300/_lib.py).
"""
import os

import numpy as np

from ... import _lib
from .. import _device
from ..data import DeviceSource, InMemorySource, default_chunksize, get_n_jobs, is_device_data, make_logger

_METRICS = ("euclidean", "minRMSD")


class AbstractClustering(object):
    """Common interface of the clustering estimators (interface.py:44).

    Parameters
    ----------
    metric : str, default='euclidean'
        Distance of the assignment: 'euclidean', or 'minRMSD' (atom-major
        coordinates, d = 3 n_atoms: the RMSD after optimal superposition,
        clustering_module.cpp:9-36).
    n_jobs : int or None
        Accepted for compatibility (thread count of the reference's OpenMP
        backend); resolved as the reference does and otherwise unused.
    precision : {'auto', 'fp32', 'fp16', 'bf16'}
        Arithmetic of the distance kernel.  Every choice gives the labels of
        the exact float32 evaluation; 'fp16' uses the tensor cores with an
        exact recheck of near ties.
    """

    def __init__(self, metric="euclidean", n_jobs=None, precision="auto"):
        self.logger = make_logger(self)
        self.metric = metric
        self.clustercenters = None
        self._previous_stride = -1
        self._dtrajs = []
        self._overwrite_dtrajs = False
        self._index_states = []
        self.n_jobs = n_jobs
        self.precision = precision
        self.chunksize = None
        self._data_producer = None
        self._estimated = False
        self.last_assign_stats = None

    # ---- parameters ------------------------------------------------------
    @property
    def metric(self):
        return self._metric

    @metric.setter
    def metric(self, value):
        if value not in _METRICS:
            raise ValueError("metric must be one of %s, was %r" % (_METRICS, value))
        self._metric = value

    @property
    def clustercenters(self):
        """Array containing the coordinates of the calculated cluster centers."""
        return self._clustercenters

    @clustercenters.setter
    def clustercenters(self, val):
        self._clustercenters = np.asarray(val, dtype="float32", order="C")[:] if val is not None else None
        self._precentered = False

    @property
    def cluster_centers_(self):
        return self.clustercenters

    @property
    def n_jobs(self):
        if not hasattr(self, "_n_jobs"):
            self._n_jobs = get_n_jobs(logger=self.logger)
        return self._n_jobs

    @n_jobs.setter
    def n_jobs(self, val):
        if val is not None and val == 0:
            raise ValueError("n_jobs must not be 0.")
        elif val is not None and val < 0:
            import warnings
            warnings.warn("Negative n_jobs will likely raise in future versions, use None instead.",
                          DeprecationWarning)
            val = None
        if val is None:
            val = get_n_jobs(logger=self.logger)
        self._n_jobs = int(val)

    @property
    def overwrite_dtrajs(self):
        return self._overwrite_dtrajs

    @overwrite_dtrajs.setter
    def overwrite_dtrajs(self, value):
        self._overwrite_dtrajs = value

    def set_params(self, **params):
        valid = set(self._param_names())
        for key, value in params.items():
            if key not in valid:
                raise ValueError("Invalid parameter %s for estimator %s" % (key, type(self).__name__))
            setattr(self, key, value)
        return self

    def get_params(self):
        return {k: getattr(self, k) for k in self._param_names()}

    def _param_names(self):
        return ("metric", "n_jobs", "precision")

    # ---- persistence (serialization.py:212-290) ----------------------------
    def save(self, file_name, model_name="default", overwrite=False, save_streaming_chain=False):
        """Stores the parameters and the model (centers, dtrajs, convergence)
        in file_name under model_name; see pyemma_gb300.serialization."""
        from ... import serialization
        serialization.save(self, file_name, model_name=model_name, overwrite=overwrite,
                           save_streaming_chain=save_streaming_chain)

    @classmethod
    def load(cls, file_name, model_name="default"):
        """The estimator stored in file_name under model_name."""
        from ... import serialization
        obj = serialization.load(file_name, model_name=model_name)
        if not isinstance(obj, cls):
            raise TypeError("model %r in %s is a %s, not a %s" % (model_name, file_name, type(obj).__name__,
                                                                  cls.__name__))
        return obj

    # ---- data producer ---------------------------------------------------
    @property
    def data_producer(self):
        return self._data_producer

    @data_producer.setter
    def data_producer(self, dp):
        self._data_producer = dp

    @property
    def in_memory(self):
        return False

    def _source(self, X, chunksize=None):
        from ...featurize import PairDistanceFrames
        if isinstance(X, (InMemorySource, PairDistanceFrames)):
            return X
        if is_device_data(X):
            return DeviceSource(X, chunksize=chunksize)
        return InMemorySource(X, chunksize=chunksize)

    # ---- estimation ------------------------------------------------------
    def estimate(self, X, chunksize=None, **params):
        """Estimates the model from X (ndarray or list of ndarrays); returns self."""
        if params:
            self.set_params(**params)
        source = self._source(X, chunksize=chunksize)
        self.data_producer = source
        self.chunksize = chunksize
        self._dtrajs = []
        self._index_states = []
        self._previous_stride = -1
        self._estimate(source)
        self._estimated = True
        return self

    def fit(self, X, y=None, **kw):
        return self.estimate(X, **kw)

    def _estimate(self, source):
        raise NotImplementedError

    # ---- outputs ---------------------------------------------------------
    def dimension(self):
        """output dimension of clustering algorithm (always 1)."""
        return 1

    def output_type(self):
        return np.int32()

    @property
    def n_clusters(self):
        if getattr(self, "_n_clusters", None) is not None:
            return self._n_clusters
        return None if self.clustercenters is None else len(self.clustercenters)

    @n_clusters.setter
    def n_clusters(self, value):
        self._n_clusters = value

    @property
    def default_chunksize(self):
        dim = self.data_producer.dimension() if self.data_producer is not None else 1
        return default_chunksize(dim, 4)

    def _chunk(self):
        return self.chunksize if self.chunksize is not None else self.default_chunksize

    def _assign_arrays(self, arrays):
        if self.clustercenters is None or len(self.clustercenters) == 0:
            raise ValueError("no cluster centers to assign to")
        labels, stats = _device.assign_trajs(arrays, self.clustercenters, precision=self.precision,
                                             metric=self.metric)
        self.last_assign_stats = stats
        return labels

    def _assign_pairs(self, src):
        """int32 labels of PairDistanceFrames (km_assign_pairs)."""
        if self.clustercenters is None or len(self.clustercenters) == 0:
            raise ValueError("no cluster centers to assign to")
        if self.metric != "euclidean":
            raise ValueError("pair-distance frames are assigned under the euclidean metric")
        C = _device.centers_to_device(self.clustercenters)
        lab, stats = _lib.assign_pairs(src.xyz, src.pairs, C, precision=self.precision)
        self.last_assign_stats = stats
        return lab.cpu().numpy()

    def _transform_array(self, X):
        """get closest index of point in clustercenters to x (column vector)."""
        if not is_device_data(X):
            X = np.asarray(X)
        if X.ndim == 1:
            X = X[:, None]
        return self._assign_arrays([X])[0][:, None]

    def transform(self, X):
        """Maps X (ndarray, CUDA tensor or a list of them) to (T, 1) int32 column vector(s)."""
        from ...featurize import PairDistanceFrames
        if isinstance(X, PairDistanceFrames):
            return self._assign_pairs(X)[:, None]
        source = DeviceSource(X) if is_device_data(X) else InMemorySource(X)
        if isinstance(X, (list, tuple)):
            return [lab[:, None] for lab in self._assign_arrays(source.data)]
        return self._transform_array(source.data[0])

    def get_output(self, dimensions=slice(0, None), stride=1, skip=0, chunk=None):
        """Assigns all frames of the data producer; list of (T_i, 1) int32 arrays."""
        if self.data_producer is None:
            raise RuntimeError("no data producer: call estimate() first")
        from ...featurize import PairDistanceFrames
        if isinstance(self.data_producer, PairDistanceFrames):
            return [self._assign_pairs(self.data_producer.strided(stride, skip))[:, None][:, dimensions]]
        trajs = self.data_producer.frames(stride=stride, skip=skip)
        labels = self._assign_arrays(trajs)
        return [lab[:, None][:, dimensions] for lab in labels]

    def assign(self, X=None, stride=1):
        """Discrete trajectories of the data producer (X=None) or of X."""
        if X is None:
            if self._previous_stride is stride and len(self._dtrajs) > 0:
                return self._dtrajs
            self._previous_stride = stride
            skip = self.skip if hasattr(self, "skip") else 0
            mapped = self.get_output(stride=stride, chunk=self.chunksize, skip=skip)
            self._dtrajs = [np.transpose(m)[0] for m in mapped]
            return self._dtrajs
        if stride != 1:
            raise ValueError("assign accepts either X or stride parameters, but not both. If you want to map "
                             "only a subset of your data, extract the subset yourself and pass it as X.")
        mapped = self.transform(X)
        if isinstance(mapped, np.ndarray):
            return np.transpose(mapped)[0]
        return [np.transpose(m)[0] for m in mapped]

    @property
    def dtrajs(self):
        """Discrete trajectories (assigned data to cluster centers)."""
        if len(self._dtrajs) == 0:
            self._dtrajs = self.assign(stride=1)
        return self._dtrajs

    @property
    def index_clusters(self):
        """Per cluster, the (trajectory, time) indexes of its frames."""
        if len(self._dtrajs) == 0:
            self._dtrajs = self.assign()
        if len(self._index_states) == 0:
            self._index_states = _index_states(self._dtrajs)
        return self._index_states

    def sample_indexes_by_cluster(self, clusters, nsample, replace=True):
        if len(self._index_states) == 0:
            self._index_states = _index_states(self.dtrajs)
        out = []
        for c in clusters:
            idx = self._index_states[c]
            if len(idx) == 0:
                out.append(np.zeros((0, 2), dtype=int))
                continue
            if not replace and nsample > len(idx):
                pick = np.random.choice(len(idx), len(idx), replace=False)
            else:
                pick = np.random.choice(len(idx), nsample, replace=replace)
            out.append(idx[pick])
        return out

    # ---- iteration / lengths ----------------------------------------------
    def __iter__(self):
        chunk = self._chunk()
        for itraj, dtraj in enumerate(self.dtrajs):
            step = chunk if chunk else max(1, len(dtraj))
            for a in range(0, len(dtraj), step):
                yield itraj, dtraj[a:a + step][:, None]

    def trajectory_length(self, itraj, stride=1, skip=None):
        return self.data_producer.trajectory_length(itraj, stride=stride, skip=skip or 0)

    def trajectory_lengths(self, stride=1, skip=0):
        return self.data_producer.trajectory_lengths(stride=stride, skip=skip)

    def n_frames_total(self, stride=1, skip=0):
        return self.data_producer.n_frames_total(stride=stride, skip=skip)

    def number_of_trajectories(self, stride=None):
        return self.data_producer.number_of_trajectories()

    # ---- files -----------------------------------------------------------
    def save_dtrajs(self, trajfiles=None, prefix="", output_dir=".", output_format="ascii",
                    extension=".dtraj"):
        """Writes the dtrajs as text (output_format='ascii') or .npy files."""
        if extension[0] != ".":
            extension = "." + extension
        if output_format == "ascii":
            def write_dtraj(filename, dtraj):
                with open(filename, "w") as f:
                    np.asarray(dtraj).tofile(f, sep="\n", format="%d")
        else:
            def write_dtraj(filename, dtraj):
                np.save(filename, np.asarray(dtraj))
        output_files = []
        if trajfiles is not None:
            for f in trajfiles:
                basename, _ = os.path.splitext(os.path.split(f)[1])
                output_files.append("%s_%s%s" % (prefix, basename, extension) if prefix != ""
                                    else "%s%s" % (basename, extension))
        else:
            for i in range(len(self.dtrajs)):
                output_files.append("%s_%i%s" % (prefix, i, extension) if prefix != "" else str(i) + extension)
        assert len(self.dtrajs) == len(output_files)
        os.makedirs(output_dir, exist_ok=True)
        for filename, dtraj in zip(output_files, self.dtrajs):
            dest = os.path.join(output_dir, filename)
            try:
                if os.path.exists(dest) and not self.overwrite_dtrajs:
                    raise EnvironmentError('Attempted to write dtraj "%s" which already existed. To automatically'
                                           ' overwrite existing files, set source.overwrite_dtrajs=True.' % dest)
                write_dtraj(dest, dtraj)
            except IOError:
                self.logger.exception('Exception during writing dtraj to "%s"' % dest)


def _index_states(dtrajs):
    """Per state, an (N_i, 2) array of (trajectory, time) indexes."""
    dtrajs = [np.asarray(d) for d in dtrajs]
    nstates = max((int(d.max()) for d in dtrajs if len(d)), default=-1) + 1
    if nstates <= 0:
        return []
    itraj = np.concatenate([np.full(len(d), i, dtype=int) for i, d in enumerate(dtrajs)])
    times = np.concatenate([np.arange(len(d)) for d in dtrajs])
    states = np.concatenate(dtrajs)
    order = np.argsort(states, kind="stable")
    bounds = np.searchsorted(states[order], np.arange(nstates + 1))
    pairs = np.stack([itraj[order], times[order]], axis=1)
    return [pairs[bounds[s]:bounds[s + 1]] for s in range(nstates)]
