"""The deeptime.clustering surface that PyEMMA's estimators call, on libkmgpu.

PyEMMA holds no k-means arithmetic of its own.  It imports ``metrics``,
``KMeans`` and ``MiniBatchKMeans`` (pyemma/coordinates/clustering/
kmeans.py:39), ``ClusterModel`` (interface.py:29) and ``RegularSpace``
(regspace.py:34) from deeptime.clustering and calls them at
kmeans.py:211-214,253-258 and 400-426, interface.py:164-165 and
regspace.py:144-170.  This module offers those names with the same call
shapes, running on this package's GPU kernels; :func:`install` makes
``import deeptime.clustering`` resolve to it when deeptime itself is absent,
so that PyEMMA's own estimator code runs unchanged on the GPU.

Metrics are 'euclidean' and 'minRMSD'.  ``metrics.register(name, impl)``
(the call at regspace.py:89) records ``impl`` for ``metrics[name]``; the
estimators here always run their own kernels for the two metrics they know
and reject any other name.

Seeds (``fixed_seed`` of KMeans, ``random_seed`` of init_centers_kmpp):
True -> 42, False / None / a value outside [0, 2^32 - 1] (deeptime's -1) ->
a random seed, an int in range -> itself, as kmeans.py:146-164 resolves them.
"""
import random
import sys

import numpy as np

from . import _lib
from .coordinates import _device
from .coordinates.clustering.regspace import minrmsd_leader_walk

__all__ = ["KMeans", "KMeansModel", "MiniBatchKMeans", "ClusterModel", "RegularSpace", "metrics",
           "MaxCentersReachedException", "install", "uninstall"]

_METRICS = ("euclidean", "minRMSD")


def _check_metric(metric):
    if metric not in _METRICS:
        raise ValueError("metric %r is not supported; use one of %s" % (metric, list(_METRICS)))
    return metric


def _seed(fixed_seed):
    if fixed_seed is None or isinstance(fixed_seed, (bool, np.bool_)):
        return 42 if fixed_seed else random.randint(0, 2 ** 32 - 1)
    s = int(fixed_seed)
    if s < 0 or s > 2 ** 32 - 1:
        return random.randint(0, 2 ** 32 - 1)
    return s


def _frames(data, metric):
    """data as one contiguous float32 (n, d) CUDA tensor (the float32 cast of
    interface.py:159 happens in the copy)."""
    torch = _device.torch_module()
    if not isinstance(data, torch.Tensor):
        data = np.asarray(data)
    if data.ndim != 2:
        raise ValueError("data must be two-dimensional (frames, features), got shape %s" % (tuple(data.shape),))
    if metric == "minRMSD":
        _device.check_minrmsd_dim(data.shape[1])
    return _device.pack_to_device([data], data.shape[1])


def _centers(centers):
    if centers is None:
        return None
    c = np.ascontiguousarray(centers, dtype=np.float32)
    if c.ndim != 2:
        raise ValueError("cluster centers have to be two-dimensional, got shape %s" % (c.shape,))
    return c


def _kmpp(X, k, seed, metric, callback=None):
    fn = _lib.kmpp_minrmsd if metric == "minRMSD" else _lib.kmpp
    C, _ = fn(X, int(k), seed, callback=callback)
    return C


def _uniform(X, k, seed):
    """k distinct frames, drawn with numpy's RandomState(seed), in frame order."""
    torch = _device.torch_module()
    n = X.shape[0]
    if k > n:
        raise ValueError("cannot draw %d centers from %d frames" % (k, n))
    idx = np.sort(np.random.RandomState(seed).choice(n, int(k), replace=False))
    return X[torch.from_numpy(idx).to(X.device)].contiguous()


class ClusterModel(object):
    """Centers and the nearest-center transform (interface.py:164-166)."""

    def __init__(self, cluster_centers=None, metric="euclidean", converged=False):
        self.cluster_centers = _centers(cluster_centers)
        self.metric = _check_metric(metric)
        self.converged = bool(converged)

    @property
    def n_clusters(self):
        return 0 if self.cluster_centers is None else self.cluster_centers.shape[0]

    @property
    def dim(self):
        return None if self.cluster_centers is None else self.cluster_centers.shape[1]

    def transform(self, data, n_jobs=None):
        """int32 label of the nearest center for every frame, shape (T,)."""
        if self.cluster_centers is None or self.n_clusters == 0:
            raise ValueError("the model has no cluster centers")
        labels, _ = _device.assign_trajs([data], self.cluster_centers, metric=self.metric)
        return labels[0]


class KMeansModel(ClusterModel):
    """A fitted k-means model: centers, the inertia of every iteration and
    the convergence flag (kmeans.py:255-262)."""

    def __init__(self, cluster_centers, metric="euclidean", tolerance=1e-5, inertias=None, converged=False):
        super(KMeansModel, self).__init__(cluster_centers, metric=metric, converged=converged)
        self.tolerance = float(tolerance)
        self.inertias = np.zeros(0) if inertias is None else np.asarray(inertias, dtype=np.float64)

    @property
    def inertia(self):
        """The inertia of the last iteration (None before any)."""
        return float(self.inertias[-1]) if len(self.inertias) else None


class KMeans(object):
    """k-means with kmeans++ or uniform initialisation and Lloyd iterations
    (the estimator built at kmeans.py:211-212 and fitted at :253-258)."""

    def __init__(self, n_clusters, max_iter=500, metric="euclidean", tolerance=1e-5, init_strategy="kmeans++",
                 fixed_seed=False, n_jobs=None, initial_centers=None, precision="auto"):
        if init_strategy not in ("kmeans++", "uniform"):
            raise ValueError('invalid init_strategy "%s"; use "kmeans++" or "uniform"' % init_strategy)
        if int(n_clusters) < 1:
            raise ValueError("n_clusters must be at least 1, got %s" % n_clusters)
        if int(max_iter) < 0:
            raise ValueError("max_iter must not be negative, got %s" % max_iter)
        self.n_clusters = int(n_clusters)
        self.max_iter = int(max_iter)
        self.metric = _check_metric(metric)
        self.tolerance = float(tolerance)
        self.init_strategy = init_strategy
        self.fixed_seed = fixed_seed
        self.n_jobs = n_jobs
        self.precision = precision
        self.initial_centers = initial_centers
        self._model = None

    @property
    def initial_centers(self):
        """Centers to start the Lloyd iterations from (skips the initialisation)."""
        return self._initial_centers

    @initial_centers.setter
    def initial_centers(self, value):
        self._initial_centers = _centers(value)

    def _start(self, X, callback=None):
        if self.initial_centers is not None:
            c = self.initial_centers
            if c.shape[0] != self.n_clusters or c.shape[1] != X.shape[1]:
                raise ValueError("initial centers have shape %s, expected (%d, %d)"
                                 % (c.shape, self.n_clusters, X.shape[1]))
            return _device.centers_to_device(c)
        if self.init_strategy == "kmeans++":
            return _kmpp(X, self.n_clusters, _seed(self.fixed_seed), self.metric, callback)
        return _uniform(X, self.n_clusters, _seed(self.fixed_seed))

    def fit(self, data, callback_init_centers=None, callback_loop=None, n_jobs=None, **kwargs):
        """Initial centers (unless given), then Lloyd iterations until the
        relative change of the inertia is at most ``tolerance`` or ``max_iter``
        iterations ran.  callback_init_centers fires once per kmeans++ center,
        callback_loop once per iteration."""
        X = _frames(data, self.metric)
        C = self._start(X, callback_init_centers)
        if self.metric == "minRMSD":
            res = _lib.lloyd_minrmsd(X, C, self.max_iter, self.tolerance, callback=callback_loop)
        else:
            res = _lib.lloyd(X, C, self.max_iter, self.tolerance, precision=self.precision, callback=callback_loop)
        self._model = KMeansModel(C.cpu().numpy(), metric=self.metric, tolerance=self.tolerance,
                                  inertias=res["inertias"], converged=res["converged"])
        return self

    def fetch_model(self):
        """The fitted KMeansModel, or None before fit."""
        return self._model

    def transform(self, data, n_jobs=None):
        if self._model is None:
            raise ValueError("fit the estimator before transforming data")
        return self._model.transform(data)


class MiniBatchKMeans(KMeans):
    """Mini-batch k-means driven by partial_fit (kmeans.py:400-426): every
    call performs one Lloyd step on the given sample from the current centers
    (the first call initialises them on that sample)."""

    def __init__(self, n_clusters, batch_size=100, max_iter=5, metric="euclidean", tolerance=1e-5,
                 init_strategy="kmeans++", fixed_seed=False, n_jobs=None, initial_centers=None, precision="auto"):
        super(MiniBatchKMeans, self).__init__(n_clusters, max_iter=max_iter, metric=metric, tolerance=tolerance,
                                              init_strategy=init_strategy, fixed_seed=fixed_seed, n_jobs=n_jobs,
                                              initial_centers=initial_centers, precision=precision)
        self.batch_size = batch_size

    def partial_fit(self, data, n_jobs=None):
        X = _frames(data, self.metric)
        if self._model is None:
            C = self._start(X)
        else:
            C = _device.centers_to_device(self._model.cluster_centers)
        if self.metric == "minRMSD":
            res = _lib.lloyd_minrmsd(X, C, 1, -1.0)
        else:
            res = _lib.lloyd(X, C, 1, -1.0, precision=self.precision)
        self._model = KMeansModel(C.cpu().numpy(), metric=self.metric, tolerance=self.tolerance,
                                  inertias=res["inertias"][:1], converged=False)
        return self

    def fit(self, data, callback_init_centers=None, callback_loop=None, n_jobs=None, **kwargs):
        raise NotImplementedError("mini-batch k-means is driven by partial_fit, as kmeans.py:400-426 does")


class MaxCentersReachedException(Exception):
    """A (max_centers + 1)-th center was about to be added; PyEMMA matches
    this class name (regspace.py:153-163)."""


class RegularSpace(object):
    """The regular space leader walk (regspace.py:144-152): a frame becomes a
    center when its distance to every center so far is at least dmin."""

    def __init__(self, dmin, max_centers=1000, metric="euclidean", n_jobs=None):
        if float(dmin) < 0:
            raise ValueError("dmin has to be positive, got %s" % dmin)
        if int(max_centers) < 1:
            raise ValueError("max_centers has to be at least 1, got %s" % max_centers)
        self.dmin = float(dmin)
        self.max_centers = int(max_centers)
        self.metric = _check_metric(metric)
        self.n_jobs = n_jobs
        self._centers = None

    def partial_fit(self, data, n_jobs=None):
        """Continues the walk over the frames of data.

        The centers found so far are walked again ahead of the new frames:
        each of them was accepted against exactly the centers before it, with
        the same arithmetic, so the walk keeps them all and then goes on.
        Raises MaxCentersReachedException when the walk stops at max_centers;
        the centers found stay in the model."""
        X = _frames(data, self.metric)
        if self._centers is not None and len(self._centers):
            if self._centers.shape[1] != X.shape[1]:
                raise ValueError("data has dimension %d, the centers %d" % (X.shape[1], self._centers.shape[1]))
            torch = _device.torch_module()
            X = torch.cat([_device.centers_to_device(self._centers), X]).contiguous()
        if self.metric == "minRMSD":
            torch = _device.torch_module()
            idx, converged = minrmsd_leader_walk(X, self.dmin, self.max_centers)
            C = X[torch.tensor(idx, dtype=torch.int64, device=X.device)]
        else:
            C, converged = _lib.regspace(X, self.dmin, self.max_centers)
        self._centers = C.cpu().numpy()
        if not converged:
            raise MaxCentersReachedException("Maximum number of cluster centers (%d) reached" % self.max_centers)
        return self

    def fit(self, data, n_jobs=None):
        self._centers = None
        return self.partial_fit(data, n_jobs=n_jobs)

    def fetch_model(self):
        """ClusterModel of the centers found so far, or None before any frame."""
        if self._centers is None:
            return None
        return ClusterModel(self._centers, metric=self.metric)


class _KmppBinding(object):
    def __init__(self, metric):
        self._metric = metric

    def init_centers_kmpp(self, X, k, random_seed=-1, n_threads=None, callback=None):
        """kmeans++ centers (k, d) float32 of X (the binding test_kmeans.py:304
        calls); random_seed -1 draws a random seed."""
        Xd = _frames(X, self._metric)
        return _kmpp(Xd, k, _seed(random_seed), self._metric, callback).cpu().numpy()


class _EuclideanImpl(object):
    """metrics['euclidean']: the kmeans++ binding."""

    name = "euclidean"

    def __init__(self):
        self.kmeans = _KmppBinding(self.name)


class _MinRMSDImpl(_EuclideanImpl):
    """metrics['minRMSD']: the kmeans++ binding and compute_metric
    (clustering_module.cpp:46-48)."""

    name = "minRMSD"

    def compute_metric(self, x, y):
        """minRMSD of two frames (3 n_atoms values each, atom-major)."""
        torch = _device.torch_module()
        a = np.ascontiguousarray(x, dtype=np.float32).reshape(1, -1)
        b = np.ascontiguousarray(y, dtype=np.float32).reshape(1, -1)
        if a.shape != b.shape:
            raise ValueError("frames of different sizes: %d and %d" % (a.shape[1], b.shape[1]))
        _device.check_minrmsd_dim(a.shape[1])
        dev = _device.device()
        out = _lib.minrmsd_rows(torch.from_numpy(a).to(dev), torch.from_numpy(b).to(dev))
        return float(out[0].item())


class _Metrics(object):
    """Registry of metric implementations (deeptime.clustering.metrics)."""

    def __init__(self):
        self._impls = {"euclidean": _EuclideanImpl(), "minRMSD": _MinRMSDImpl()}

    def register(self, name, impl):
        self._impls[name] = impl

    def __getitem__(self, name):
        return self._impls[name]

    def __contains__(self, name):
        return name in self._impls

    @property
    def available(self):
        return list(self._impls)


metrics = _Metrics()

_INSTALLED = []


def install(force=False):
    """Makes ``import deeptime.clustering`` resolve to this module.

    Does nothing and returns False when a real deeptime is importable (unless
    force); returns True when the module was put in place."""
    import importlib.util
    import types
    if not force:
        try:
            if importlib.util.find_spec("deeptime") is not None:
                return False
        except (ImportError, ValueError):
            pass
    saved = {name: sys.modules.get(name) for name in ("deeptime", "deeptime.clustering")}
    pkg = types.ModuleType("deeptime")
    pkg.__path__ = []
    pkg.__doc__ = "deeptime names backed by pyemma_gb300 (clustering only)."
    me = sys.modules[__name__]
    pkg.clustering = me
    sys.modules["deeptime"] = pkg
    sys.modules["deeptime.clustering"] = me
    _INSTALLED.append(saved)
    return True


def uninstall():
    """Undoes the last install()."""
    if not _INSTALLED:
        return
    for name, mod in _INSTALLED.pop().items():
        if mod is None:
            sys.modules.pop(name, None)
        else:
            sys.modules[name] = mod
