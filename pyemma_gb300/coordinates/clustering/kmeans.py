"""k-means estimator on the GPU.

Mirrors KmeansClustering of pyemma/coordinates/clustering/kmeans.py:47-338.
The reference collects all (strided, skipped) frames into one float32 array
(_collect_data, kmeans.py:326-338) and hands it to deeptime's KMeans.fit
(kmeans.py:211-258).  Here the frames are packed into one device-resident
float32 tensor, kmeans++ runs as kernel (d) (km_kmpp) and the Lloyd loop as
kernels (a)/(b) + (c), one CUDA graph launch per iteration (km_lloyd).
"""
import math
import random

import numpy as np

from ... import _lib
from .. import _device
from .interface import AbstractClustering

__all__ = ["KmeansClustering", "MiniBatchKmeansClustering"]


class KmeansClustering(AbstractClustering):
    r"""Kmeans clustering (kmeans.py:47).

    Parameters
    ----------
    n_clusters : int or None
        Number of centers; None gives min(sqrt(N), 5000) for N frames.
    max_iter : int
        Maximum number of Lloyd iterations.
    metric : str
        'euclidean' or 'minRMSD' (atom-major coordinates; assignment by the
        RMSD after optimal superposition, centers as member means).
    tolerance : float
        Stop when the relative change of the inertia
        C(S) = sum_i sum_{x in S_i} ||x - mu_i||^2 is <= tolerance.
    init_strategy : {'kmeans++', 'uniform'}
    fixed_seed : bool or int
        True -> 42, False/None -> a random seed, int in [0, 2^32-1] -> itself.
    oom_strategy : str
        Accepted for compatibility; device memory is checked by the caching
        allocator instead of falling back to a memory map.
    stride, skip : int
        Frames used for estimation: traj[skip::stride].
    n_jobs : int or None
        Accepted for compatibility.
    clustercenters : array (k, d) or None
        Resume from these centers (init_strategy is ignored).
    keep_data : bool
        Keep the device copy of the frames for a later resume.
    precision : {'auto', 'fp32', 'fp16', 'bf16'}
        Distance arithmetic of the assignment step (labels are exact in all
        cases).
    """

    def __init__(self, n_clusters, max_iter=5, metric="euclidean", tolerance=1e-5, init_strategy="kmeans++",
                 fixed_seed=False, oom_strategy="memmap", stride=1, n_jobs=None, skip=0, clustercenters=None,
                 keep_data=False, precision="auto"):
        super(KmeansClustering, self).__init__(metric=metric, n_jobs=n_jobs, precision=precision)
        if clustercenters is None:
            clustercenters = []
        self._in_memory_chunks_set = False
        self._converged = False
        self.inertias = np.zeros(0)
        self.n_iter = 0
        self.set_params(n_clusters=n_clusters, max_iter=max_iter, tolerance=tolerance,
                        init_strategy=init_strategy, oom_strategy=oom_strategy, fixed_seed=fixed_seed,
                        stride=stride, skip=skip, clustercenters=clustercenters, keep_data=keep_data)

    def _param_names(self):
        return ("n_clusters", "max_iter", "metric", "tolerance", "init_strategy", "fixed_seed", "oom_strategy",
                "stride", "n_jobs", "skip", "clustercenters", "keep_data", "precision")

    @property
    def init_strategy(self):
        """Strategy to get an initial guess for the centers."""
        return self._init_strategy

    @init_strategy.setter
    def init_strategy(self, value):
        valid = ("kmeans++", "uniform")
        if value not in valid:
            raise ValueError('invalid parameter "{}" for init_strategy. Should be one of {}'.format(value, valid))
        self._init_strategy = value

    @property
    def fixed_seed(self):
        """Seed of the initial-center draw (kmeans.py:146-164)."""
        return self._fixed_seed

    @fixed_seed.setter
    def fixed_seed(self, val):
        if isinstance(val, bool) or val is None:
            self._fixed_seed = 42 if val else random.randint(0, 2 ** 32 - 1)
        elif isinstance(val, (int, np.integer)):
            if val < 0 or val > 2 ** 32 - 1:
                self.logger.warning("seed has to be positive (or smaller than 2**32-1). Seed will be chosen randomly.")
                self.fixed_seed = False
            else:
                self._fixed_seed = int(val)
        else:
            raise ValueError("fixed seed has to be bool or integer")

    @property
    def converged(self):
        return self._converged

    def describe(self):
        return "[Kmeans, k=%i, inp_dim=%i]" % (self.n_clusters, self.data_producer.dimension())

    def _check_resume_iteration(self):
        return self.clustercenters.size != 0

    # ------------------------------------------------------------------
    def _init_in_memory_chunks(self, size, dim):
        chunks = getattr(self, "_in_memory_chunks", None)
        if chunks is not None and chunks.numel() == size * dim:
            self.logger.debug("re-use in memory data.")
            return True
        if self._check_resume_iteration() and not self._in_memory_chunks_set and not self.keep_data:
            self.logger.warning('Resuming kmeans iteration without the setting "keep_data=True", will re-create'
                                ' the linear in-memory data. This is inefficient! Consider setting keep_data=True,'
                                ' when you intend to resume the kmeans iteration.')
        return False

    def _uniform_indices(self, traj_lengths, total_length):
        # kmeans.py:299-305: per trajectory, a share of the centers proportional to its length.
        old = random.getstate()
        random.seed(self.fixed_seed)
        try:
            return {idx: random.sample(list(range(0, traj_len)),
                                       int(math.ceil((traj_len / float(total_length)) * self.n_clusters)))
                    for idx, traj_len in enumerate(traj_lengths)}
        finally:
            random.setstate(old)

    def _uniform_centers(self, trajs, indices):
        # kmeans.py:314-324: frames in iteration order whose index was drawn, until n_clusters.
        picked = []
        for itraj, X in enumerate(trajs):
            chosen = set(indices.get(itraj, ()))
            for t in range(len(X)):
                if len(picked) >= self.n_clusters:
                    break
                if t in chosen:
                    row = X[t]
                    picked.append(row if isinstance(row, np.ndarray) else row.cpu().numpy())
        dim = trajs[0].shape[1]
        return np.asarray(picked).reshape(-1, dim)

    def _estimate_pairs(self, source):
        """The estimate on PairDistanceFrames: the pair-distance features are
        computed where the kernels read them (km_kmpp_pairs, km_lloyd_pairs).
        The dtrajs are assigned on demand to the final centers
        (km_assign_pairs), as for array input."""
        stride = self.stride if self.stride else 1
        src = source.strided(stride, self.skip)
        total_length = src.n_frames
        if total_length == 0:
            raise ValueError("no frames to cluster (stride=%s, skip=%s)" % (stride, self.skip))
        if not self.n_clusters:
            self.n_clusters = min(int(math.sqrt(total_length)), 5000)
        if self.metric == "minRMSD":
            raise ValueError("minRMSD needs atom coordinates as frames, not pair-distance features")
        dim = src.dimension()
        if not self._check_resume_iteration() and self.init_strategy == "uniform":
            indices = self._uniform_indices(np.array([total_length]), total_length)
            rows = np.array(sorted(indices.get(0, ())), dtype=np.int64)[:self.n_clusters]
            self.clustercenters = src.features(_device.torch_module().from_numpy(rows).to(src.xyz.device)).cpu().numpy()
        # as for array input: the centers known before kmeans++ (none for a
        # kmeans++ start)
        self.initial_centers_ = self.clustercenters[:]
        if self._check_resume_iteration():
            if self.clustercenters.ndim != 2 or self.clustercenters.shape[1] != dim:
                raise ValueError("initial centers have shape %s, data has dimension %d"
                                 % (self.clustercenters.shape, dim))
            C = _device.centers_to_device(self.clustercenters)
        else:
            C, _ = _lib.kmpp_pairs(src.xyz, src.pairs, int(self.n_clusters), self.fixed_seed)
        res = _lib.lloyd_pairs(src.xyz, src.pairs, C, int(self.max_iter), float(self.tolerance),
                               precision=self.precision)
        self.clustercenters = C.cpu().numpy()
        self._converged = res["converged"]
        self.inertias = res["inertias"]
        self.n_iter = res["n_iter"]
        self._in_memory_chunks_set = False
        if not self.converged:
            self.logger.warning("Algorithm did not reach convergence criterion of %g in %i iterations. "
                                "Consider increasing max_iter.", self.tolerance, self.max_iter)
        return self

    def _estimate(self, source):
        from ...featurize import PairDistanceFrames
        if isinstance(source, PairDistanceFrames):
            return self._estimate_pairs(source)
        stride = self.stride if self.stride else 1
        traj_lengths = source.trajectory_lengths(stride=stride, skip=self.skip)
        total_length = int(sum(traj_lengths))
        if total_length == 0:
            raise ValueError("no frames to cluster (stride=%s, skip=%s)" % (stride, self.skip))
        if not self.n_clusters:
            self.n_clusters = min(int(math.sqrt(total_length)), 5000)
            self.logger.info("The number of cluster centers was not specified, "
                             "using min(sqrt(N), 5000)=%s as n_clusters." % self.n_clusters)
        dim = source.dimension()
        minrmsd = self.metric == "minRMSD"
        if minrmsd:
            _device.check_minrmsd_dim(dim)
        reuse = self._init_in_memory_chunks(total_length, dim)

        host_parts = None
        if not self._check_resume_iteration() or not self._in_memory_chunks_set or not reuse:
            trajs = source.frames(stride=stride, skip=self.skip)
            if not self._check_resume_iteration() and self.init_strategy == "uniform":
                indices = self._uniform_indices(traj_lengths, total_length)
                self.clustercenters = self._uniform_centers(trajs, indices)
            if self._check_resume_iteration() and not minrmsd:
                # Centers known (given, or drawn uniformly above) before the
                # frames reach the device: the copy overlaps the first
                # assignment (km_lloyd_host).
                host_parts = _device.host_parts(trajs)
            if host_parts is None:
                self._in_memory_chunks = _device.pack_to_device(trajs, dim)
            self.initial_centers_ = self.clustercenters[:]
            self._in_memory_chunks_set = True
        else:
            if len(self.clustercenters) != self.n_clusters:
                raise RuntimeError("Passed clustercenters do not match n_clusters: {} vs. {}".format(
                    len(self.clustercenters), self.n_clusters))

        try:
            if self._check_resume_iteration():
                if self.clustercenters.ndim != 2 or self.clustercenters.shape[1] != dim:
                    raise ValueError("initial centers have shape %s, data has dimension %d"
                                     % (self.clustercenters.shape, dim))
                C = _device.centers_to_device(self.clustercenters)
            elif minrmsd:
                C, _ = _lib.kmpp_minrmsd(self._in_memory_chunks, int(self.n_clusters), self.fixed_seed)
            else:
                C, _ = _lib.kmpp(self._in_memory_chunks, int(self.n_clusters), self.fixed_seed)
            if minrmsd:
                res = _lib.lloyd_minrmsd(self._in_memory_chunks, C, int(self.max_iter), float(self.tolerance))
            elif host_parts is not None:
                res = _lib.lloyd_host(host_parts, C, int(self.max_iter), float(self.tolerance),
                                      precision=self.precision)
                self._in_memory_chunks = res["X"]
            else:
                res = _lib.lloyd(self._in_memory_chunks, C, int(self.max_iter), float(self.tolerance),
                                 precision=self.precision)
            self.clustercenters = C.cpu().numpy()
            self._converged = res["converged"]
            self.inertias = res["inertias"]
            self.n_iter = res["n_iter"]
        finally:
            if not self.keep_data or self._converged or not hasattr(self, "_in_memory_chunks"):
                if hasattr(self, "_in_memory_chunks"):
                    del self._in_memory_chunks
                self._in_memory_chunks_set = False

        if self.converged:
            self.logger.debug("Cluster centers converged after %i steps.", self.n_iter)
        else:
            self.logger.warning("Algorithm did not reach convergence criterion of %g in %i iterations. "
                                "Consider increasing max_iter.", self.tolerance, self.max_iter)
        return self


class MiniBatchKmeansClustering(KmeansClustering):
    r"""Mini-batch k-means clustering (kmeans.py:340-447).

    Every pass draws a random sample of ``batch_size`` of the frames (per
    trajectory in proportion to its length, without replacement, in time
    order; kmeans.py:363-398) and performs one Lloyd step (assignment, mean
    of the members, inertia of the sample) on it from the current centers.
    The first pass starts from kmeans++ (or uniform) centers of its sample.
    Passes stop when the relative change of the sample inertia is at most
    ``tolerance`` or after ``max_iter`` passes.
    """

    def __init__(self, n_clusters, max_iter=5, metric="euclidean", tolerance=1e-5, init_strategy="kmeans++",
                 batch_size=0.2, oom_strategy="memmap", fixed_seed=False, stride=None, n_jobs=None, skip=0,
                 clustercenters=None, keep_data=False, precision="auto"):
        if stride is not None:
            raise ValueError("stride is a dummy value in MiniBatch Kmeans")
        if batch_size > 1:
            raise ValueError("batch_size should be less or equal to 1, but was %s" % batch_size)
        if keep_data:
            raise ValueError("keep_data is a dummy value in MiniBatch Kmeans")
        super(MiniBatchKmeansClustering, self).__init__(n_clusters, max_iter, metric, tolerance, init_strategy,
                                                        False, oom_strategy, stride=stride, n_jobs=n_jobs,
                                                        skip=skip, clustercenters=clustercenters, keep_data=False,
                                                        precision=precision)
        self.batch_size = batch_size

    def _param_names(self):
        return KmeansClustering._param_names(self) + ("batch_size",)

    def _sample_sizes(self, traj_lengths):
        total = int(sum(traj_lengths))
        samples = int(math.ceil(total * self.batch_size))
        return [int(math.floor(L / float(total) * samples)) for L in traj_lengths]

    def _draw_sample(self, frames, sizes):
        parts = []
        for X, m in zip(frames, sizes):
            if m == 0:
                continue
            choice = np.sort(np.random.choice(len(X), m, replace=False))
            if not isinstance(X, np.ndarray):  # frames on the GPU (torch tensor)
                import torch
                parts.append(X[torch.from_numpy(choice).to(X.device)].float())
            else:
                parts.append(np.asarray(X[choice], dtype=np.float32))
        return parts

    def _estimate(self, source):
        self.stride = None
        frames = source.frames(stride=1, skip=self.skip)
        traj_lengths = [len(X) for X in frames]
        if sum(traj_lengths) == 0:
            raise ValueError("no frames to cluster (skip=%s)" % self.skip)
        if not self.n_clusters:
            self.n_clusters = min(int(math.sqrt(sum(traj_lengths))), 5000)
        sizes = self._sample_sizes(traj_lengths)
        if sum(sizes) == 0:
            raise ValueError("batch_size %s selects no frames" % self.batch_size)
        dim = source.dimension()
        minrmsd = self.metric == "minRMSD"
        if minrmsd:
            _device.check_minrmsd_dim(dim)
        C = None
        if self._check_resume_iteration():
            C = _device.centers_to_device(self.clustercenters)
        self._converged = False
        prev_cost = 0.0
        i_pass = 0
        inertias = []
        while not (self._converged or i_pass + 1 > self.max_iter):
            Xb = _device.pack_to_device(self._draw_sample(frames, sizes), dim)
            if C is None:
                if self.init_strategy == "uniform":
                    idx = np.random.choice(Xb.shape[0], int(self.n_clusters), replace=False)
                    C = Xb[_device.torch_module().from_numpy(np.sort(idx)).to(Xb.device)].contiguous()
                else:
                    seed = int(np.random.randint(0, 2 ** 32 - 1, dtype=np.int64))
                    C, _ = (_lib.kmpp_minrmsd if minrmsd else _lib.kmpp)(Xb, int(self.n_clusters), seed)
                self.initial_centers_ = C.cpu().numpy()
            if minrmsd:
                res = _lib.lloyd_minrmsd(Xb, C, 1, -1.0)
            else:
                res = _lib.lloyd(Xb, C, 1, -1.0, precision=self.precision)
            cost = float(res["inertias"][0])
            inertias.append(cost)
            rel_change = abs(cost - prev_cost) / cost if cost != 0.0 else 0.0
            prev_cost = cost
            if rel_change <= self.tolerance:
                self._converged = True
                self.logger.info("Cluster centers converged after %i steps.", i_pass + 1)
            i_pass += 1
            del Xb
        self.clustercenters = C.cpu().numpy()
        self.inertias = np.asarray(inertias)
        self.n_iter = i_pass
        if not self._converged:
            self.logger.info("Algorithm did not reach convergence criterion of %g in %i iterations. "
                             "Consider increasing max_iter.", self.tolerance, self.max_iter)
        return self
