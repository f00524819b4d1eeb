"""User API: cluster_kmeans, assign_to_centers and the sibling estimators.

Same signatures and outputs as pyemma.coordinates.cluster_kmeans
(pyemma/coordinates/api.py:1727-1867), assign_to_centers (api.py:2060-2156),
cluster_mini_batch_kmeans (api.py:1671-1725), cluster_uniform_time
(api.py:1870-1951) and cluster_regspace (api.py:1953-2057), plus an optional
``precision`` keyword.
"""
from .clustering.assign import AssignCenters
from .clustering.kmeans import KmeansClustering, MiniBatchKmeansClustering
from .clustering.regspace import RegularSpaceClustering
from .clustering.uniform_time import UniformTimeClustering

__all__ = ["cluster_kmeans", "assign_to_centers", "cluster_mini_batch_kmeans", "cluster_uniform_time",
           "cluster_regspace"]


def _chunksize(chunksize, kwargs):
    # api.py _check_old_chunksize_arg: the old spelling 'chunk_size' is still accepted.
    if "chunk_size" in kwargs:
        if chunksize is not None:
            raise ValueError("both chunksize and chunk_size given")
        chunksize = kwargs.pop("chunk_size")
    if kwargs:
        raise TypeError("unexpected keyword arguments: %s" % sorted(kwargs))
    return chunksize


def cluster_kmeans(data=None, k=None, max_iter=10, tolerance=1e-5, stride=1, metric="euclidean",
                   init_strategy="kmeans++", fixed_seed=False, n_jobs=None, chunksize=None, skip=0,
                   keep_data=False, clustercenters=None, precision="auto", **kwargs):
    r"""k-means clustering; returns a KmeansClustering object.

    If data is given, kmeans++ (or uniform) initialisation and Lloyd
    iterations run on the GPU; the object then holds ``clustercenters`` and
    the int32 ``dtrajs`` of the data.  Parameters as in PyEMMA
    (api.py:1727); ``precision`` selects the distance arithmetic of the
    assignment step ('auto', 'fp32', 'fp16', 'bf16'; the labels are exact in all
    cases).
    """
    res = KmeansClustering(n_clusters=k, max_iter=max_iter, metric=metric, tolerance=tolerance,
                           init_strategy=init_strategy, fixed_seed=fixed_seed, n_jobs=n_jobs, skip=skip,
                           keep_data=keep_data, clustercenters=clustercenters, stride=stride, precision=precision)
    cs = _chunksize(chunksize, kwargs)
    if data is not None:
        res.estimate(data, chunksize=cs)
    else:
        res.chunksize = cs
    return res


def assign_to_centers(data=None, centers=None, stride=1, return_dtrajs=True, metric="euclidean", n_jobs=None,
                      chunksize=None, skip=0, precision="auto", **kwargs):
    r"""Assigns data to the nearest cluster centers (Voronoi discretization).

    Returns the list of int32 discrete trajectories (return_dtrajs=True and
    data given) or the AssignCenters object.  Parameters as in PyEMMA
    (api.py:2060).
    """
    if centers is None:
        raise ValueError("You have to provide centers in form of a filename"
                         " or NumPy array or a reader created by source function")
    res = AssignCenters(centers, metric=metric, n_jobs=n_jobs, skip=skip, stride=stride, precision=precision)
    cs = _chunksize(chunksize, kwargs)
    if data is not None:
        res.estimate(data, chunksize=cs)
        if return_dtrajs:
            return res.dtrajs
    else:
        res.chunksize = cs
    return res


def cluster_mini_batch_kmeans(data=None, k=100, max_iter=10, batch_size=0.2, metric="euclidean",
                              init_strategy="kmeans++", n_jobs=None, chunksize=None, skip=0, clustercenters=None,
                              precision="auto", **kwargs):
    r"""k-means with mini-batches (api.py:1671); returns a MiniBatchKmeansClustering object."""
    res = MiniBatchKmeansClustering(n_clusters=k, max_iter=max_iter, metric=metric, init_strategy=init_strategy,
                                    batch_size=batch_size, n_jobs=n_jobs, skip=skip, clustercenters=clustercenters,
                                    precision=precision)
    cs = _chunksize(chunksize, kwargs)
    if data is not None:
        res.estimate(data, chunksize=cs)
    else:
        res.chunksize = cs
    return res


def cluster_uniform_time(data=None, k=None, stride=1, metric="euclidean", n_jobs=None, chunksize=None, skip=0,
                         precision="auto", **kwargs):
    r"""Uniform time clustering (api.py:1870); returns a UniformTimeClustering object."""
    res = UniformTimeClustering(k, metric=metric, n_jobs=n_jobs, skip=skip, stride=stride, precision=precision)
    cs = _chunksize(chunksize, kwargs)
    if data is not None:
        res.estimate(data, chunksize=cs)
    else:
        res.chunksize = cs
    return res


def cluster_regspace(data=None, dmin=-1, max_centers=1000, stride=1, metric="euclidean", n_jobs=None,
                     chunksize=None, skip=0, precision="auto", **kwargs):
    r"""Regular space clustering (api.py:1953); returns a RegularSpaceClustering object."""
    if dmin == -1:
        raise ValueError("provide a minimum distance for clustering, e.g. 2.0")
    res = RegularSpaceClustering(dmin, max_centers=max_centers, metric=metric, n_jobs=n_jobs, stride=stride,
                                 skip=skip, precision=precision)
    cs = _chunksize(chunksize, kwargs)
    if data is not None:
        res.estimate(data, chunksize=cs)
    else:
        res.chunksize = cs
    return res
