"""Transition counts of discrete trajectories on the GPU.

The step after discretization in PyEMMA's pipeline: the lag-tau count matrix
of pyemma/msm/estimators/_dtraj_stats.py:139-145 (deeptime
count_matrix(dtrajs, lag, sliding=...) / TransitionCountEstimator), computed
by km_count_matrix over trajectories packed back to back.
"""
import numpy as np

from . import _lib

__all__ = ["count_matrix"]


def count_matrix(dtrajs, lag, sliding=True, nstates=None, sparse=True):
    r"""Lag-``lag`` transition count matrix of one or more int32 dtrajs.

    Parameters
    ----------
    dtrajs : array or list of arrays of int
        Discrete trajectories; negative states (unassigned frames) are left
        out.
    lag : int
        Lag time in trajectory steps.
    sliding : bool
        Sliding-window counts (T - lag per trajectory) or one count per lag
        step (``count_mode='sample'``).
    nstates : int or None
        Matrix size; None gives the largest state + 1.
    sparse : bool
        Return a scipy.sparse.csr_matrix (as the reference) instead of a
        dense int64 array.
    """
    import torch
    if isinstance(dtrajs, np.ndarray) and dtrajs.ndim == 1:
        dtrajs = [dtrajs]
    dtrajs = [np.ascontiguousarray(d, dtype=np.int32).ravel() for d in dtrajs]
    if int(lag) < 1:
        raise ValueError("lag must be >= 1")
    if nstates is None:
        nstates = max((int(d.max()) for d in dtrajs if len(d)), default=-1) + 1
    nstates = max(1, int(nstates))
    offsets = np.concatenate([[0], np.cumsum([len(d) for d in dtrajs])]).astype(np.int64)
    packed = torch.from_numpy(np.concatenate(dtrajs) if dtrajs else np.zeros(0, np.int32)).cuda()
    C = _lib.count_matrix(packed, offsets, int(lag), nstates, sliding=sliding).cpu().numpy()
    if sparse:
        import scipy.sparse
        return scipy.sparse.csr_matrix(C)
    return C
