"""C-alpha pair-distance features computed on the device.

The reference featurizes on the host (pyemma/coordinates/data/featurization/
featurizer.py:337-372, add_distances_ca -> mdtraj.compute_distances) and
hands the (T, n_pairs) float32 features to the clustering.  Here the
coordinates go to the GPU (n_atoms * 12 bytes per frame) and km_pair_distances
writes the features into device memory, where cluster_kmeans /
assign_to_centers take them without another copy.
"""
import numpy as np

from . import _lib

__all__ = ["ca_pairs", "ca_distances"]


def ca_pairs(n_atoms, excluded_neighbors=2):
    """Pairs (i, j), i < j, j > i + excluded_neighbors, in the order of
    Featurizer.pairs (featurizer.py:198-235) for consecutive residues."""
    p = [(i, j) for i in range(n_atoms) for j in range(i + 1, n_atoms) if j > i + excluded_neighbors]
    return np.asarray(p, dtype=np.int32).reshape(-1, 2)


def ca_distances(xyz, excluded_neighbors=2, pairs=None):
    """Distance features of C-alpha coordinates.

    Parameters
    ----------
    xyz : (T, n_atoms, 3) float32 array (host, pinned host or CUDA tensor)
        One coordinate per residue (C-alpha), in nm.
    excluded_neighbors : int
        As add_distances_ca: pairs of residues closer than this in sequence
        are left out.
    pairs : (m, 2) int array or None
        Explicit atom pairs (add_distances) instead of the C-alpha rule.

    Returns a (T, n_pairs) float32 CUDA tensor.
    """
    torch = _lib._torch()
    if isinstance(xyz, np.ndarray):
        xyz = torch.from_numpy(np.ascontiguousarray(xyz, dtype=np.float32))
    if xyz.device.type != "cuda":
        xyz = xyz.to("cuda", non_blocking=xyz.is_pinned())
    xyz = xyz.float().contiguous()
    if xyz.dim() != 3 or xyz.shape[2] != 3:
        raise ValueError("xyz must have shape (T, n_atoms, 3)")
    if pairs is None:
        pairs = ca_pairs(xyz.shape[1], excluded_neighbors)
    pairs_d = torch.from_numpy(np.ascontiguousarray(pairs, dtype=np.int32)).to(xyz.device)
    return _lib.pair_distances(xyz, pairs_d)
