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

__all__ = ["ca_pairs", "ca_distances", "PairDistanceFrames", "pair_distance_frames"]


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


class PairDistanceFrames(object):
    """Atom-pair distance features that are never written out.

    Holds the coordinates (T, n_atoms, 3) and the atom pairs on the device.
    cluster_kmeans, KmeansClustering.estimate, assign_to_centers and the
    estimators' dtrajs / assign / transform accept it in place of the
    (T, n_pairs) feature array: the kernels compute every feature where they
    read it (km_assign_pairs, km_lloyd_pairs, km_kmpp_pairs), with the
    float32 arithmetic of ca_distances, so the results equal those on
    ca_distances(xyz) and no T x n_pairs matrix is allocated.
    """

    def __init__(self, xyz, pairs):
        torch = _lib._torch()
        if isinstance(xyz, np.ndarray):
            xyz = torch.from_numpy(np.ascontiguousarray(xyz, dtype=np.float32))
        if xyz.device.type != "cuda":
            xyz = xyz.to("cuda", non_blocking=xyz.is_pinned())
        xyz = xyz.float().contiguous()
        if xyz.dim() != 3 or xyz.shape[2] != 3:
            raise ValueError("xyz must have shape (T, n_atoms, 3)")
        pairs = np.ascontiguousarray(pairs, dtype=np.int32).reshape(-1, 2)
        if len(pairs) == 0:
            raise ValueError("no atom pairs")
        if pairs.min() < 0 or pairs.max() >= xyz.shape[1]:
            raise ValueError("atom pairs must index atoms in [0, %d)" % xyz.shape[1])
        self.xyz = xyz
        self.pairs_host = pairs
        self.pairs = torch.from_numpy(pairs).to(xyz.device)

    # the parts of the trajectory-source interface the estimators use
    @property
    def n_frames(self):
        return int(self.xyz.shape[0])

    def dimension(self):
        return int(self.pairs.shape[0])

    @property
    def ntraj(self):
        return 1

    def number_of_trajectories(self, stride=None):
        return 1

    def trajectory_length(self, itraj, stride=1, skip=0):
        return max((self.n_frames - skip - 1) // stride + 1, 0)

    def trajectory_lengths(self, stride=1, skip=0):
        return np.array([self.trajectory_length(0, stride, skip)])

    def n_frames_total(self, stride=1, skip=0):
        return self.trajectory_length(0, stride, skip)

    @property
    def default_chunksize(self):
        return self.n_frames

    def strided(self, stride=1, skip=0):
        """The frames [skip::stride] as PairDistanceFrames (a copy of the
        coordinates only when stride or skip changes anything)."""
        if stride == 1 and skip == 0:
            return self
        out = PairDistanceFrames.__new__(PairDistanceFrames)
        out.xyz = self.xyz[skip::stride].contiguous()
        out.pairs_host = self.pairs_host
        out.pairs = self.pairs
        return out

    def features(self, frames=None):
        """The float32 features of the given frames (all when None) as a
        CUDA tensor; km_pair_distances."""
        xyz = self.xyz if frames is None else self.xyz[frames].contiguous()
        return _lib.pair_distances(xyz, self.pairs)


def pair_distance_frames(xyz, excluded_neighbors=2, pairs=None):
    """PairDistanceFrames of C-alpha coordinates (the pairs of ca_distances,
    or explicit atom pairs)."""
    if pairs is None:
        shape = xyz.shape
        pairs = ca_pairs(int(shape[1]), excluded_neighbors)
    return PairDistanceFrames(xyz, pairs)
