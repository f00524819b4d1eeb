"""Seeded synthetic trajectories with the shapes of the discretization workloads.

No public dataset is involved; these generators stand in for MD feature
trajectories (the reference ships its own toy generators in
pyemma/datasets).  All take a seed and return float32 arrays.
"""
import numpy as np


def gaussian_mixture(n, d, n_comp, sigma, box, seed):
    """n frames of an equal-weight mixture of isotropic Gaussians, means U[-box, box]^d."""
    rng = np.random.default_rng(seed)
    means = rng.uniform(-box, box, size=(n_comp, d))
    comp = rng.integers(0, n_comp, size=n)
    out = np.empty((n, d), dtype=np.float32)
    step = 1 << 18
    for a in range(0, n, step):
        b = min(n, a + step)
        out[a:b] = means[comp[a:b]] + sigma * rng.standard_normal((b - a, d))
    return out


def small_mixture(seed=0):
    """100,000 x 2: 10 Gaussians, sigma 0.5, means U[-5, 5]^2 (kmeans++ k=50 case)."""
    return gaussian_mixture(100_000, 2, 10, 0.5, 5.0, seed)


def metastable_trajectories(n_traj=20, d=10, lmin=50_000, lmax=500_000, n_states=8, jump_every=5000,
                            seed=0):
    """Uneven AR(1) trajectories with jumps between metastable means.

    Lengths are log-uniform in [lmin, lmax].  Each trajectory is
    x_t = m_{s(t)} + y_t with y_{t+1} = 0.995 y_t + 0.1 eps_t and a state s
    that jumps to a uniformly drawn one of n_states means (U[-3, 3]^d) after
    geometric waiting times of mean jump_every steps.
    """
    from scipy.signal import lfilter
    rng = np.random.default_rng(seed)
    means = rng.uniform(-3.0, 3.0, size=(n_states, d))
    lengths = np.exp(rng.uniform(np.log(lmin), np.log(lmax), size=n_traj)).astype(np.int64)
    trajs = []
    for T in lengths:
        eps = rng.standard_normal((T, d))
        y = lfilter([0.1], [1.0, -0.995], eps, axis=0)
        n_jumps = max(1, int(T // jump_every) * 2 + 2)
        waits = rng.geometric(1.0 / jump_every, size=n_jumps)
        starts = np.concatenate([[0], np.cumsum(waits)])
        states = rng.integers(0, n_states, size=len(starts))
        seg = np.searchsorted(starts, np.arange(T), side="right") - 1
        trajs.append((means[states[seg]] + y).astype(np.float32))
    return trajs


def calpha_distances(n_frames=2_000_000, n_beads=33, bond=0.38, jitter=0.05, n_conf=64, dwell=2000, seed=0,
                     device=None):
    """All i<j pair distances (n_beads*(n_beads-1)/2 features) of a jittered chain.

    n_conf base conformations are 3D random walks with fixed bond length; the
    trajectory dwells on one conformation for geometric times of mean dwell
    frames, and every frame adds Gaussian jitter of sigma `jitter` (nm) to the
    bead coordinates.  Distances come out at about 0.3-6 nm.  With a CUDA
    `device` the frames are generated there (seeded, but a different random
    stream than the NumPy path) and a CUDA tensor is returned.
    """
    if device is not None:
        return _calpha_distances_torch(n_frames, n_beads, bond, jitter, n_conf, dwell, seed, device)
    rng = np.random.default_rng(seed)
    steps = rng.standard_normal((n_conf, n_beads - 1, 3))
    steps *= bond / np.linalg.norm(steps, axis=2, keepdims=True)
    base = np.concatenate([np.zeros((n_conf, 1, 3)), np.cumsum(steps, axis=1)], axis=1)
    waits = rng.geometric(1.0 / dwell, size=n_frames // dwell * 2 + 2)
    starts = np.concatenate([[0], np.cumsum(waits)])
    conf = rng.integers(0, n_conf, size=len(starts))
    iu, ju = np.triu_indices(n_beads, k=1)
    out = np.empty((n_frames, len(iu)), dtype=np.float32)
    step = 1 << 15
    for a in range(0, n_frames, step):
        b = min(n_frames, a + step)
        seg = np.searchsorted(starts, np.arange(a, b), side="right") - 1
        xyz = base[conf[seg]] + jitter * rng.standard_normal((b - a, n_beads, 3))
        diff = xyz[:, iu, :] - xyz[:, ju, :]
        out[a:b] = np.sqrt(np.einsum("fpk,fpk->fp", diff, diff))
    return out


def _calpha_distances_torch(n_frames, n_beads, bond, jitter, n_conf, dwell, seed, device):
    import torch
    rng = np.random.default_rng(seed)
    steps = rng.standard_normal((n_conf, n_beads - 1, 3))
    steps *= bond / np.linalg.norm(steps, axis=2, keepdims=True)
    base = np.concatenate([np.zeros((n_conf, 1, 3)), np.cumsum(steps, axis=1)], axis=1)
    waits = rng.geometric(1.0 / dwell, size=n_frames // dwell * 2 + 2)
    starts = np.concatenate([[0], np.cumsum(waits)])
    conf = rng.integers(0, n_conf, size=len(starts))
    seg = np.searchsorted(starts, np.arange(n_frames), side="right") - 1
    frame_conf = torch.from_numpy(conf[seg]).to(device)
    base_t = torch.from_numpy(base).to(device=device, dtype=torch.float32)
    iu, ju = np.triu_indices(n_beads, k=1)
    iu_t = torch.from_numpy(iu).to(device)
    ju_t = torch.from_numpy(ju).to(device)
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    out = torch.empty((n_frames, len(iu)), dtype=torch.float32, device=device)
    step = 1 << 17
    for a in range(0, n_frames, step):
        b = min(n_frames, a + step)
        xyz = base_t[frame_conf[a:b]] + jitter * torch.randn((b - a, n_beads, 3), generator=gen, device=device)
        diff = xyz[:, iu_t, :] - xyz[:, ju_t, :]
        out[a:b] = torch.sqrt((diff * diff).sum(-1))
    return out


def calpha_coordinates(n_frames=2_000_000, n_beads=33, bond=0.38, jitter=0.05, n_conf=64, dwell=2000, seed=0,
                       device="cuda"):
    """(n_frames, n_beads, 3) float32 C-alpha coordinates of the same jittered
    chain model as calpha_distances (generated on `device`; a CUDA tensor)."""
    import torch
    rng = np.random.default_rng(seed)
    steps = rng.standard_normal((n_conf, n_beads - 1, 3))
    steps *= bond / np.linalg.norm(steps, axis=2, keepdims=True)
    base = np.concatenate([np.zeros((n_conf, 1, 3)), np.cumsum(steps, axis=1)], axis=1)
    waits = rng.geometric(1.0 / dwell, size=n_frames // dwell * 2 + 2)
    starts = np.concatenate([[0], np.cumsum(waits)])
    conf = rng.integers(0, n_conf, size=len(starts))
    seg = np.searchsorted(starts, np.arange(n_frames), side="right") - 1
    frame_conf = torch.from_numpy(conf[seg]).to(device)
    base_t = torch.from_numpy(base).to(device=device, dtype=torch.float32)
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    out = torch.empty((n_frames, n_beads, 3), dtype=torch.float32, device=device)
    step = 1 << 17
    for a in range(0, n_frames, step):
        b = min(n_frames, a + step)
        out[a:b] = base_t[frame_conf[a:b]] + jitter * torch.randn((b - a, n_beads, 3), generator=gen, device=device)
    return out


def sweep_mixture(n, d, k, seed=0):
    """Precision-sweep data: 4k true clusters, sigma 0.3, means U[-5, 5]^d."""
    return gaussian_mixture(n, d, 4 * k, 0.3, 5.0, seed)
