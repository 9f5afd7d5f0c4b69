"""Seeded synthetic k-space trajectories and images for tests and benchmarks.

No public dataset is involved: every workload is generated here from a
formula and a seed, with the shapes and value ranges of the MRI workloads it
stands in for.  All trajectories return ``omega`` as float64 ``[M, ndim]`` in
radians, ``omega[:, d]`` pairing with image axis ``d`` (the reference's
convention, mrrt/nufft/_nufft.py:130-133).
"""
import math

import numpy as np

GOLDEN_ANGLE_DEG = 111.246


def radial_readout(n_read):
    """Readout positions r_j = -pi + 2 pi j / n_read, j = 0..n_read-1."""
    return -np.pi + 2 * np.pi * np.arange(n_read) / n_read


def radial_2d(n_spokes, n_read, golden=False, first_spoke=0):
    """2-D radial trajectory, spoke-major sample order.

    ``golden=False``: angles pi s / n_spokes (uniform over a half turn).
    ``golden=True``: angles s * 111.246 degrees.
    """
    s = np.arange(first_spoke, first_spoke + n_spokes, dtype=np.float64)
    theta = s * np.deg2rad(GOLDEN_ANGLE_DEG) if golden else np.pi * s / n_spokes
    r = radial_readout(n_read)
    om0 = (r[None, :] * np.cos(theta)[:, None]).ravel()
    om1 = (r[None, :] * np.sin(theta)[:, None]).ravel()
    return np.stack([om0, om1], axis=-1)


def kooshball_3d(n_spokes, n_read):
    """3-D radial trajectory with spoke directions on a Fibonacci sphere."""
    k = np.arange(n_spokes, dtype=np.float64) + 0.5
    phi = np.arccos(1 - 2 * k / n_spokes)
    vt = np.pi * (1 + math.sqrt(5.0)) * k
    dirs = np.stack([np.sin(phi) * np.cos(vt), np.sin(phi) * np.sin(vt), np.cos(phi)], axis=-1)
    r = radial_readout(n_read)
    return (r[None, :, None] * dirs[:, None, :]).reshape(-1, 3)


def spiral_2d(n_interleaves, n_samples, n_turns=32):
    """Variable-density spiral: tau = (i / n)^1.5, theta = 2 pi n_turns tau + 2 pi l / L."""
    tau = (np.arange(n_samples, dtype=np.float64) / n_samples) ** 1.5
    out = []
    for l in range(n_interleaves):
        theta = 2 * np.pi * n_turns * tau + 2 * np.pi * l / n_interleaves
        out.append(np.stack([np.pi * tau * np.cos(theta), np.pi * tau * np.sin(theta)], axis=-1))
    return np.concatenate(out, axis=0)


def uneven_series_2d(n_frames, n_read, min_spokes=13, max_spokes=89, seed=4):
    """Dynamic series: frame f has U{min..max} golden-angle spokes (seeded).

    Returns a list of per-frame ``omega`` arrays; golden-angle numbering runs
    on across frames.
    """
    rng = np.random.default_rng(seed)
    counts = rng.integers(min_spokes, max_spokes + 1, size=n_frames)
    frames, first = [], 0
    for c in counts:
        frames.append(radial_2d(int(c), n_read, golden=True, first_spoke=first))
        first += int(c)
    return frames


def perturbed_grid(Nd, rel_std=0.5, seed=1234):
    """Jittered Cartesian frequency grid scaled into [0, 2 pi] (the trajectory
    the reference's own tests use, mrrt/nufft/tests/test_nufft.py:20-44)."""
    Nd = np.atleast_1d(np.asarray(Nd))
    rs = np.random.RandomState(seed)
    fs = [2 * np.pi * np.arange(n) / n for n in Nd]
    fs = np.meshgrid(*fs, indexing="ij")
    omega = np.hstack([f.reshape((-1, 1), order="F") for f in fs])
    df = 2 * np.pi / Nd
    for d in range(len(Nd)):
        omega[:, d] += df[d] * rel_std * rs.rand(omega.shape[0])
        omega[:, d] += np.min(omega[:, d])
        omega[:, d] *= (2 * np.pi) / np.max(omega[:, d])
    return omega


def complex_image(shape, seed=0, dtype=np.complex64):
    """i.i.d. N(0,1) real and imaginary parts from ``default_rng(seed)``."""
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(shape) + 1j * rng.standard_normal(shape)).astype(dtype)


def gaussian_coil_maps(Nd, n_coils, sigma_frac=0.3, radius_frac=0.35):
    """Smooth synthetic coil maps: Gaussian blobs of width sigma_frac * max(Nd)
    centred on a circle of radius radius_frac * N in the first two axes (the
    third axis, if any, is centred), each with phase exp(i 2 pi c / C).
    Returns [C, *Nd]."""
    Nd = tuple(Nd)
    axes = np.meshgrid(*[np.arange(n) - n / 2 for n in Nd], indexing="ij")
    sig = sigma_frac * max(Nd)
    maps = []
    for c in range(n_coils):
        ang = 2 * np.pi * c / n_coils
        centre = [radius_frac * Nd[0] * math.cos(ang), radius_frac * Nd[1] * math.sin(ang)]
        centre += [0.0] * (len(Nd) - 2)
        r2 = sum((a - c0) ** 2 for a, c0 in zip(axes, centre))
        maps.append(np.exp(-r2 / (2 * sig * sig)) * np.exp(1j * ang))
    return np.stack(maps, axis=0)
