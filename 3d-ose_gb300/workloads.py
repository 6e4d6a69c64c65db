"""Seeded synthetic workloads of the benchmark configurations (velocity model in
the reference layout [x][y][z], float32, plus the modeler parameters).

No public dataset is involved: each model is generated from a fixed seed with
the shapes, sizes and value ranges the configuration names.
"""
from __future__ import annotations

import numpy as np


def smooth_random_salt(nx: int, ny: int, nz: int, seed: int = 2024, vmin: float = 1500.0,
                       vmax: float = 4500.0, sigma: float = 6.0) -> np.ndarray:
    """Gaussian-smoothed random field rescaled to [vmin, vmax], increasing on
    average with depth, with a salt-like ellipsoid at vmax."""
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(seed)
    f = gaussian_filter(rng.standard_normal((nx, ny, nz)), sigma=sigma, mode="wrap")
    f = (f - f.min()) / max(f.max() - f.min(), 1e-12)
    depth = np.linspace(0.0, 1.0, nz)[None, None, :]
    v = vmin + (vmax - vmin) * np.clip(0.6 * depth + 0.4 * f, 0.0, 1.0)
    x, y, z = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    ell = (((x - 0.5 * nx) / (0.22 * nx)) ** 2 + ((y - 0.55 * ny) / (0.18 * ny)) ** 2 +
           ((z - 0.6 * nz) / (0.12 * nz)) ** 2) <= 1.0
    v[ell] = vmax
    return np.ascontiguousarray(v, dtype=np.float32)


def layered_perturbed(nx: int, ny: int, nz: int, seed: int = 7) -> np.ndarray:
    """Four horizontal layers 1500/2200/3000/3800 m/s at depth quarters times
    (1 + d), d a Gaussian-smoothed (sigma = 3 cells) normal field scaled to
    max |d| = 0.05."""
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(seed)
    z = np.arange(nz)
    base = np.choose(np.minimum(4 * z // nz, 3), [1500.0, 2200.0, 3000.0, 3800.0])
    d = gaussian_filter(rng.standard_normal((nx, ny, nz)), sigma=3.0, mode="nearest")
    d *= 0.05 / np.abs(d).max()
    return np.ascontiguousarray(base[None, None, :] * (1.0 + d), dtype=np.float32)


# name -> (model builder, modeler parameters)
CONFIGS = {
    # Plain OSE, FP32, padded 256^3 = interior 196^3 + 30-cell sponge, 25 Hz Ricker
    # near the surface centre, dt 2 ms, 2000 steps, full-surface receivers.
    "ose256": (lambda: smooth_random_salt(196, 196, 196),
               dict(nx=196, ny=196, nz=196, bu=30, bd=30, bl=30, br=30, bf=30, bb=30, nt=2000,
                    fm=25.0, dt=0.002, amp=100.0, dx=10.0, dy=10.0, dz=10.0,
                    sxbeg=98, sybeg=98, szbeg=5, gzbeg=0)),
    # Non-power-of-two variant: padded 320 x 288 x 256.
    "ose320x288x256": (lambda: smooth_random_salt(260, 228, 196, seed=2025),
                       dict(nx=260, ny=228, nz=196, bu=30, bd=30, bl=30, br=30, bf=30, bb=30,
                            nt=2000, fm=25.0, dt=0.002, amp=100.0, dx=10.0, dy=10.0, dz=10.0,
                            sxbeg=130, sybeg=114, szbeg=5, gzbeg=0)),
    # Precision-form workload: padded 384 x 384 x 256 = interior 324 x 324 x 196
    # + 30-cell sponge, same velocity generator, 15 Hz Ricker, 1500 steps.
    "ose384x384x256": (lambda: smooth_random_salt(324, 324, 196, seed=2026),
                       dict(nx=324, ny=324, nz=196, bu=30, bd=30, bl=30, br=30, bf=30, bb=30,
                            nt=1500, fm=15.0, dt=0.002, amp=100.0, dx=10.0, dy=10.0, dz=10.0,
                            sxbeg=162, sybeg=162, szbeg=5, gzbeg=0)),
    # Interior 101^3 + 20-cell sponge (padded 142^3), 20 Hz at (50,50,10), 1000 steps,
    # receivers at z = 5.
    "ose142": (lambda: layered_perturbed(101, 101, 101),
               dict(nx=101, ny=101, nz=101, bu=20, bd=20, bl=20, br=20, bf=20, bb=20, nt=1000,
                    fm=20.0, dt=0.002, amp=100.0, dx=10.0, dy=10.0, dz=10.0,
                    sxbeg=50, sybeg=50, szbeg=10, gzbeg=5)),
    # the same with the Cerjan sponge, factor 0.015
    "ose142cerjan": (lambda: layered_perturbed(101, 101, 101),
                     dict(nx=101, ny=101, nz=101, bu=20, bd=20, bl=20, br=20, bf=20, bb=20, nt=1000,
                          fm=20.0, dt=0.002, amp=100.0, dx=10.0, dy=10.0, dz=10.0,
                          sxbeg=50, sybeg=50, szbeg=10, gzbeg=5, sponge_mode=1, cerjan_factor=0.015)),
}


def batched_windows(nshots: int = 64, seed: int = 64, model_shape=(512, 512, 192), sponge: int = 16,
                    depth: int = 5):
    """Shot windows of the batched workload: sources on a seeded grid of
    sqrt(nshots) x sqrt(nshots) surface positions, each shot on a window centred
    on its source whose PADDED size (interior + 2 * sponge) is drawn from
    96..192 (x, y) and 128..192 (z) in steps of 16."""
    rng = np.random.default_rng(seed)
    mx, my, mz = model_shape
    g = int(round(nshots ** 0.5))
    wins = []
    for s in range(nshots):
        i, j = s % g, s // g
        sx = int((i + 0.5) * mx / g + rng.integers(-8, 9))
        sy = int((j + 0.5) * my / g + rng.integers(-8, 9))
        nxp = int(rng.choice(np.arange(96, 193, 16)))
        nyp = int(rng.choice(np.arange(96, 193, 16)))
        nzp = int(rng.choice(np.arange(128, 193, 16)))
        nx, ny, nz = nxp - 2 * sponge, nyp - 2 * sponge, nzp - 2 * sponge
        x0, y0 = sx - nx // 2, sy - ny // 2
        wins.append(dict(x0=x0, y0=y0, z0=0, nx=nx, ny=ny, nz=nz, sx=sx - x0, sy=sy - y0, sz=depth))
    return wins


# 64 shots on a 512 x 512 x 192 model, windows 96..192 cells, dt 2 ms, 1200 steps
BATCHED = dict(model=lambda: smooth_random_salt(512, 512, 192, seed=77),
               params=dict(bu=16, bd=16, bl=16, br=16, bf=16, bb=16, nt=1200, fm=20.0, dt=0.002,
                           amp=100.0, dx=10.0, dy=10.0, dz=10.0, gzbeg=0),
               windows=lambda: batched_windows())
