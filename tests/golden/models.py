"""Seeded velocity models of the golden cases, in the reference model layout
[x][y][z] (z fastest), float32 (input_file_xyz_boundary, ose_3d_lib.cu:887-909)."""
from __future__ import annotations

import numpy as np


def two_layer_model(nx, ny, nz, v_top, v_bottom, z_interface):
    """v = v_top above interior depth z_interface, v_bottom from it down.  With
    (101,101,101,3000,4000,30) this reproduces the reference's own
    input/v3d_nx101_ny101_nz101.bin bit for bit (checked when the goldens are made)."""
    v = np.empty((nx, ny, nz), np.float32)
    v[:, :, :z_interface] = v_top
    v[:, :, z_interface:] = v_bottom
    return v


def layered_noise_model(nx, ny, nz, seed):
    """Three layers (2000/2800/3500 m/s at depth thirds) times (1 + 3% white noise)."""
    rng = np.random.default_rng(seed)
    z = np.arange(nz)
    base = np.where(z < nz * 3 // 8, 2000.0, np.where(z < nz * 11 // 16, 2800.0, 3500.0))
    v = np.broadcast_to(base[None, None, :], (nx, ny, nz)).astype(np.float32)
    v = v * (1.0 + 0.03 * rng.standard_normal((nx, ny, nz))).astype(np.float32)
    return np.ascontiguousarray(v, dtype=np.float32)


def layered_perturbed_model(nx, ny, nz, seed):
    """The config-1 generator of the benchmark workloads (four layers
    1500/2200/3000/3800 m/s times 1 + a smoothed 5% perturbation)."""
    import os
    import sys
    pkg = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "..", "3d-ose_gb300")
    if pkg not in sys.path:
        sys.path.insert(0, pkg)
    import workloads
    return workloads.layered_perturbed(nx, ny, nz, seed)
