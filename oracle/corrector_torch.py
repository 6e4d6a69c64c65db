"""FP64 restatement of the learned boundary corrector (3d-ose_gb300/csrc/
ose_learn.cu) with torch autograd on the CPU: the gradient check of the
network's hand-written CUDA training kernels.

TEST INFRASTRUCTURE: imported only by tests/.  The corrector has no
counterpart in the reference (whose only boundary treatment is the sponge,
ose_3d_kernel.cu:242-288), so this file restates the network as the library
defines it:

  features  P/s, Q/s, v/4500, ex, ey, ez, 0, 0
            s = s(x) = sqrt(m/2 + f^2): m the mean of P^2 + Q^2 (shell cells,
            zero elsewhere) over the periodic 17^3 box around the cell, f =
            1e-3 x the RMS of P, Q over the shell
  conv 3x3x3 8->32 ReLU, 32->32 ReLU, 32->32 ReLU, 32->2
  periodic grid; every layer's input is zero outside the shell
  loss = mean over write cells of |out - (target - state)/s(x)|^2
"""
from __future__ import annotations

import numpy as np

CIN = (8, 32, 32, 32)
COUT = (32, 32, 32, 2)


def param_count() -> int:
    return sum(27 * ci * co + co for ci, co in zip(CIN, COUT))


def masks(shape_zyx, shell: int, sponge6):
    """(shell mask, write mask) as bool arrays [z][y][x]; sponge6 = widths
    x-, x+, y-, y+, z-, z+."""
    nz, ny, nx = shape_zyx
    z, y, x = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    d = np.minimum.reduce([x, nx - 1 - x, y, ny - 1 - y, z, nz - 1 - z])
    sh = d < shell
    s = sponge6
    wr = sh & (x >= s[0]) & (x < nx - s[1]) & (y >= s[2]) & (y < ny - s[3]) & (z >= s[4]) & (z < nz - s[5])
    return sh, wr


def face_coord(n: int, shell: int) -> np.ndarray:
    v = np.arange(n)
    lo, hi = v, n - 1 - v
    out = np.zeros(n)
    a = (lo < shell) & (lo <= hi)
    out[a] = -(shell - lo[a]) / shell
    b = ~a & (hi < shell)
    out[b] = (shell - hi[b]) / shell
    return out


def scales(P, Q, shell, sponge6):
    """(global shell RMS, local scale s(x) [z][y][x])."""
    from scipy.ndimage import uniform_filter
    sh, _ = masks(P.shape, shell, sponge6)
    e = (P ** 2 + Q ** 2) * sh
    sg = np.sqrt(e.sum() / (2.0 * sh.sum()))
    m = uniform_filter(e, size=17, mode="wrap")
    return sg, np.sqrt(0.5 * m + (1e-3 * sg) ** 2)


def features(P, Q, vel, shell, sponge6):
    """[8][z][y][x] features, the global shell RMS and the local scale."""
    nz, ny, nx = P.shape
    sh, _ = masks(P.shape, shell, sponge6)
    s, sl = scales(P, Q, shell, sponge6)
    inv = 1.0 / sl
    F = np.zeros((8, nz, ny, nx))
    F[0], F[1], F[2] = P * inv, Q * inv, vel / 4500.0
    F[3] = face_coord(nx, shell)[None, None, :]
    F[4] = face_coord(ny, shell)[None, :, None]
    F[5] = face_coord(nz, shell)[:, None, None]
    return F * sh[None], s, sl


def unpack(params, torch):
    """Per layer (weight [Cout][Cin][3][3][3] as torch conv3d wants, bias)."""
    out, o = [], 0
    for ci, co in zip(CIN, COUT):
        w = params[o:o + 27 * ci * co].reshape(3, 3, 3, ci, co)   # [dz][dy][dx][ci][co]
        o += 27 * ci * co
        b = params[o:o + co]
        o += co
        out.append((w.permute(4, 3, 0, 1, 2).contiguous(), b))
    return out


def forward(params, F, shell_mask):
    """params: torch float64 vector (may require grad); F: [8][z][y][x] tensor."""
    import torch
    import torch.nn.functional as tf
    m = torch.as_tensor(shell_mask, dtype=F.dtype)[None, None]
    h = F[None] * m
    layers = unpack(params, torch)
    for i, (w, b) in enumerate(layers):
        h = tf.conv3d(tf.pad(h * m, (1, 1, 1, 1, 1, 1), mode="circular"), w, b)
        if i < 3:
            h = torch.relu(h)
    return h[0] * m[0]


def loss_and_grads(params_np, P, Q, vel, target_P, target_Q, shell, sponge6):
    """(loss, d loss / d params as float64 numpy, output [2][z][y][x], global
    shell RMS, local scale s(x))."""
    import torch
    F, s, sl = features(P, Q, vel, shell, sponge6)
    sh, wr = masks(P.shape, shell, sponge6)
    p = torch.tensor(np.asarray(params_np, np.float64), requires_grad=True)
    out = forward(p, torch.as_tensor(F), sh)
    inv = 1.0 / sl
    r = torch.as_tensor(np.stack([(target_P - P) * inv, (target_Q - Q) * inv]))
    w = torch.as_tensor(wr.astype(np.float64))[None]
    loss = (((out - r) ** 2) * w).sum() / wr.sum()
    loss.backward()
    return float(loss.detach()), p.grad.numpy().copy(), out.detach().numpy(), s, sl


def init_params(seed: int = 0, scale: float = 1.0) -> np.ndarray:
    """He-style random initialisation (the training script's starting point)."""
    rng = np.random.default_rng(seed)
    out = []
    for i, (ci, co) in enumerate(zip(CIN, COUT)):
        fan = 27 * (6 if i == 0 else ci)
        std = scale * np.sqrt(2.0 / fan) * (0.1 if i == 3 else 1.0)
        out.append(rng.standard_normal(27 * ci * co) * std)
        out.append(np.zeros(co))
    return np.concatenate(out).astype(np.float32)
