"""FP64 restatement of the OSE time loop executed with torch (CPU or GPU), for
accuracy checks over long runs at full size, where the C oracle
(ose_oracle.c) would take hours.

TEST INFRASTRUCTURE: imported only by tests/.  It follows the same reference
lines as ose_oracle.c (ose_3d_lib.cu:639-874 for the step, ose_3d.cu:252-274 for
the loop) and takes its set-up values (padded model, sponge, wavelets, Bessel
coefficients, series order) from the C oracle, so the two differ only in the
FFT and the arithmetic order; tests/test_oracle_torch.py checks them against
each other.
"""
from __future__ import annotations

import numpy as np

import oracle as O


class TorchOracle:
    def __init__(self, params: dict, vel_xyz: np.ndarray, device: str = "cpu", shot: int = 0,
                 single: bool = False, fp32_constants: bool = False):
        """single=True runs the same loop in complex64 / float32 (the
        arithmetic class of the reference's cuFFT FP32 path), for comparison.
        fp32_constants=True keeps FP64 arithmetic but rounds the per-step
        constants (Bessel coefficients, v/R, |k|, sponge) to float32 first, to
        separate their systematic error from round-off in the arithmetic."""
        import torch

        self.torch = torch
        self.rdt = torch.float32 if single else torch.float64
        self.cdt = torch.complex64 if single else torch.complex128
        self.dev = torch.device(device)
        p = O.make_params(**params)
        d = O.derive(p)
        self.p, self.d = p, d
        self.shape = (d.nzb, d.nyb, d.nxb)
        vb = O.pad_model(p, vel_xyz)
        self.R, self.dtR, self.M = O.series(p, float(vb.max()))
        self.J = O.bessel(self.M, self.dtR)
        r32 = (lambda a: np.asarray(a, np.float32).astype(np.float64)) if fp32_constants else (lambda a: a)
        self.J = r32(self.J)
        ax = O.sponge(p.bl, p.nx, d.br, p.sponge_mode, p.cerjan_factor).astype(np.float64)
        ay = O.sponge(p.bf, p.ny, d.bb, p.sponge_mode, p.cerjan_factor).astype(np.float64)
        az = O.sponge(p.bu, p.nz, d.bd, p.sponge_mode, p.cerjan_factor).astype(np.float64)
        self.ricker = O.ricker(p.nt, p.fm, p.dt, p.amp).astype(np.float64)
        self.hil = O.hilbert(self.ricker.astype(np.float32), bool(p.hilbert_div_nt)).astype(np.float64)
        t = lambda a: torch.as_tensor(a, dtype=self.rdt, device=self.dev)  # noqa: E731
        self.att = t(r32(az[:, None, None] * ay[None, :, None] * ax[None, None, :]))
        # v / R; torch's inverse FFT already divides by N (ose_3d_kernel.cu:355-357)
        self.vr = t(r32(vb.astype(np.float64) / self.R))

        def kw(n, dk):
            i = np.arange(n)
            return dk * np.where(i > n // 2, n - i, i)

        kx, ky, kz = kw(d.nxb, d.dkx), kw(d.nyb, d.dky), kw(d.nzb, d.dkz)
        self.kabs = t(r32(np.sqrt(kz[:, None, None] ** 2 + ky[None, :, None] ** 2 + kx[None, None, :] ** 2)))
        nx, ny = p.nx, p.ny
        sx0, sy0, sz0 = p.sxbeg + shot * p.jsx, p.sybeg + shot * p.jsy, p.szbeg + shot * p.jsz
        sxyz = sz0 * nx * ny + sy0 * nx + sx0
        self.src = (p.bu + sxyz // (nx * ny), p.bf + sxyz % (nx * ny) // nx, p.bl + sxyz % (nx * ny) % nx)
        self.gz = p.bu + p.gzbeg
        self.W = torch.zeros(self.shape, dtype=self.cdt, device=self.dev)
        # 2 J_{n+1}, rounded like the kernels' coefficients when asked
        self.r2 = (lambda c: float(np.float32(2.0 * c))) if fp32_constants else (lambda c: 2.0 * c)
        self.it = 0

    def L(self, x):
        f = self.torch.fft
        return self.vr * f.ifftn(self.kabs * f.fftn(x))

    def step(self):
        """inject + one OSE step + record (ose_3d.cu:252-274)."""
        r2 = self.r2
        z, y, x = self.src
        self.W[z, y, x] += complex(self.ricker[self.it], self.hil[self.it])
        a0 = self.W
        a1 = -1j * self.L(a0)
        S = self.J[0] * a0 + r2(self.J[1]) * a1
        am, an = a0, a1
        for n in range(1, self.M + 1):
            ap = am - 2j * self.L(an)
            S = (S + r2(self.J[n + 1]) * ap) * self.att
            am, an = an, ap
        self.W = S
        self.it += 1
        p = self.p
        return S.imag[self.gz, p.bf:p.bf + p.ny, p.bl:p.bl + p.nx].reshape(-1)

    def run(self, nsteps: int):
        """Gather rows [it][ig] of the next nsteps steps (float64 numpy)."""
        rows = [self.step() for _ in range(nsteps)]
        return self.torch.stack(rows).cpu().numpy().astype(np.float64)

    def P(self):
        return self.W.real.cpu().numpy().astype(np.float64)

    def Q(self):
        return self.W.imag.cpu().numpy().astype(np.float64)
