"""Which FP32 stage accumulates the late-time error of the OSE loop?

The FP64 restatement of the loop (oracle/oracle_torch.py, torch complex128 on
one GPU) is run with FP32 rounding injected at one stage at a time, all
variants in lockstep with the plain FP64 run (and optionally this library's
FP32 path); one JSON line per checkpoint gives, per variant, the rel-L2 of
[gather so far, Q, P] against FP64.

    python tests/accuracy_stages.py [--workload ose256] [--steps 2000] [--every 250]
        [--stages fft,store,W,S,a,consts,fftroll,fftphase,fftrot4,storesr] [--gpu-path]

Stages: fft = every FFT in complex64 (|k| in float); store = the terms a_n,
S and the state rounded to float after every write (W, S, a: one of them);
consts = the per-step constants rounded to float; fftroll / fftphase /
fftrot4 = complex64 FFTs of a randomly shifted grid / of the field times a
random phase / times i^k, to decorrelate round-off between applications;
storesr = stochastic rounding of the stored fields.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
for sub in ("", "oracle", "3d-ose_gb300"):
    sys.path.insert(0, os.path.join(ROOT, sub))


def main():
    import torch
    from oracle_torch import TorchOracle

    def rd(x):
        return x.to(torch.complex64).to(torch.complex128)

    def sr64(r):
        f = r.to(torch.float32)
        d = r - f.to(torch.float64)
        inf = torch.full_like(f, float("inf"))
        nxt = torch.nextafter(f, torch.where(d >= 0, inf, -inf))
        gap = (nxt.to(torch.float64) - f.to(torch.float64)).abs()
        p = torch.where(gap > 0, d.abs() / gap, torch.zeros_like(d))
        return torch.where(torch.rand_like(p) < p, nxt, f).to(torch.float64)

    def rds(x):
        return torch.complex(sr64(x.real), sr64(x.imag))

    class Variant(TorchOracle):
        def __init__(self, kw, vel, stage, **k):
            super().__init__(kw, vel, "cuda", **k)
            self.stage = stage
            self.k32 = self.kabs.to(torch.float32)
            self.q = 0

        def L(self, x):
            f, st = torch.fft, self.stage
            if st == "fft":
                return self.vr * f.ifftn(self.k32 * f.fftn(x.to(torch.complex64))).to(torch.complex128)
            if st == "fftroll":
                sh = tuple(int(v) for v in torch.randint(0, min(self.shape), (3,)))
                y = f.ifftn(self.k32 * f.fftn(torch.roll(x, sh, (0, 1, 2)).to(torch.complex64)))
                return self.vr * torch.roll(y, tuple(-v for v in sh), (0, 1, 2)).to(torch.complex128)
            if st in ("fftphase", "fftrot4"):
                if st == "fftphase":
                    th = float(torch.rand(1)) * 2.0 * np.pi
                    ph = complex(np.cos(th), np.sin(th))
                else:
                    self.q = (self.q + 1) % 4
                    ph = [1, 1j, -1, -1j][self.q]
                y = f.ifftn(self.k32 * f.fftn((x * ph).to(torch.complex64)))
                return self.vr * (y.to(torch.complex128) * ph.conjugate())
            return self.vr * f.ifftn(self.kabs * f.fftn(x))

        def rnd(self, x, what):
            st = self.stage
            if st == "storesr":
                return rds(x)
            if st == what or st == "store":
                return rd(x)
            return x

        def step(self):
            r2 = self.r2
            z, y, x = self.src
            self.W[z, y, x] += complex(self.ricker[self.it], self.hil[self.it])
            self.W = self.rnd(self.W, "W")
            a0 = self.W
            a1 = self.rnd(-1j * self.L(a0), "a")
            S = self.rnd(self.J[0] * a0 + r2(self.J[1]) * a1, "S")
            am, an = a0, a1
            for n in range(1, self.M + 1):
                ap = self.rnd(am - 2j * self.L(an), "a")
                S = self.rnd(S + r2(self.J[n + 1]) * ap, "S")
                S = self.rnd(S * self.att, "S")
                am, an = an, ap
            self.W = S
            self.it += 1
            p = self.p
            return S.imag[self.gz, p.bf:p.bf + p.ny, p.bl:p.bl + p.nx].reshape(-1)

    def rel(a, b):
        a = np.asarray(a, np.float64)
        b = np.asarray(b, np.float64)
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="ose256")
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--every", type=int, default=250)
    ap.add_argument("--stages", default="fft,store,W,S,a,consts")
    ap.add_argument("--gpu-path", action="store_true", help="also this library's FP32 path")
    a = ap.parse_args()
    import workloads
    build, kw = workloads.CONFIGS[a.workload]
    vel = build()
    base = TorchOracle(kw, vel, "cuda")
    vs = {s: (Variant(kw, vel, "none", fp32_constants=True) if s == "consts" else Variant(kw, vel, s))
          for s in a.stages.split(",") if s}
    m = None
    if a.gpu_path:
        import __graft_entry__ as ge
        ge.build_library()
        import ose3d
        m = ose3d.Modeler(ose3d.default_params(**kw), vel)
        m.reset_shot(0)
    rows = {k: [] for k in ["base"] + list(vs) + (["gpu"] if m else [])}
    done, t0 = 0, time.time()
    while done < min(a.steps, kw["nt"]):
        n = min(a.every, a.steps - done)
        rows["base"].append(base.run(n))
        for k, v in vs.items():
            rows[k].append(v.run(n))
        if m:
            rows["gpu"].append(m.run_record(n))
        done += n
        g64, Q64, P64 = np.concatenate(rows["base"]), base.Q(), base.P()
        out = {"step": done, "Q_norm": float(np.linalg.norm(Q64)), "elapsed_s": round(time.time() - t0, 1)}
        for k in rows:
            if k == "base":
                continue
            Q = m.wavefield(ose3d.FIELD_Q) if k == "gpu" else vs[k].Q()
            P = m.wavefield(ose3d.FIELD_P) if k == "gpu" else vs[k].P()
            out[k] = [rel(np.concatenate(rows[k]), g64), rel(Q, Q64), rel(P, P64)]
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
