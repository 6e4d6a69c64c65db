"""Training and evaluation of the learned boundary corrector (ose_learn.cu).

The corrector lets a grid carry a thin sponge (8 cells) and still behave like
one with a wide sponge (64 cells).  Training pairs come from the solver itself:
for each seeded velocity model and Ricker source, a THIN run (interior + 8-cell
sponge) and a WIDE run (same interior + 64-cell sponge) advance in lockstep.
After every step the thin run's state u is paired with the wide run's state
restricted to the thin grid (the target); then the thin run's interior is
reset to the wide run's, so the next pair starts from the true interior with
the thin run's own sponge content.  The network learns the one-step residual
(target - u) / s(x) on the write cells (the 8 interior cells next to the
sponge); s(x) is the local RMS of the state (17^3 box), so inputs and targets
have the same range on any grid size.

    python 3d-ose_gb300/learn_boundary.py train --runs 200 --out corrector.npy
    python 3d-ose_gb300/learn_boundary.py eval --weights corrector.npy

All compute runs in libose3d (solver, network forward, gradients, Adam); torch
only holds the device buffers of the training set.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if HERE not in sys.path:
    sys.path.insert(0, HERE)

import ose3d  # noqa: E402

THIN = 8          # thin sponge, cells
WIDE = 64         # wide sponge, cells
SHELL = ose3d.CORRECTOR_SHELL
WEIGHTS = os.path.join(HERE, "weights", "corrector.npy")

CIN = (8, 32, 32, 32)
COUT = (32, 32, 32, 2)


def init_params(seed: int = 0) -> np.ndarray:
    """He initialisation; the output layer starts 10x smaller."""
    rng = np.random.default_rng(seed)
    out = []
    for i, (ci, co) in enumerate(zip(CIN, COUT)):
        fan = 27 * (6 if i == 0 else ci)
        std = np.sqrt(2.0 / fan) * (0.1 if i == 3 else 1.0)
        out.append(rng.standard_normal(27 * ci * co) * std)
        out.append(np.zeros(co))
    p = np.concatenate(out).astype(np.float32)
    assert p.size == ose3d.corrector_param_count()
    return p


def random_model(rng, n: int) -> np.ndarray:
    """Seeded smooth random model 1500-4500 m/s ([x][y][z]): a Gaussian-smoothed
    field (sigma 2-8 cells) plus a random depth trend, sometimes with a
    4500 m/s ellipsoid."""
    from scipy.ndimage import gaussian_filter
    f = gaussian_filter(rng.standard_normal((n, n, n)), sigma=rng.uniform(2.0, 8.0), mode="wrap")
    f = (f - f.min()) / max(f.max() - f.min(), 1e-12)
    trend = rng.uniform(0.0, 0.7)
    depth = np.linspace(0.0, 1.0, n)[None, None, :]
    v = 1500.0 + 3000.0 * np.clip(trend * depth + (1.0 - trend) * f, 0.0, 1.0)
    if rng.random() < 0.5:
        c = rng.uniform(0.3, 0.7, 3) * n
        r = rng.uniform(0.1, 0.25, 3) * n
        x, y, z = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
        v[((x - c[0]) / r[0]) ** 2 + ((y - c[1]) / r[1]) ** 2 + ((z - c[2]) / r[2]) ** 2 <= 1.0] = 4500.0
    return np.ascontiguousarray(v, np.float32)


def pair_params(n: int, fm: float, src, nt: int, sponge: int) -> dict:
    return dict(nx=n, ny=n, nz=n, bu=sponge, bd=sponge, bl=sponge, br=sponge, bf=sponge, bb=sponge, nt=nt,
                fm=fm, dt=0.002, amp=100.0, dx=10.0, dy=10.0, dz=10.0, sxbeg=src[0], sybeg=src[1],
                szbeg=src[2], gzbeg=0)


def draw_case(rng, n: int):
    vel = random_model(rng, n)
    fm = float(rng.uniform(10.0, 30.0))
    src = (int(rng.integers(n // 4, 3 * n // 4)), int(rng.integers(n // 4, 3 * n // 4)),
           int(rng.integers(2, n // 2)))
    return vel, fm, src


class Pair:
    """A thin and a wide modeler on the same interior model and source."""

    def __init__(self, vel, fm, src, nt):
        n = vel.shape[0]
        self.n = n
        self.thin = ose3d.Modeler(ose3d.default_params(**pair_params(n, fm, src, nt, THIN)), vel)
        self.wide = ose3d.Modeler(ose3d.default_params(**pair_params(n, fm, src, nt, WIDE)), vel)
        self.nb = n + 2 * THIN
        off = WIDE - THIN
        self.wide_box = (off, off, off, self.nb, self.nb, self.nb)
        self.full = (0, 0, 0, self.nb, self.nb, self.nb)
        self.buf = (self.nb, self.nb, 0, 0, 0)
        self.interior = (THIN, THIN, THIN, n, n, n)
        self.interior_buf = (self.nb, self.nb, THIN, THIN, THIN)

    def reset(self):
        self.thin.reset_shot(0)
        self.wide.reset_shot(0)

    def close(self):
        self.thin.close()
        self.wide.close()


def generate(runs: int, seed: int, n: int = 48, steps: int = 150, t0: int = 20, every: int = 5,
             log=print):
    """Training set on the device: X (thin state after a step), Y (wide state
    restricted), V (padded velocity per run), run index per sample."""
    import torch
    rng = np.random.default_rng(seed)
    nb = n + 2 * THIN
    per_run = len(range(t0, steps, every))
    S = runs * per_run
    X = torch.zeros((S, nb, nb, nb, 2), dtype=torch.float32, device="cuda")
    Y = torch.zeros_like(X)
    V = torch.zeros((runs, nb, nb, nb), dtype=torch.float32, device="cuda")
    run_of = np.zeros(S, np.int64)
    tgt = torch.zeros((nb, nb, nb, 2), dtype=torch.float32, device="cuda")
    i = 0
    t_start = time.time()
    for r in range(runs):
        vel, fm, src = draw_case(rng, n)
        pr = Pair(vel, fm, src, steps + 1)
        V[r] = torch.as_tensor(pr.thin.wavefield(ose3d.FIELD_V), device="cuda")
        pr.reset()
        for t in range(steps):
            pr.wide.run(1)
            pr.thin.run(1)
            pr.wide.state_box(0, pr.wide_box, tgt.data_ptr(), pr.buf)
            if t >= t0 and (t - t0) % every == 0:
                pr.thin.state_box(0, pr.full, X[i].data_ptr(), pr.buf)
                Y[i].copy_(tgt)
                run_of[i] = r
                i += 1
            pr.thin.state_box(1, pr.interior, tgt.data_ptr(), pr.interior_buf)
        pr.close()
        if log and (r + 1) % 20 == 0:
            log(f"generate: {r + 1}/{runs} runs, {i} samples, {time.time() - t_start:.0f} s")
    torch.cuda.synchronize()
    return dict(X=X[:i], Y=Y[:i], V=V, run=run_of[:i], n=n)


def train(data, epochs: int = 4, batch: int = 16, lr: float = 1e-3, seed: int = 0, log=print, init=None):
    """Adam with cosine decay over `epochs` passes of the samples, from the
    seeded initialisation or from `init` (parameters to continue from)."""
    import torch
    X, Y, V, run = data["X"], data["Y"], data["V"], data["run"]
    S = X.shape[0]
    nb = X.shape[1]
    rng = np.random.default_rng(seed)
    hist = []
    with ose3d.Corrector((nb, nb, nb), (THIN,) * 6, shell=SHELL) as c:
        c.set_params(init_params(seed) if init is None else np.asarray(init, np.float32))
        steps = epochs * (S // batch)
        k = 0
        t_start = time.time()
        for ep in range(epochs):
            order = rng.permutation(S)
            ep_loss = []
            for b0 in range(0, S - batch + 1, batch):
                for j in order[b0:b0 + batch]:
                    c.train_sample(X[j].data_ptr(), V[run[j]].data_ptr(), Y[j].data_ptr())
                # cosine decay to lr / 20
                a = lr * (0.05 + 0.95 * 0.5 * (1.0 + np.cos(np.pi * k / max(1, steps))))
                ep_loss.append(c.adam(float(a), batch))
                k += 1
            hist.append(float(np.mean(ep_loss)))
            if log:
                log(f"train: epoch {ep + 1}/{epochs} loss {hist[-1]:.4e} ({time.time() - t_start:.0f} s)")
        torch.cuda.synchronize()
        return c.params(), hist


def evaluate(params, seed: int, cases: int = 4, n: int = 48, steps: int = 300, every: int = 5):
    """Thin run without and with the corrector against the wide run, per case:
    interior error energy sum_t |W_thin - W_wide|^2 / sum_t |W_wide|^2 over the
    interior (sampled every `every` steps) and the receiver gather rel-L2."""
    import torch
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(cases):
        vel, fm, src = draw_case(rng, n)
        res = {"fm": fm, "src": src}
        ref_rows = None
        wide_int = []
        for mode in ("wide", "plain", "learned"):
            sp = WIDE if mode == "wide" else THIN
            m = ose3d.Modeler(ose3d.default_params(**pair_params(n, fm, src, steps + 1, sp)), vel)
            if mode == "learned":
                m.set_corrector(params, SHELL)
            m.reset_shot(0)
            buf = torch.zeros((n, n, n, 2), dtype=torch.float32, device="cuda")
            err = ref = 0.0
            rows = []
            for t in range(0, steps, every):
                rows.append(m.run_record(every))
                m.state_box(0, (sp, sp, sp, n, n, n), buf.data_ptr(), (n, n, 0, 0, 0))
                if mode == "wide":
                    wide_int.append(buf.clone())
                else:
                    w = wide_int[t // every]
                    err += float(((buf - w) ** 2).sum())
                    ref += float((w ** 2).sum())
            g = np.concatenate(rows)
            if mode == "wide":
                ref_rows = g
            else:
                res[mode] = {"interior_error_energy": err / max(ref, 1e-300),
                             "gather_rel_l2": float(np.linalg.norm(g - ref_rows) / np.linalg.norm(ref_rows))}
            m.close()
        res["gain"] = res["plain"]["interior_error_energy"] / max(res["learned"]["interior_error_energy"], 1e-300)
        out.append(res)
    return out


def main():
    ap = argparse.ArgumentParser()
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--runs", type=int, default=200)
    t.add_argument("--n", type=int, default=48)
    t.add_argument("--steps", type=int, default=150)
    t.add_argument("--every", type=int, default=5)
    t.add_argument("--t0", type=int, default=20, help="first step sampled")
    t.add_argument("--epochs", type=int, default=4)
    t.add_argument("--batch", type=int, default=16)
    t.add_argument("--lr", type=float, default=1e-3)
    t.add_argument("--seed", type=int, default=1234)
    t.add_argument("--out", default=WEIGHTS)
    t.add_argument("--init", default=None, help="continue from these parameters (.npy)")
    e = sub.add_parser("eval")
    e.add_argument("--weights", default=WEIGHTS)
    e.add_argument("--cases", type=int, default=4)
    e.add_argument("--n", type=int, default=48)
    e.add_argument("--steps", type=int, default=300)
    e.add_argument("--seed", type=int, default=99)
    a = ap.parse_args()
    if a.cmd == "train":
        t0 = time.time()
        data = generate(a.runs, a.seed, n=a.n, steps=a.steps, t0=a.t0, every=a.every)
        t_gen = time.time() - t0
        params, hist = train(data, epochs=a.epochs, batch=a.batch, lr=a.lr, seed=a.seed,
                             init=np.load(a.init) if a.init else None)
        os.makedirs(os.path.dirname(os.path.abspath(a.out)), exist_ok=True)
        np.save(a.out, params)
        print(json.dumps({"samples": int(data["X"].shape[0]), "runs": a.runs, "generate_s": round(t_gen, 1),
                          "train_s": round(time.time() - t0 - t_gen, 1), "loss": hist, "out": a.out}))
    else:
        params = np.load(a.weights)
        for r in evaluate(params, a.seed, cases=a.cases, n=a.n, steps=a.steps):
            print(json.dumps(r))


if __name__ == "__main__":
    main()
