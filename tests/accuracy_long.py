"""Long-run accuracy of the FP32 GPU path against the FP64 restatement
(oracle/oracle_torch.py, run with torch on the same GPU) on a bench workload.

    python tests/accuracy_long.py [--workload ose256] [--steps 2000] [--every 250]
                                  [--precision fp32,tf32,tf32x3,bf16x3]

Prints one JSON line per checkpoint: step, rel-L2 of the gather so far and of
the current P and Q, plus the first dropped series coefficient |J_{M+2}(dtR)|.
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


def rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="ose256")
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--every", type=int, default=250)
    ap.add_argument("--path", default="default",
                    choices=["default", "generic", "torch32", "fp64c32"])
    ap.add_argument("--precision", default="fp32",
                    help="comma list of fp32, tf32, tf32x3, bf16x3 (one FP64 run serves all)")
    a = ap.parse_args()
    import __graft_entry__ as ge
    ge.build_library()
    import ose3d
    import workloads
    from oracle_torch import TorchOracle

    build, kw = workloads.CONFIGS[a.workload]
    vel = build()
    steps = min(a.steps, kw["nt"])
    # torch32: the same loop in complex64 with cuFFT, the arithmetic class of
    # the reference's FP32 cuFFT path, in place of libose3d
    # fp64c32: FP64 arithmetic with the per-step constants rounded to float32
    precs = a.precision.split(",")
    ms = {}
    if a.path not in ("torch32", "fp64c32"):
        for pr in precs:
            m = ose3d.Modeler(ose3d.default_params(**kw), vel)
            if a.path == "generic":
                m.select_path(ose3d.PATH_GENERIC)
            m.precision = pr
            m.reset_shot(0)
            ms[pr] = m
    t32 = None
    if a.path == "torch32":
        t32 = TorchOracle(kw, vel, "cuda", single=True)
    elif a.path == "fp64c32":
        t32 = TorchOracle(kw, vel, "cuda", fp32_constants=True)
    t = TorchOracle(kw, vel, "cuda")
    rows32 = {k: [] for k in (ms or {a.path: None})}
    rows64 = []
    done = 0
    t0 = time.time()
    while done < steps:
        n = min(a.every, steps - done)
        for k in rows32:
            rows32[k].append(ms[k].run_record(n) if ms else t32.run(n))
        rows64.append(t.run(n))
        done += n
        g64 = np.concatenate(rows64)
        P64, Q64 = t.P(), t.Q()
        for k in rows32:
            m = ms.get(k)
            g32 = np.concatenate(rows32[k])
            P32 = m.wavefield(ose3d.FIELD_P) if m is not None else t32.P()
            Q32 = m.wavefield(ose3d.FIELD_Q) if m is not None else t32.Q()
            name = a.path if m is None else ("plane" if m.derived.path == 1 else "generic")
            out = {"workload": a.workload, "path": name, "precision": k if m is not None else None,
                   "step": done, "gather_rel_l2": rel(g32, g64), "P_rel_l2": rel(P32, P64),
                   "Q_rel_l2": rel(Q32, Q64), "Q_norm": float(np.linalg.norm(Q64)),
                   "P_norm": float(np.linalg.norm(P64)), "M": t.M,
                   "elapsed_s": round(time.time() - t0, 1)}
            print(json.dumps(out), flush=True)
    for m in ms.values():
        m.close()


if __name__ == "__main__":
    main()
