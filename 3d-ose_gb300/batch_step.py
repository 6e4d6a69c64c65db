"""Run or time the batched form on the first K shots of the 64-shot workload
(padded windows 96..192 cells on the seeded 512 x 512 x 192 model) under
explicit tunings, e.g. to capture one step's launches under a profiler.

    python 3d-ose_gb300/batch_step.py run K GROUP_MB LANES [STEPS]
    python 3d-ose_gb300/batch_step.py time K

run: reset, then STEPS (default 2) steps with the given shot-group size (MB of
fields per L2-sized group, 0 = one group) and number of concurrent per-shot
lanes (0 = batched launches, -1 = one persistent launch per step).  time:
the step time of a few fixed tunings.
"""
from __future__ import annotations

import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import ose3d  # noqa: E402
import workloads  # noqa: E402


def main(argv):
    mode, k = argv[1], int(argv[2])
    cfg = workloads.BATCHED
    model = cfg["model"]()
    wins = cfg["windows"]()[:k]
    p = ose3d.default_params(**cfg["params"])
    with ose3d.Batch(p, model, wins) as b:
        cells = sum(b.info(s)[1] for s in range(b.nshots))
        if mode == "run":
            b.set_tuning(group_mb=int(argv[3]), lanes=int(argv[4]))
            b.reset()
            b.run(int(argv[5]) if len(argv) > 5 else 2)
            return 0
        out = {}
        for g, lanes in ((0, 0), (48, 0), (96, 0), (0, 2), (0, 4), (0, -1), (48, -1), (96, -1)):
            b.set_tuning(group_mb=g, lanes=lanes)
            b.reset()
            b.run(3)
            out[f"group{g}_lanes{lanes}"] = round(b.run_timed(10) / 10, 3)
        print(json.dumps({"shots": k, "cells": cells, "ms_per_step": out,
                          "gcell_steps_s": {n: round(cells / (v * 1e-3) / 1e9, 3) for n, v in out.items()}}))
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
