#!/usr/bin/env python3
"""Benchmark of the plain FP32 OSE time step on GB300 (one JSON line on rank 0).

A step is one OSE time step (source injection, M+1 operator applications with
the fused series update, receiver row) of the padded 256^3 workload
(interior 196^3 + 30-cell sponge, seeded smooth random 1500-4500 m/s model with
a 4500 m/s salt ellipsoid, 25 Hz Ricker, dt = 2 ms).  Inputs stay resident in
HBM; every field (134 MB) is larger than L2, so no L2 flush is needed.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of the same step (the oracle, FP64,
all host threads) on a bounded sample; the reference program itself has no
CPU path and its multi-GPU cuFFT-Xt path needs two GPUs.
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "3d-ose_gb300")
for p in (PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

METRIC = "Gcell-steps/s at 256³ vs plain OSE at ≤1e-4 rel-L2 vs FP64; % HBM roofline"
UNIT = "Gcell-steps/s"
WORKLOAD = "ose256"
WORKLOAD_TEXT = ("plain OSE FP32 time step, padded 256x256x256 (interior 196^3 + 30-cell sponge), "
                 "M=10 (11 operator applications), 25 Hz Ricker near the surface centre, dt 2 ms, "
                 "full-surface receiver gather")
DATA = "synthetic: seeded smooth random 1500-4500 m/s model with a 4500 m/s salt ellipsoid"


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class Dist:
    """Barrier and max-reduction over ranks (gloo, host tensors)."""

    def __init__(self, world):
        self.world = world
        self.dist = None
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.dist = dist

    def barrier(self):
        if self.dist:
            self.dist.barrier()

    def max(self, v: float) -> float:
        return self._reduce(v, "MAX")

    def sum(self, v: float) -> float:
        return self._reduce(v, "SUM")

    def _reduce(self, v: float, op: str) -> float:
        if not self.dist:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.dist.all_reduce(t, op=getattr(self.dist.ReduceOp, op))
        return float(t.item())

    def close(self):
        if self.dist:
            self.dist.destroy_process_group()


def replica_rate(world: int, cells: float, steps: int, ms_max: float) -> float:
    """Whole-job Gcell-steps/s of `world` independent replicas (one shot per
    rank, each `cells` cells for `steps` steps) timed by the slowest rank."""
    return world * cells * steps / (ms_max * 1e-3) / 1e9


def device_sync():
    try:
        import torch
        if torch.cuda.is_available():
            torch.cuda.synchronize()
    except Exception:
        pass


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self):
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.QUERY, "--format=csv,noheader,nounits",
                                          "-i", os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0],
                                          "-lms", "50"], stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.f.close()
        rows = [r for r in csv.reader(io.StringIO(open(self.path).read())) if len(r) >= 9]
        os.unlink(self.path)
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].strip() == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons, "samples": len(rows)}


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(workload: str, kernel: str):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(path) as f:
            t = json.load(f)
        return t.get(workload, {}).get(kernel)
    except Exception:
        return None


def oracle_rate(kw, vel, nsteps: int, warm: int = 0):
    """Gcell-steps/s of the FP64 oracle over nsteps full-size steps (setup
    excluded), after `warm` untimed steps."""
    import oracle as O
    O.build()
    p = O.make_params(**kw)
    d = O.derive(p)
    if warm > 0:
        O.run(p, vel, warm)
    t0 = time.perf_counter()
    O.run(p, vel, 0)
    t_setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    O.run(p, vel, nsteps)
    t = time.perf_counter() - t0 - t_setup
    cells = d.nxb * d.nyb * d.nzb
    return cells * nsteps / max(t, 1e-9) / 1e9, O.threads(), t


def accuracy_vs_fp64(m, kw, vel, shot: int, nsteps: int):
    """Checker leg (outside every timed region): rel-L2 of the modeler's
    receiver gather over its first nsteps steps and of its P and Q after them,
    against the FP64 restatement of the same loop (oracle/oracle_torch.py,
    torch complex128 on the same GPU) run from the same start for the same
    steps."""
    import ose3d
    from oracle_torch import TorchOracle
    t0 = time.perf_counter()
    g = m.gather()[:, :nsteps].T.astype(np.float64)
    P = m.wavefield(ose3d.FIELD_P)
    Q = m.wavefield(ose3d.FIELD_Q)
    o = TorchOracle(kw, vel, "cuda", shot=shot)
    g64 = o.run(nsteps)
    P64, Q64 = o.P(), o.Q()
    del o

    def rel(a, b):
        return float(np.linalg.norm(np.asarray(a, np.float64) - b) / max(np.linalg.norm(b), 1e-300))

    return {"steps": nsteps, "gather_rel_l2": rel(g, g64), "P_rel_l2": rel(P, P64), "Q_rel_l2": rel(Q, Q64),
            "bar": 1e-4, "vs": "FP64 restatement of the same loop (torch complex128 on the same GPU)",
            "check_s": round(time.perf_counter() - t0, 1)}


def run_reference(args, rank):
    if rank != 0:
        return 0
    import workloads
    build, kw = workloads.CONFIGS[WORKLOAD]
    vel = build()
    nsteps = max(1, min(args.steps, 2))
    warm = min(max(args.warmup, 0), 1)      # one untimed step is enough on the host
    value, cores, t = oracle_rate(kw, vel, nsteps, warm)
    sample = (f"{nsteps} full-size step(s) of the {WORKLOAD} workload on the FP64 CPU oracle "
              f"(the reference has no CPU path of its own) after {warm} untimed, {t:.1f} s")
    line = {"metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": nsteps, "warmup": warm, "ms_per_step": 1e3 * t / nsteps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": DATA,
            "config": {"workload": WORKLOAD, "text": WORKLOAD_TEXT},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def shard(items, rank: int, world: int):
    """Round-robin share of independent units (shots) for one rank."""
    return list(items)[rank::world]


def run_batched(args, rank):
    """--workload batched64: 64 shots on windows of a 512 x 512 x 192 model
    advanced together (ose_batch_*), against the same 64 shots run one after
    another on single-shot handles.  Reports aggregate padded-cell throughput
    and the effective throughput (cells of the full model per shot).  On N
    GPUs the shots go round-robin to the ranks (no collective in the step);
    the slowest rank's time sets the aggregate."""
    _, world, local = dist_env()
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    dist = Dist(world)
    import __graft_entry__ as ge
    ge.build_library()
    import ose3d
    import workloads

    cfg = workloads.BATCHED
    model = cfg["model"]()
    all_wins = cfg["windows"]()
    wins = shard(all_wins, rank, world)
    p = ose3d.default_params(**cfg["params"])
    K = max(1, min(args.steps, 50))
    with ose3d.Batch(p, model, wins) as b:
        cells = [b.info(s)[1] for s in range(b.nshots)]
        t_tune = time.perf_counter()
        plans = "batch_plans.txt" if world == 1 else f"batch_plans_rank{rank}.txt"
        b.autotune(steps=2, cache_path=os.path.join(ROOT, "3d-ose_gb300", "lib", plans))
        t_tune = time.perf_counter() - t_tune
        tuning = b.tuning()
        b.reset()
        b.run(max(3, args.warmup))
        dist.barrier()
        ms = b.run_timed(K)
        dist.barrier()
    ms = dist.max(ms)
    total = dist.sum(float(sum(cells)))
    value = total * K / (ms * 1e-3) / 1e9
    effective = len(all_wins) * float(np.prod(model.shape)) * K / (ms * 1e-3) / 1e9
    if world > 1:
        if rank == 0:
            print(json.dumps({"metric": "aggregate Gcell-steps/s of 64 windowed shots (batched form)", "value": value,
                              "unit": UNIT, "n_gpus": world, "steps": K, "warmup": max(3, args.warmup),
                              "ms_per_step": ms / K, "higher_is_better": True, "scaling": "strong",
                              "vs_baseline": None, "dtype": "fp32", "data": "synthetic: seeded smooth random "
                              "1500-4500 m/s 512x512x192 model + salt",
                              "config": {"workload": "batched64", "shots": len(all_wins),
                                         "parallelism": f"shots round-robin over {world} GPUs",
                                         "padded_cells_total": total, "tuning_rank0": tuning},
                              "effective_gcell_steps_s": effective}), flush=True)
        dist.close()
        return 0
    # the same shots, one handle after another
    seq_ms = 0.0
    for w in wins:
        ix = np.clip(np.arange(w["x0"], w["x0"] + w["nx"]), 0, model.shape[0] - 1)
        iy = np.clip(np.arange(w["y0"], w["y0"] + w["ny"]), 0, model.shape[1] - 1)
        iz = np.clip(np.arange(w["z0"], w["z0"] + w["nz"]), 0, model.shape[2] - 1)
        ps = ose3d.default_params(nx=w["nx"], ny=w["ny"], nz=w["nz"], sxbeg=w["sx"], sybeg=w["sy"],
                                  szbeg=w["sz"], **cfg["params"])
        with ose3d.Modeler(ps, model[np.ix_(ix, iy, iz)]) as m:
            m.reset_shot(0)
            m.run(3)
            seq_ms += m.run_timed(K)
    seq = total * K / (seq_ms * 1e-3) / 1e9
    line = {"metric": "aggregate Gcell-steps/s of 64 windowed shots (batched form)", "value": value,
            "unit": UNIT, "n_gpus": 1, "steps": K, "warmup": max(3, args.warmup),
            "ms_per_step": ms / K, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "fp32", "data": "synthetic: seeded smooth random 1500-4500 m/s 512x512x192 model + salt",
            "config": {"workload": "batched64", "shots": len(wins), "padded_cells_total": total,
                       "window_range": [min(cells), max(cells)], "tuning": tuning,
                       "autotune_s": round(t_tune, 2)},
            "effective_gcell_steps_s": effective,
            "sequential_single_shot": {"value": seq, "ms_per_step": seq_ms / K,
                                       "speedup_of_batch": value / seq}}
    print(json.dumps(line), flush=True)
    return 0


def run_precision(args, rank):
    """--workload precision: the precision form.  For each z-pass arithmetic
    (FP32 FFT kernels; TF32, TF32X3, BF16X3 tensor-core DFT matmuls) the step
    rate on the padded 384 x 384 x 256 workload (15 Hz, 1500 steps) and on the
    256^3 workload, and the z-pass kernel's HBM rate and tensor FLOP rate
    (per cell per z pass: 4 DFT-16 matmul stages x 128 flop x products)."""
    if rank != 0:
        return 0
    import __graft_entry__ as ge
    ge.build_library()
    import ose3d
    import workloads

    peak, peak_kind = measured_peak_hbm()
    K = max(1, min(args.steps, 100))
    out = {}
    for wl in ("ose384x384x256", "ose256"):
        build, kw = workloads.CONFIGS[wl]
        vel = build()
        res = {}
        with ose3d.Modeler(ose3d.default_params(**kw), vel) as m:
            d = m.derived
            cells = d.nxb * d.nyb * d.nzb
            for name, mode in ose3d.PRECISIONS.items():
                m.precision = mode
                m.reset_shot(0)
                m.run(max(3, args.warmup))
                ms = m.run_timed(K)
                rows, _ = m.profile_step(reps=2)
                z = [r for r in rows if r["name"] in ("fft_z_kscale", "zpass")][0]
                prods = {"fp32": 0, "tf32": 1, "tf32x3": 3, "bf16x3": 3}[name]
                res[name] = {"gcell_steps_s": cells * K / (ms * 1e-3) / 1e9, "ms_per_step": ms / K,
                             "zpass_ms": z["ms"], "zpass_gbs": z["bytes"] / (z["ms"] * 1e-3) / 1e9,
                             "zpass_hbm_frac": z["bytes"] / (z["ms"] * 1e-3) / 1e9 / peak,
                             "zpass_tensor_tflops": 512.0 * prods * cells / (z["ms"] * 1e-3) / 1e12}
            out[wl] = {"grid": [d.nxb, d.nyb, d.nzb], "M": d.M,
                       "kernel_path": "generic" if d.path == 0 else "plane", "variants": res}
    base = out["ose384x384x256"]["variants"]
    line = {"metric": "Gcell-steps/s of the precision form (tensor-core z pass) vs the FP32 FFT z pass",
            "value": base["tf32x3"]["gcell_steps_s"], "unit": UNIT, "n_gpus": 1, "steps": K,
            "warmup": max(3, args.warmup), "ms_per_step": base["tf32x3"]["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "tf32x3",
            "data": DATA, "config": {"workload": "precision", "peak_hbm_gbs": peak,
                                     "peak_source": peak_kind, "results": out}}
    print(json.dumps(line), flush=True)
    return 0


def run_learned(args, rank):
    """--workload learned: the learned-boundary form.  Padded 256^3 grid =
    interior 240^3 + 8-cell sponge with the trained corrector on its 16-cell
    shell (tensor-core inference), against the same interior with a 64-cell
    sponge (padded 368^3, the plain run the form replaces) and against the thin
    grid without the corrector.  Reports step rates, the effective rate (cells
    of the wide grid per second of the learned step) and, over a bounded run,
    the interior error energy and receiver-gather rel-L2 of both thin runs
    against the wide run."""
    if rank != 0:
        return 0
    import __graft_entry__ as ge
    ge.build_library()
    import ose3d
    import torch
    import workloads
    import learn_boundary as LB

    params = np.load(LB.WEIGHTS)
    n = 240
    vel = workloads.smooth_random_salt(n, n, n, seed=505)
    K = max(1, min(args.steps, 100))
    acc_steps = 0 if args.no_accuracy else 300
    kw = lambda sp: LB.pair_params(n, 20.0, (120, 120, 8), acc_steps + K + 10, sp)  # noqa: E731
    res = {}
    wide_int = []
    ref_rows = None
    for mode in ("wide", "plain", "learned"):
        sp = LB.WIDE if mode == "wide" else LB.THIN
        m = ose3d.Modeler(ose3d.default_params(**kw(sp)), vel)
        if mode == "learned":
            m.set_corrector(params, LB.SHELL)
        d = m.derived
        m.reset_shot(0)
        buf = torch.zeros((n, n, n, 2), dtype=torch.float32, device="cuda")
        err = ref = 0.0
        rows = []
        every = 25
        for t in range(0, acc_steps, every):
            rows.append(m.run_record(every))
            m.state_box(0, (sp, sp, sp, n, n, n), buf.data_ptr(), (n, n, 0, 0, 0))
            if mode == "wide":
                wide_int.append(buf.clone())
            else:
                w = wide_int[t // every]
                err += float(((buf - w) ** 2).sum())
                ref += float((w ** 2).sum())
        g = np.concatenate(rows) if rows else np.zeros((0, 1), np.float32)
        m.run(max(3, args.warmup))
        ms = m.run_timed(K)
        prof, _ = m.profile_step(reps=1)
        cells = d.nxb * d.nyb * d.nzb
        r = {"grid": [d.nxb, d.nyb, d.nzb], "kernel_path": "generic" if d.path == 0 else "plane",
             "ms_per_step": ms / K, "gcell_steps_s": cells * K / (ms * 1e-3) / 1e9,
             "kernels_ms": {p["name"]: p["ms"] * p["launches_per_step"] for p in prof}}
        if mode == "wide":
            ref_rows = g
            wide_cells = cells
        elif acc_steps:
            r["interior_error_energy"] = err / max(ref, 1e-300)
            r["gather_rel_l2"] = float(np.linalg.norm(g - ref_rows) / np.linalg.norm(ref_rows))
        res[mode] = r
        m.close()
    lr = res["learned"]
    line = {"metric": "effective Gcell-steps/s of the learned-boundary form (cells of the 64-cell-sponge grid it "
                      "replaces per second)",
            "value": wide_cells * K / (lr["ms_per_step"] * K * 1e-3) / 1e9, "unit": UNIT, "n_gpus": 1,
            "steps": K, "warmup": max(3, args.warmup), "ms_per_step": lr["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32 solver, bf16 corrector",
            "data": "synthetic: seeded smooth random 1500-4500 m/s 240^3 interior + salt, 20 Hz Ricker",
            "config": {"workload": "learned", "interior": [n, n, n], "thin_sponge": LB.THIN,
                       "wide_sponge": LB.WIDE, "shell": LB.SHELL, "accuracy_steps": acc_steps,
                       "speedup_vs_wide": res["wide"]["ms_per_step"] / lr["ms_per_step"], "results": res}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true", help="timing only (no FP64 check)")
    ap.add_argument("--accuracy-steps", type=int, default=300,
                    help="steps of the shot compared with the FP64 restatement (the timed steps included)")
    ap.add_argument("--e2e-steps", type=int, default=0, help="steps of the end-to-end job (0: the workload's nt)")
    ap.add_argument("--workload", default=WORKLOAD,
                    choices=[WORKLOAD, "ose320x288x256", "ose384x384x256", "ose142", "ose142cerjan", "batched64",
                             "precision", "learned"])
    args = ap.parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank)
    if args.workload == "batched64":
        import numpy as np  # noqa: F401
        return run_batched(args, rank)
    if args.workload == "precision":
        return run_precision(args, rank)
    if args.workload == "learned":
        return run_learned(args, rank)
    if world > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    dist = Dist(world)

    import numpy as np
    import __graft_entry__ as ge
    ge.build_library()
    import ose3d
    import workloads

    wl = args.workload
    build, kw = workloads.CONFIGS[wl]
    vel = build()
    warm = max(3, args.warmup)
    if warm + args.steps + 1 > kw["nt"]:
        raise SystemExit(f"steps + warmup must stay below nt = {kw['nt']}")
    params = ose3d.default_params(**kw)
    m = ose3d.Modeler(params, vel)
    d = m.derived
    cells = d.nxb * d.nyb * d.nzb
    m.reset_shot(rank)
    m.run(warm)

    dist.barrier()
    device_sync()
    clk = ClockSampler()
    clk.start()
    ms = m.run_timed(args.steps)
    clocks = clk.stop()
    device_sync()
    dist.barrier()
    ms = dist.max(ms)
    value = replica_rate(world, cells, args.steps, ms)

    # accuracy of this shot against FP64 (rank 0): the timed steps plus
    # untimed ones up to --accuracy-steps, then gather, P and Q compared
    accuracy = None
    if rank == 0 and not args.no_accuracy:
        acc_steps = min(max(args.accuracy_steps, warm + args.steps), kw["nt"] - 3)
        if acc_steps > warm + args.steps:
            m.run(acc_steps - (warm + args.steps))
        accuracy = accuracy_vs_fp64(m, kw, vel, rank, acc_steps)

    # per-kernel launch durations (events bracketing each launch, one step)
    rows, launches_per_step = m.profile_step(reps=2)
    per_step = {r["name"]: r["launches_per_step"] for r in rows}
    share = {r["name"]: r["ms"] * per_step[r["name"]] for r in rows}
    total = sum(share.values())
    dom = max(rows, key=lambda r: share[r["name"]])
    achieved = dom["bytes"] / (dom["ms"] * 1e-3) / 1e9
    peak, peak_kind = measured_peak_hbm()
    roofline = {"bound": "hbm", "kernel": dom["name"], "achieved": achieved, "peak": peak,
                "unit": "GB/s", "frac": achieved / peak, "peak_source": peak_kind,
                "traffic": ncu_traffic(wl, dom["name"]),
                "algorithmic_bytes_per_launch": dom["bytes"], "ms_per_launch": dom["ms"],
                "kernel_shares": {k: v / total for k, v in share.items()},
                "step_bytes_model": sum(r["bytes"] * per_step[r["name"]] for r in rows) / cells,
                "step_achieved_gbs": sum(r["bytes"] * per_step[r["name"]] for r in rows) /
                (ms * 1e-3 / args.steps) / 1e9}
    m.close()

    # end to end through the C ABI from host buffers, the whole job of the
    # workload (its nt steps, as the reference's main runs it): create (model
    # upload), reset (wavelets), every step copying its receiver row to the
    # host, final P and Q back to the host
    e2e_steps = kw["nt"] if args.e2e_steps <= 0 else min(args.e2e_steps, kw["nt"])
    device_sync()
    t0 = time.perf_counter()
    m2 = ose3d.Modeler(params, vel)
    m2.reset_shot(rank)
    rows_out = m2.run_record(e2e_steps)
    q = m2.wavefield(ose3d.FIELD_Q)
    p_ = m2.wavefield(ose3d.FIELD_P)
    t_e2e = time.perf_counter() - t0
    m2.close()
    t_e2e = dist.max(t_e2e)
    h2d = (vel.nbytes + 2 * 4 * kw["nt"]) / e2e_steps
    d2h = (rows_out.nbytes + q.nbytes + p_.nbytes) / e2e_steps
    e2e = {"value": replica_rate(world, cells, e2e_steps, t_e2e * 1e3), "unit": UNIT,
           "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "steps": e2e_steps,
           "seconds": round(t_e2e, 3),
           "timing": "host wall clock around create + reset_shot + run_record (one receiver row to the host per "
                     "step) + final P and Q reads, over the workload's whole job"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        v, cores, t = oracle_rate(kw, vel, 1)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"1 full-size {wl} step on the FP64 CPU oracle ({t:.1f} s)"}
    dist.close()
    if rank != 0:
        return 0
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": warm, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp32", "data": DATA,
            "config": {"workload": wl, "text": WORKLOAD_TEXT if wl == WORKLOAD else wl, "grid": [d.nxb, d.nyb, d.nzb],
                       "M": d.M, "kernel_path": "generic" if d.path == 0 else "plane",
                       "l2": f"inputs larger than L2 (each field {cells * 8 / 1e6:.0f} MB)",
                       "parallelism": f"replicas x{world} (one independent shot per GPU)"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "accuracy": accuracy,
            "gpu_launches": launches_per_step * args.steps, "clocks": clocks}
    print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
