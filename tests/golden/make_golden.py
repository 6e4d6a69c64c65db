"""Generate the golden fixtures of tests/golden/ by running the REFERENCE's own
code (ose_3d_lib.cu + ose_3d_kernel.cu from the reference tree, built by
`make -C oracle ref` into oracle/_ref/ref_ose and run on the host emulation of
the CUDA runtime and cuFFT).

Run from the repository root, where the reference tree is readable:
    python tests/golden/make_golden.py [--ref-dir DIR]

Each case writes <name>.npz holding the parameters, the inputs' provenance and
the reference outputs: padded model (or its hash), sponge tables, the shot's
Ricker and Hilbert traces, the receiver gather [it][ig] and the final P and Q.
"""
from __future__ import annotations

import argparse
import hashlib
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, HERE)
from models import layered_noise_model, layered_perturbed_model, two_layer_model  # noqa: E402

CASES = [
    dict(name="small_judge_odd",
         model=dict(kind="layered_noise", nx=20, ny=18, nz=16, seed=1),
         params=dict(nx=20, ny=18, nz=16, bu=6, bd=6, bl=6, br=5, bf=6, bb=6, nt=64, nsteps=40,
                     fm=40.0, dt=0.001, amp=100.0, dx=10.0, dy=10.0, dz=10.0,
                     sxbeg=10, sybeg=9, szbeg=2),
         full_fields=True),
    dict(name="small_deep_source_odd_nt",
         model=dict(kind="layered_noise", nx=16, ny=22, nz=18, seed=2),
         params=dict(nx=16, ny=22, nz=18, bu=5, bd=7, bl=4, br=6, bf=6, bb=4, nt=63, nsteps=30,
                     fm=30.0, dt=0.0015, amp=50.0, dx=12.0, dy=10.0, dz=8.0,
                     sxbeg=7, sybeg=11, szbeg=12),
         full_fields=True),
    dict(name="reference_default",
         model=dict(kind="two_layer", nx=101, ny=101, nz=101, v_top=3000.0, v_bottom=4000.0,
                    z_interface=30, reference_file="input/v3d_nx101_ny101_nz101.bin"),
         params=dict(nx=101, ny=101, nz=101, bu=25, bd=25, bl=25, br=25, bf=25, bb=25, nt=300,
                     nsteps=3, fm=40.0, dt=0.001, amp=100.0, dx=10.0, dy=10.0, dz=10.0,
                     sxbeg=50, sybeg=50, szbeg=0),
         full_fields=False),
    # the benchmark's config 1 (interior 101^3 + 20-cell sponge, padded 142^3 =
    # 2 x 71 on every axis; 20 Hz Ricker at (50, 50, 10), dt 2 ms) for a few
    # steps, with the reference's own sponge and receiver plane (z = 0)
    dict(name="config1_142",
         model=dict(kind="layered_perturbed", nx=101, ny=101, nz=101, seed=7),
         params=dict(nx=101, ny=101, nz=101, bu=20, bd=20, bl=20, br=20, bf=20, bb=20, nt=1000,
                     nsteps=4, fm=20.0, dt=0.002, amp=100.0, dx=10.0, dy=10.0, dz=10.0,
                     sxbeg=50, sybeg=50, szbeg=10),
         full_fields=False),
]


def make_model(spec):
    if spec["kind"] == "layered_noise":
        return layered_noise_model(spec["nx"], spec["ny"], spec["nz"], spec["seed"])
    if spec["kind"] == "layered_perturbed":
        return layered_perturbed_model(spec["nx"], spec["ny"], spec["nz"], spec["seed"])
    return two_layer_model(spec["nx"], spec["ny"], spec["nz"], spec["v_top"], spec["v_bottom"],
                           spec["z_interface"])


def padded(p):
    def fix(b0, n, b1):
        nb = b0 + n + b1
        return nb + (nb % 2)
    return fix(p["bl"], p["nx"], p["br"]), fix(p["bf"], p["ny"], p["bb"]), fix(p["bu"], p["nz"], p["bd"])


def run_case(case, ref_dir):
    spec, p = case["model"], case["params"]
    vel = make_model(spec)
    extra = {}
    if "reference_file" in spec:
        ref_path = os.path.join(ref_dir, spec["reference_file"])
        ref_vel = np.fromfile(ref_path, "<f4").reshape(vel.shape)
        assert np.array_equal(ref_vel, vel), "generator does not reproduce " + ref_path
        extra["reference_model_sha256"] = hashlib.sha256(ref_vel.tobytes()).hexdigest()
    nxb, nyb, nzb = padded(p)
    with tempfile.TemporaryDirectory() as td:
        for sub in ("output", "temp", "wf"):
            os.makedirs(os.path.join(td, sub))
        vel.astype("<f4").tofile(os.path.join(td, "model.bin"))
        with open(os.path.join(td, "params.txt"), "w") as f:
            f.write("model=model.bin\n")
            for k, v in p.items():
                f.write(f"{k}={v}\n")
        out = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "ref_ose"), "params.txt"],
                             cwd=td, check=True, capture_output=True, text=True).stdout
        last = out.strip().splitlines()[-1]
        stats = dict(kv.split("=") for kv in last.split())
        rd = lambda n: np.fromfile(os.path.join(td, n), "<f4")  # noqa: E731
        ng, nt, ns = p["nx"] * p["ny"], p["nt"], p["nsteps"]
        gather = rd("output/qshot2.bin").reshape(ng, nt)[:, :ns].T.copy()      # [it][ig]
        to_zyx = lambda a: a.reshape(nyb, nxb, nzb).transpose(2, 0, 1)  # noqa: E731
        q = to_zyx(rd("wf/q-final.bin"))
        pp = to_zyx(rd("wf/p-final.bin"))
        vpad = rd("temp/vpad.bin").reshape(nzb, nyb, nxb)
        res = dict(
            params=np.array(repr(p)), model_spec=np.array(repr(spec)),
            model_sha256=np.array(hashlib.sha256(vel.astype("<f4").tobytes()).hexdigest()),
            vpad_sha256=np.array(hashlib.sha256(vpad.tobytes()).hexdigest()),
            att_x=rd("temp/att_x_0.bin")[:nxb], att_y=rd("temp/att_y.bin"), att_z=rd("temp/att_z.bin"),
            ricker=rd("temp/ricker_card.bin"), hilbert=rd("temp/hilbert_card.bin"),
            ricker_hil_main=rd("temp/ricker_hil.bin"),
            att_x_dump=rd("temp/att_x_0.bin"),
            partest=np.array(open(os.path.join(td, "output/partest.txt"), "rb").read()),
            qshot2_bytes=np.int64(os.path.getsize(os.path.join(td, "output/qshot2.bin"))),
            gather=gather,
            vmax=np.float32(float(stats["vmax"])), M=np.int32(int(stats["M"])),
            dims=np.array([nxb, nyb, nzb], np.int32),
            P_norm=np.float64(np.linalg.norm(pp.astype(np.float64))),
            Q_norm=np.float64(np.linalg.norm(q.astype(np.float64))),
        )
        for k, v in extra.items():
            res[k] = np.array(v)
        if case["full_fields"]:
            res["P"] = pp.copy()
            res["Q"] = q.copy()
            res["vpad"] = vpad.copy()
        else:
            zs, ys = p["bu"] + p["szbeg"], p["bf"] + p["sybeg"]
            res["P_plane_z"], res["Q_plane_z"] = pp[zs].copy(), q[zs].copy()
            res["P_plane_y"], res["Q_plane_y"] = pp[:, ys].copy(), q[:, ys].copy()
            res["plane_index"] = np.array([zs, ys], np.int32)
    np.savez_compressed(os.path.join(HERE, case["name"] + ".npz"), **res)
    print(case["name"], last)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-dir", default=os.environ.get("OSE_REF_DIR") or os.path.abspath(
        os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "..", "..", "reference")))
    ap.add_argument("--only", default=None)
    a = ap.parse_args()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF_DIR={a.ref_dir}"],
                   check=True)
    for c in CASES:
        if a.only and c["name"] != a.only:
            continue
        run_case(c, a.ref_dir)


if __name__ == "__main__":
    main()
