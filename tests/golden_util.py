"""Loading of the golden fixtures made by tests/golden/make_golden.py."""
import ast
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
CASES = ["small_judge_odd", "small_deep_source_odd_nt", "reference_default", "config1_142"]


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    g = {k: z[k] for k in z.files}
    g["params"] = ast.literal_eval(str(g["params"]))
    g["model_spec"] = ast.literal_eval(str(g["model_spec"]))
    return g


def model_of(g):
    from models import layered_noise_model, layered_perturbed_model, two_layer_model
    s = g["model_spec"]
    if s["kind"] == "layered_noise":
        return layered_noise_model(s["nx"], s["ny"], s["nz"], s["seed"])
    if s["kind"] == "layered_perturbed":
        return layered_perturbed_model(s["nx"], s["ny"], s["nz"], s["seed"])
    return two_layer_model(s["nx"], s["ny"], s["nz"], s["v_top"], s["v_bottom"], s["z_interface"])


def rel_l2(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    a = a.astype(np.complex128 if np.iscomplexobj(a) else np.float64)
    b = b.astype(np.complex128 if np.iscomplexobj(b) else np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
