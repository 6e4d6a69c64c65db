"""The FP64 torch restatement (oracle/oracle_torch.py) against the C oracle:
both are FP64, so they agree to rounding (1e-10 rel-L2) at test sizes."""
import numpy as np
import pytest

import oracle as O
from golden_util import load, model_of, rel_l2

torch = pytest.importorskip("torch")


@pytest.mark.parametrize("name", ["small_judge_odd", "small_deep_source_odd_nt"])
def test_torch_oracle_matches_c_oracle(name):
    from oracle_torch import TorchOracle
    g = load(name)
    kw = dict(g["params"])
    ns = kw.pop("nsteps")
    vel = model_of(g)
    t = TorchOracle(kw, vel, "cpu")
    gt = t.run(ns)
    gc, Pc, Qc = O.run(O.make_params(**kw), vel, ns)
    assert rel_l2(gt, gc) < 1e-6       # the C gather is stored as float32
    assert rel_l2(t.Q(), Qc) < 1e-10
    assert rel_l2(t.P(), Pc) < 1e-10
    # and the golden reference run
    assert rel_l2(gt, g["gather"]) < 3e-5
