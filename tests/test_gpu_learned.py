"""The trained boundary corrector (3d-ose_gb300/weights/corrector.npy, made by
learn_boundary.py train: 200 solver pairs, interior 48^3, 8- vs 64-cell
sponge) on held-out cases: the thin-sponge run with the corrector against the
same run without it, both measured against the 64-cell-sponge run.

Measured when the weights were made (4 held-out cases, 300 steps): interior
error energy 0.24-0.42 without, 0.022-0.050 with the corrector (gain 8-11x);
gather rel-L2 0.63-1.48 without, 0.31-0.45 with.  On the two cases of this
test (200 steps) the gains were 6.0x and 6.8x; the test asks for 4x.  At twice
the training size (interior 96^3, 112^3 thin grid against 224^3 wide, 300
steps, two held-out cases) the gains were 5.1x and 7.1x; asked: 4x."""
import os

import numpy as np
import pytest

import ose3d

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as ge
    ge.build_library()
    ose3d.load_library()


@pytest.mark.parametrize("n,steps,seed", [(48, 200, 4242), (96, 300, 777)])
def test_trained_corrector_reduces_boundary_error(n, steps, seed):
    pytest.importorskip("torch")
    import learn_boundary as LB
    assert os.path.exists(LB.WEIGHTS)
    params = np.load(LB.WEIGHTS)
    assert params.size == ose3d.corrector_param_count()
    res = LB.evaluate(params, seed=seed, cases=2, n=n, steps=steps)
    for r in res:
        print(f"fm {r['fm']:.1f} Hz: error energy {r['plain']['interior_error_energy']:.3e} -> "
              f"{r['learned']['interior_error_energy']:.3e} (gain {r['gain']:.1f}x), gather "
              f"{r['plain']['gather_rel_l2']:.3f} -> {r['learned']['gather_rel_l2']:.3f}")
        assert r["gain"] > 4.0
        assert r["learned"]["gather_rel_l2"] < r["plain"]["gather_rel_l2"]
