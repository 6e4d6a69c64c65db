"""Register column transforms (ose_cols.cu, y and z passes of the generic path
for lengths 16 C) against the FP64 oracle: one operator application on grids
whose y and z lengths cover every compiled C (4, 6, 8, 9, 10, 11, 12, 16, 18,
20, 23, 24), and grids with 256 z planes, whose z pass is the 16-column
256-point kernel with runtime strides.  Bound: 2e-6 relative L2 (FP32
transforms)."""
import numpy as np
import pytest

import oracle as O
import ose3d
from golden_util import rel_l2

pytestmark = pytest.mark.gpu

# padded (nxb, nyb, nzb); sponge 4 on every side
GRIDS = [(48, 64, 96), (40, 144, 176), (24, 160, 192), (16, 288, 320), (16, 368, 384), (16, 256, 128),
         (64, 96, 256), (32, 48, 256)]


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as ge
    ge.build_library()
    ose3d.load_library()


@pytest.mark.parametrize("grid", GRIDS, ids=lambda g: "x".join(map(str, g)))
def test_generic_operator_with_column_kernels(grid):
    nxb, nyb, nzb = grid
    b = 4
    kw = dict(nx=nxb - 2 * b, ny=nyb - 2 * b, nz=nzb - 2 * b, bu=b, bd=b, bl=b, br=b, bf=b, bb=b, nt=4)
    rng = np.random.default_rng(nxb * 7 + nyb)
    vel = (1500 + 3000 * rng.random((kw["nx"], kw["ny"], kw["nz"]))).astype(np.float32)
    with ose3d.Modeler(ose3d.default_params(**kw), vel) as m:
        assert m.shape == (nzb, nyb, nxb)
        assert m.derived.path == ose3d.PATH_GENERIC
        x = (rng.standard_normal(m.shape) + 1j * rng.standard_normal(m.shape)).astype(np.complex64)
        y = m.apply_operator(x)
        vb = m.wavefield(ose3d.FIELD_V)
        R = m.derived.R
    ref = O.apply_operator(O.make_params(**kw), vb, R, x.astype(np.complex128))
    err = rel_l2(y, ref)
    print(f"{grid}: rel-L2 {err:.2e}")
    assert err < 2e-6
