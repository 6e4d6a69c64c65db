"""Precision form (ose_tensor.cu): the z pass (FFT_z, * |k|, IFFT_z) as four
batched DFT-16 matmuls on the tcgen05 tensor cores, against the FP64 oracle.

Tolerances (relative L2 of one operator application) follow the arithmetic of
each variant's products: TF32 rounds every operand to 11 significant bits
(unit round-off 2^-11 = 4.9e-4) over four matmul stages: measured 4.8e-4,
bound 1e-3; TF32X3 keeps about 22 bits (hi + lo, lo*lo dropped), the FP32 FFT
class: measured 4.0e-7, bound 2e-6; BF16X3 keeps about 16 bits: measured
6.5e-6, bound 2e-5.  The FP32 FFT kernels measure 2.3e-7."""
import numpy as np
import pytest

import oracle as O
import ose3d
from golden_util import rel_l2

pytestmark = pytest.mark.gpu

TOL = {"fp32": 1e-6, "tf32": 1e-3, "tf32x3": 2e-6, "bf16x3": 2e-5}
# 40 steps on a rough random model (gather and final Q).  FP32 and TF32X3
# meet the 1e-4 parity bar of the FP32 path with room to spare; BF16X3 (about
# 16 significant bits per product) does not meet it and is held to the bound
# of its own arithmetic class; single-pass TF32 is far outside both.
TOL_STEPS = {"fp32": 5e-5, "tf32x3": 5e-5}
PARITY_BAR = 1e-4
TOL_STEPS_BF16X3 = 3e-4

# padded 32 x 24 x 256
KW = dict(nx=12, ny=8, nz=216, bu=20, bd=20, bl=10, br=10, bf=8, bb=8, nt=40, fm=30.0, dt=0.001,
          amp=100.0, dx=10.0, dy=10.0, dz=10.0, sxbeg=6, sybeg=4, szbeg=5, gzbeg=0)


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as ge
    ge.build_library()
    ose3d.load_library()


@pytest.fixture(scope="module")
def vel():
    rng = np.random.default_rng(5)
    return (1500 + 3000 * rng.random((KW["nx"], KW["ny"], KW["nz"]))).astype(np.float32)


@pytest.mark.parametrize("mode", ["fp32", "tf32", "tf32x3", "bf16x3"])
def test_operator_matches_oracle(vel, mode):
    rng = np.random.default_rng(17)
    with ose3d.Modeler(ose3d.default_params(**KW), vel) as m:
        assert m.shape == (256, 24, 32)
        m.precision = mode
        assert m.precision == ose3d.PRECISIONS[mode]
        x = (rng.standard_normal(m.shape) + 1j * rng.standard_normal(m.shape)).astype(np.complex64)
        y = m.apply_operator(x)
        vb = m.wavefield(ose3d.FIELD_V)
        R = m.derived.R
    ref = O.apply_operator(O.make_params(**KW), vb, R, x.astype(np.complex128))
    err = rel_l2(y, ref)
    print(f"operator {mode}: rel-L2 {err:.3e}")
    assert err < TOL[mode]


def _steps_error(vel, mode):
    p = O.make_params(**KW)
    with ose3d.Modeler(ose3d.default_params(**KW), vel) as m:
        m.precision = mode
        m.reset_shot(0)
        g = m.run_record(KW["nt"])
        q = m.wavefield(ose3d.FIELD_Q)
    G, P, Q = O.run(p, vel, KW["nt"])
    eg, eq = rel_l2(g, G), rel_l2(q, Q)
    print(f"40 steps {mode}: gather {eg:.3e} Q {eq:.3e}")
    return eg, eq


@pytest.mark.parametrize("mode", ["fp32", "tf32x3"])
def test_steps_meet_parity_bar(vel, mode):
    """40 steps (gather and final Q) against the FP64 C oracle, inside the
    1e-4 bar."""
    eg, eq = _steps_error(vel, mode)
    assert eg < TOL_STEPS[mode] and eq < TOL_STEPS[mode]
    assert max(eg, eq) < PARITY_BAR


def test_bf16x3_steps_within_its_class(vel):
    """BF16X3 after 40 steps: within the bound of its arithmetic class, which
    is above the 1e-4 parity bar (the variant does not meet it)."""
    eg, eq = _steps_error(vel, "bf16x3")
    assert eg < TOL_STEPS_BF16X3 and eq < TOL_STEPS_BF16X3


def test_switching_back_to_fp32_is_bitwise(vel):
    with ose3d.Modeler(ose3d.default_params(**KW), vel) as a, \
            ose3d.Modeler(ose3d.default_params(**KW), vel) as b:
        b.precision = "bf16x3"
        b.reset_shot(0)
        b.run(3)
        b.precision = "fp32"
        a.reset_shot(0)
        b.reset_shot(0)
        a.run(5)
        b.run(5)
        assert np.array_equal(a.wavefield(ose3d.FIELD_Q), b.wavefield(ose3d.FIELD_Q))


def test_unsupported_sizes_are_rejected():
    kw = dict(KW, nz=100)   # nzb = 140
    vel = np.full((kw["nx"], kw["ny"], kw["nz"]), 2000.0, np.float32)
    with ose3d.Modeler(ose3d.default_params(**kw), vel) as m:
        with pytest.raises(ose3d.OseError) as ei:
            m.precision = "tf32x3"
        assert "256" in str(ei.value)
        assert m.precision == ose3d.PRECISION_FP32


def test_plane_path_with_tensor_zpass():
    """256^3: the cluster path and the generic path share the tensor-core z
    pass; both against the FP64 oracle."""
    import workloads
    kw = dict(nx=196, ny=196, nz=196, bu=30, bd=30, bl=30, br=30, bf=30, bb=30, nt=8, fm=25.0,
              dt=0.002, amp=100.0, dx=10.0, dy=10.0, dz=10.0, sxbeg=98, sybeg=98, szbeg=5, gzbeg=0)
    vel = workloads.smooth_random_salt(196, 196, 196, seed=3)
    rng = np.random.default_rng(3)
    out = {}
    with ose3d.Modeler(ose3d.default_params(**kw), vel) as m:
        assert m.derived.path == ose3d.PATH_PLANE
        m.precision = "tf32x3"
        x = (rng.standard_normal(m.shape) + 1j * rng.standard_normal(m.shape)).astype(np.complex64)
        out["plane"] = m.apply_operator(x)
        m.select_path(ose3d.PATH_GENERIC)
        out["generic"] = m.apply_operator(x)
        vb = m.wavefield(ose3d.FIELD_V)
        R = m.derived.R
    ref = O.apply_operator(O.make_params(**kw), vb, R, x.astype(np.complex128))
    for k, y in out.items():
        err = rel_l2(y, ref)
        print(f"256^3 {k} tf32x3: rel-L2 {err:.3e}")
        assert err < TOL["tf32x3"]
