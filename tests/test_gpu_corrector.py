"""Learned boundary corrector (ose_learn.cu): the hand-written CUDA forward and
gradient kernels against the FP64 torch-autograd restatement on the CPU
(oracle/corrector_torch.py), and the corrector inside a modeler's step.

Tolerances: FP32 kernels against FP64 -- output and loss 1e-5 relative,
gradients 1e-5 relative L2 per layer (sums over ~10^4 products; measured
about 1.5e-7)."""
import numpy as np
import pytest

import corrector_torch as CT
import ose3d
from golden_util import rel_l2

pytestmark = pytest.mark.gpu

SHAPE = (16, 20, 24)          # z, y, x: 20 is not a multiple of the 8-cell tile
SHELL = 6
SPONGE = (3, 2, 3, 3, 2, 3)   # x-, x+, y-, y+, z-, z+


@pytest.fixture(scope="module", autouse=True)
def built():
    import __graft_entry__ as ge
    ge.build_library()
    ose3d.load_library()


def smooth(rng, shape, sigma=2.0):
    from scipy.ndimage import gaussian_filter
    return gaussian_filter(rng.standard_normal(shape), sigma, mode="wrap")


def sample(seed):
    rng = np.random.default_rng(seed)
    P, Q = smooth(rng, SHAPE), smooth(rng, SHAPE)
    vel = 1500 + 3000 * rng.random(SHAPE)
    tP = P + 0.05 * smooth(rng, SHAPE)
    tQ = Q + 0.05 * smooth(rng, SHAPE)
    return P, Q, vel, tP, tQ


def dev(torch, *arrs):
    return [torch.as_tensor(np.ascontiguousarray(a, np.float32), device="cuda") for a in arrs]


def pack(P, Q):
    return np.stack([P, Q], axis=-1)


def test_forward_and_gradients_match_fp64_autograd():
    torch = pytest.importorskip("torch")
    P, Q, vel, tP, tQ = sample(1)
    params = CT.init_params(seed=3, scale=1.0)
    params[-2:] = [0.01, -0.02]
    # round-trip the parameters through float32 so both sides use the same values
    p64 = params.astype(np.float64)
    loss64, g64, out64, s64, _ = CT.loss_and_grads(p64, P.astype(np.float32).astype(np.float64),
                                                Q.astype(np.float32).astype(np.float64),
                                                vel.astype(np.float32).astype(np.float64),
                                                tP.astype(np.float32).astype(np.float64),
                                                tQ.astype(np.float32).astype(np.float64), SHELL, SPONGE)
    st, v, tg = dev(torch, pack(P, Q), vel, pack(tP, tQ))
    out = torch.zeros(SHAPE + (2,), dtype=torch.float32, device="cuda")
    with ose3d.Corrector(SHAPE, SPONGE, shell=SHELL) as c:
        info = c.info()
        sh, wr = CT.masks(SHAPE, SHELL, SPONGE)
        assert info["shell_cells"] == sh.sum() and info["write_cells"] == wr.sum()
        c.set_params(params)
        s = c.forward(st.data_ptr(), v.data_ptr(), out.data_ptr())
        torch.cuda.synchronize()
        assert abs(s - s64) / s64 < 1e-6
        o = out.cpu().numpy()
        e_out = rel_l2(np.moveaxis(o, -1, 0), out64)
        c.train_sample(st.data_ptr(), v.data_ptr(), tg.data_ptr())
        torch.cuda.synchronize()
        loss = c.loss()
        g = c.grads()
    print(f"corrector fp32 vs fp64: out {e_out:.2e} loss {abs(loss - loss64) / loss64:.2e}")
    assert e_out < 1e-5
    assert abs(loss - loss64) / loss64 < 1e-5
    off = 0
    for i, (ci, co) in enumerate(zip(CT.CIN, CT.COUT)):
        nw = 27 * ci * co
        if i == 0:   # channels 6, 7 are zero inputs: their weights get zero gradient
            gw = g[off:off + nw].reshape(27, ci, co)
            assert np.all(gw[:, 6:, :] == 0)
        ew = rel_l2(g[off:off + nw], g64[off:off + nw])
        eb = rel_l2(g[off + nw:off + nw + co], g64[off + nw:off + nw + co])
        print(f"layer {i}: dW {ew:.2e} db {eb:.2e}")
        assert ew < 1e-5 and eb < 1e-5
        off += nw + co


def test_apply_adds_the_scaled_output_at_write_cells_only():
    torch = pytest.importorskip("torch")
    P, Q, vel, _, _ = sample(2)
    params = CT.init_params(seed=5)
    params[-2:] = [0.3, -0.1]
    st, v = dev(torch, pack(P, Q), vel)
    before = st.cpu().numpy().copy()
    out = torch.zeros(SHAPE + (2,), dtype=torch.float32, device="cuda")
    with ose3d.Corrector(SHAPE, SPONGE, shell=SHELL) as c:
        c.set_params(params)
        s = c.forward(st.data_ptr(), v.data_ptr(), out.data_ptr())
        c.apply(st.data_ptr(), v.data_ptr())
    after = st.cpu().numpy()
    o = out.cpu().numpy()
    _, wr = CT.masks(SHAPE, SHELL, SPONGE)
    _, sl = CT.scales(P.astype(np.float32).astype(np.float64), Q.astype(np.float32).astype(np.float64),
                      SHELL, SPONGE)
    assert np.array_equal(after[~wr], before[~wr])
    np.testing.assert_allclose(after[wr], before[wr] + sl[wr][:, None] * o[wr], rtol=1e-5,
                               atol=1e-6 * np.abs(before).max())


def test_adam_reduces_the_loss():
    torch = pytest.importorskip("torch")
    P, Q, vel, tP, tQ = sample(4)
    st, v, tg = dev(torch, pack(P, Q), vel, pack(tP, tQ))
    with ose3d.Corrector(SHAPE, SPONGE, shell=SHELL) as c:
        c.set_params(CT.init_params(seed=7))
        losses = []
        for it in range(60):
            c.train_sample(st.data_ptr(), v.data_ptr(), tg.data_ptr())
            losses.append(c.adam(1e-3, 1))
    print(f"adam: loss {losses[0]:.4e} -> {losses[-1]:.4e}")
    assert losses[-1] < 0.5 * losses[0]


def test_zero_corrector_leaves_the_modeler_bitwise_unchanged():
    kw = dict(nx=40, ny=40, nz=40, bu=8, bd=8, bl=8, br=8, bf=8, bb=8, nt=30, fm=25.0, dt=0.002,
              amp=100.0, sxbeg=20, sybeg=20, szbeg=5)
    vel = np.full((40, 40, 40), 2500.0, np.float32)
    zero = np.zeros(ose3d.corrector_param_count(), np.float32)
    with ose3d.Modeler(ose3d.default_params(**kw), vel) as a, ose3d.Modeler(ose3d.default_params(**kw), vel) as b:
        b.set_corrector(zero)
        for m in (a, b):
            m.reset_shot(0)
            m.run(20)
        assert np.array_equal(a.wavefield(ose3d.FIELD_Q), b.wavefield(ose3d.FIELD_Q))
        rows, _ = b.profile_step(reps=1)
        assert "corrector" in [r["name"] for r in rows]


@pytest.mark.parametrize("kernels", ["tensor", "fp32"])
def test_modeler_step_applies_the_corrector(kernels, monkeypatch):
    """One step with a non-zero corrector equals one plain step followed by the
    training object's FP32 apply on the same state: to FP32 rounding with the
    FP32 kernels, to BF16 rounding of the correction (2e-2 relative) with the
    tensor-core kernels."""
    torch = pytest.importorskip("torch")
    if kernels == "fp32":
        monkeypatch.setenv("OSE3D_CORRECTOR", "fp32")
    else:
        monkeypatch.delenv("OSE3D_CORRECTOR", raising=False)
    kw = dict(nx=40, ny=40, nz=40, bu=8, bd=8, bl=8, br=8, bf=8, bb=8, nt=30, fm=25.0, dt=0.002,
              amp=100.0, sxbeg=20, sybeg=20, szbeg=5)
    rng = np.random.default_rng(9)
    vel = (1500 + 3000 * rng.random((40, 40, 40))).astype(np.float32)
    params = CT.init_params(seed=11)
    params[-2:] = [0.2, 0.1]
    with ose3d.Modeler(ose3d.default_params(**kw), vel) as a, ose3d.Modeler(ose3d.default_params(**kw), vel) as b:
        a.reset_shot(0)
        b.reset_shot(0)
        a.run(10)
        b.run(10)
        b.set_corrector(params)
        a.run(1)
        b.run(1)
        shape = a.shape
        st = torch.zeros(shape + (2,), dtype=torch.float32, device="cuda")
        a.state_box(0, (0, 0, 0, shape[2], shape[1], shape[0]), st.data_ptr(), (shape[2], shape[1], 0, 0, 0))
        vb = a.wavefield(ose3d.FIELD_V)
        v = torch.as_tensor(vb, device="cuda")
        with ose3d.Corrector(shape, (8, 8, 8, 8, 8, 8), shell=16) as c:
            c.set_params(params)
            c.apply(st.data_ptr(), v.data_ptr())
        q = st.cpu().numpy()[..., 1]
        qb = b.wavefield(ose3d.FIELD_Q)
        qa = a.wavefield(ose3d.FIELD_Q)
        assert not np.array_equal(qb, qa)
        if kernels == "fp32":
            assert rel_l2(qb, q) < 1e-6
        else:
            e = rel_l2(qb.astype(np.float64) - qa, q.astype(np.float64) - qa)
            print(f"tensor-core correction vs FP32: {e:.2e}")
            assert e < 2e-2
