"""The FP64 oracle against the golden outputs of the reference's own code
(tests/golden/, made by make_golden.py from ose_3d_lib.cu + ose_3d_kernel.cu)."""
import hashlib

import numpy as np
import pytest

import oracle as O
from golden_util import CASES, load, model_of, rel_l2


def oracle_params(g):
    p = dict(g["params"])
    p.pop("nsteps")
    return O.make_params(**p)


@pytest.mark.parametrize("name", CASES)
def test_model_generator_and_padding(name):
    g = load(name)
    vel = model_of(g)
    assert hashlib.sha256(vel.astype("<f4").tobytes()).hexdigest() == str(g["model_sha256"])
    p = oracle_params(g)
    d = O.derive(p)
    assert [d.nxb, d.nyb, d.nzb] == list(g["dims"])
    vb = O.pad_model(p, vel)
    # add_pml_layers_v_h is pure copying: the padded model must match bit for bit
    assert hashlib.sha256(vb.tobytes()).hexdigest() == str(g["vpad_sha256"])
    assert np.float32(vb.max()) == g["vmax"]
    R, dtR, M = O.series(p, float(vb.max()))
    assert M == int(g["M"])


@pytest.mark.parametrize("name", CASES)
def test_sponge_and_wavelets(name):
    g = load(name)
    p = g["params"]
    d = O.derive(oracle_params(g))
    ax = O.sponge(p["bl"], p["nx"], d.br)
    ay = O.sponge(p["bf"], p["ny"], d.bb)
    az = O.sponge(p["bu"], p["nz"], d.bd)
    for mine, ref in ((ax, g["att_x"]), (ay, g["att_y"]), (az, g["att_z"])):
        assert np.max(np.abs(mine - ref)) <= 2e-7
    w = O.ricker(p["nt"], p["fm"], p["dt"], p["amp"])
    assert np.max(np.abs(w - g["ricker"])) <= 1e-6 * np.max(np.abs(g["ricker"]))
    h = O.hilbert(w)
    assert np.max(np.abs(h - g["hilbert"])) <= 2e-6 * np.max(np.abs(g["hilbert"]))
    # main's own copy (ose_3d.cu:179) is divided by nt; the per-shot one is not
    h2 = O.hilbert(w, div_nt=True)
    assert np.max(np.abs(h2 - g["ricker_hil_main"])) <= 2e-6 * np.max(np.abs(g["ricker_hil_main"]))


@pytest.mark.parametrize("name", CASES)
def test_time_loop_matches_reference(name):
    """Gather and final wavefield of the FP64 restatement vs the reference's FP32
    code path: rel-L2 well inside the 1e-4 parity bar."""
    g = load(name)
    p = oracle_params(g)
    gather, P, Q = O.run(p, model_of(g), g["params"]["nsteps"])
    assert gather.shape == g["gather"].shape
    assert rel_l2(gather, g["gather"]) < 3e-5
    assert abs(np.linalg.norm(P) / g["P_norm"] - 1) < 3e-5
    assert abs(np.linalg.norm(Q) / g["Q_norm"] - 1) < 3e-5
    if "Q" in g:
        assert rel_l2(P, g["P"]) < 3e-5
        assert rel_l2(Q, g["Q"]) < 3e-5
    else:
        zs, ys = g["plane_index"]
        assert rel_l2(P[zs], g["P_plane_z"]) < 3e-5
        assert rel_l2(Q[zs], g["Q_plane_z"]) < 3e-5
        assert rel_l2(P[:, ys], g["P_plane_y"]) < 3e-5
        assert rel_l2(Q[:, ys], g["Q_plane_y"]) < 3e-5


def test_operator_is_real_and_linear():
    """L maps real fields to real fields (|k| is even), so the packed p + i q
    application equals two real applications."""
    rng = np.random.default_rng(5)
    p = O.make_params(nx=10, ny=12, nz=8, bu=3, bd=3, bl=3, br=3, bf=2, bb=2, nt=8)
    d = O.derive(p)
    vel = (2000 + 500 * rng.random((10, 12, 8))).astype(np.float32)
    vb = O.pad_model(p, vel)
    R, _, _ = O.series(p, float(vb.max()))
    a = rng.standard_normal((d.nzb, d.nyb, d.nxb))
    b = rng.standard_normal((d.nzb, d.nyb, d.nxb))
    La = O.apply_operator(p, vb, R, a.astype(np.complex128))
    Lb = O.apply_operator(p, vb, R, b.astype(np.complex128))
    Lab = O.apply_operator(p, vb, R, a + 1j * b)
    assert np.max(np.abs(La.imag)) < 1e-12 * np.max(np.abs(La.real))
    assert np.allclose(Lab, La.real + 1j * Lb.real, rtol=0, atol=1e-12 * np.max(np.abs(Lab)))
