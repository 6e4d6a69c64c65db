"""ctypes binding of liboseoracle.so, the FP64 CPU restatement of the
reference OSE loop (ose_oracle.c).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, always as the checker or the timed CPU baseline.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboseoracle.so")
REF_BIN = os.path.join(HERE, "_ref", "ref_ose")


class OseParams(ctypes.Structure):
    """Mirror of ose_params in include/ose3d.h."""

    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("bu", ctypes.c_int), ("bd", ctypes.c_int), ("bl", ctypes.c_int),
        ("br", ctypes.c_int), ("bf", ctypes.c_int), ("bb", ctypes.c_int),
        ("nt", ctypes.c_int),
        ("fm", ctypes.c_float), ("dt", ctypes.c_float), ("amp", ctypes.c_float),
        ("dx", ctypes.c_float), ("dy", ctypes.c_float), ("dz", ctypes.c_float),
        ("nshot", ctypes.c_int),
        ("sxbeg", ctypes.c_int), ("sybeg", ctypes.c_int), ("szbeg", ctypes.c_int),
        ("jsx", ctypes.c_int), ("jsy", ctypes.c_int), ("jsz", ctypes.c_int),
        ("gxbeg", ctypes.c_int), ("gybeg", ctypes.c_int), ("gzbeg", ctypes.c_int),
        ("jgx", ctypes.c_int), ("jgy", ctypes.c_int), ("jgz", ctypes.c_int),
        ("csdgather", ctypes.c_int),
        ("sponge_mode", ctypes.c_int), ("cerjan_factor", ctypes.c_float),
        ("hilbert_div_nt", ctypes.c_int), ("M_override", ctypes.c_int),
    ]


class OseDerived(ctypes.Structure):
    """Mirror of ose_derived in include/ose3d.h."""

    _fields_ = [
        ("nxb", ctypes.c_int), ("nyb", ctypes.c_int), ("nzb", ctypes.c_int),
        ("br", ctypes.c_int), ("bb", ctypes.c_int), ("bd", ctypes.c_int),
        ("ng", ctypes.c_int), ("M", ctypes.c_int), ("vmax", ctypes.c_float),
        ("R", ctypes.c_double), ("dtR", ctypes.c_double),
        ("dkx", ctypes.c_double), ("dky", ctypes.c_double), ("dkz", ctypes.c_double),
        ("bessel_tail", ctypes.c_double), ("device_bytes", ctypes.c_size_t),
        ("path", ctypes.c_int),
    ]


def make_params(**kw) -> OseParams:
    """Parameter block with the reference main()'s values (ose_3d.cu:75-118),
    overridden by keyword."""
    p = OseParams()
    base = dict(nx=101, ny=101, nz=101, bu=25, bd=25, bl=25, br=25, bf=25, bb=25,
                nt=300, fm=40.0, dt=0.001, amp=100.0, dx=10.0, dy=10.0, dz=10.0,
                nshot=1, sxbeg=50, sybeg=50, szbeg=0, jsx=1, jsy=1, jsz=1,
                gxbeg=0, gybeg=0, gzbeg=0, jgx=1, jgy=1, jgz=1, csdgather=0,
                sponge_mode=0, cerjan_factor=0.0, hilbert_div_nt=0, M_override=0)
    base.update(kw)
    for k, v in base.items():
        setattr(p, k, v)
    return p


def build(force: bool = False) -> str:
    """Compile liboseoracle.so with the committed Makefile (gcc, OpenMP)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE, "liboseoracle.so"], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER
        L.orc_derive_dims.argtypes = [P(OseParams), P(OseDerived)]
        L.orc_pad_model.argtypes = [P(OseParams), P(ctypes.c_float), P(ctypes.c_float)]
        L.orc_series.argtypes = [P(OseParams), ctypes.c_float, P(ctypes.c_double),
                                 P(ctypes.c_double), P(ctypes.c_int)]
        L.orc_sponge.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_float, P(ctypes.c_float)]
        L.orc_ricker.argtypes = [ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                 P(ctypes.c_float)]
        L.orc_hilbert.argtypes = [P(ctypes.c_float), ctypes.c_int, ctypes.c_int, P(ctypes.c_float)]
        L.orc_bessel.argtypes = [ctypes.c_int, ctypes.c_double, P(ctypes.c_double)]
        L.orc_apply_operator.argtypes = [P(OseParams), P(ctypes.c_float), ctypes.c_double,
                                         P(ctypes.c_double), P(ctypes.c_double)]
        L.orc_run.argtypes = [P(OseParams), P(ctypes.c_float), ctypes.c_int, ctypes.c_int,
                              ctypes.c_int, P(ctypes.c_double), P(ctypes.c_double),
                              P(ctypes.c_float)]
        L.orc_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _fp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def derive(p: OseParams) -> OseDerived:
    d = OseDerived()
    if lib().orc_derive_dims(ctypes.byref(p), ctypes.byref(d)):
        raise ValueError("bad parameters")
    return d


def pad_model(p: OseParams, vel_xyz: np.ndarray) -> np.ndarray:
    d = derive(p)
    v = np.ascontiguousarray(vel_xyz, dtype=np.float32)
    out = np.zeros((d.nzb, d.nyb, d.nxb), np.float32)
    lib().orc_pad_model(ctypes.byref(p), _fp(v), _fp(out))
    return out


def series(p: OseParams, vmax: float):
    R, dtR, M = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
    lib().orc_series(ctypes.byref(p), vmax, ctypes.byref(R), ctypes.byref(dtR), ctypes.byref(M))
    return R.value, dtR.value, M.value


def sponge(before: int, nn: int, after: int, mode: int = 0, factor: float = 0.0) -> np.ndarray:
    out = np.zeros(before + nn + after, np.float32)
    lib().orc_sponge(before, nn, after, mode, factor, _fp(out))
    return out


def ricker(nt: int, fm: float, dt: float, amp: float) -> np.ndarray:
    out = np.zeros(nt, np.float32)
    lib().orc_ricker(nt, fm, dt, amp, _fp(out))
    return out


def hilbert(w: np.ndarray, div_nt: bool = False) -> np.ndarray:
    w = np.ascontiguousarray(w, dtype=np.float32)
    out = np.zeros_like(w)
    lib().orc_hilbert(_fp(w), w.size, int(div_nt), _fp(out))
    return out


def bessel(M: int, dtR: float) -> np.ndarray:
    J = np.zeros(M + 2, np.float64)
    lib().orc_bessel(M, dtR, _dp(J))
    return J


def apply_operator(p: OseParams, vb: np.ndarray, R: float, x: np.ndarray) -> np.ndarray:
    """x: complex128 [nzb][nyb][nxb]; returns v*IFFT3(|k|FFT3(x))/(R N)."""
    xin = np.ascontiguousarray(x, dtype=np.complex128)
    out = np.zeros_like(xin)
    vbc = np.ascontiguousarray(vb, dtype=np.float32)
    rc = lib().orc_apply_operator(ctypes.byref(p), _fp(vbc), R,
                                  xin.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                  out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    if rc:
        raise RuntimeError("orc_apply_operator failed")
    return out


def run(p: OseParams, vel_xyz: np.ndarray, nsteps: int, shot: int = 0, it0: int = 0,
        P: np.ndarray | None = None, Q: np.ndarray | None = None):
    """Run nsteps of shot `shot` from step it0.  Returns (gather [it][ig] f32,
    P, Q as float64 [nzb][nyb][nxb])."""
    d = derive(p)
    shape = (d.nzb, d.nyb, d.nxb)
    P = np.zeros(shape, np.float64) if P is None else np.array(P, np.float64, copy=True)
    Q = np.zeros(shape, np.float64) if Q is None else np.array(Q, np.float64, copy=True)
    g = np.zeros((nsteps, d.ng), np.float32)
    v = np.ascontiguousarray(vel_xyz, dtype=np.float32)
    rc = lib().orc_run(ctypes.byref(p), _fp(v), shot, it0, nsteps, _dp(P), _dp(Q), _fp(g))
    if rc:
        raise RuntimeError("orc_run failed")
    return g, P, Q


def threads() -> int:
    return int(lib().orc_threads())
