"""Python binding of libose3d.so (ctypes over the C ABI of include/ose3d.h).

The class mirrors the reference program's flow (ose_3d.cu:145-304): create
(Alloc + model + sponge + plan), reset_shot (Xtdata_value + Alloc_wavelet),
step (inject + wavefield_extro_ori2 + record), run (the time loop), and the
output writers.  There is no CPU fallback: if the library or a GPU is missing,
loading or creating raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libose3d.so")

OK = 0
FIELD_P, FIELD_Q, FIELD_V = 0, 1, 2
LAYOUT_ZYX, LAYOUT_YXZ = 0, 1
SPONGE_REFERENCE, SPONGE_CERJAN = 0, 1
PATH_GENERIC, PATH_PLANE = 0, 1
PRECISION_FP32, PRECISION_TF32, PRECISION_TF32X3, PRECISION_BF16X3 = 0, 1, 2, 3
PRECISIONS = {"fp32": PRECISION_FP32, "tf32": PRECISION_TF32, "tf32x3": PRECISION_TF32X3,
              "bf16x3": PRECISION_BF16X3}
NOALLOC_MAX_CELLS = 262144   # OSE_NOALLOC_MAX_CELLS

STATUS = {0: "OSE_OK", 1: "OSE_ERR_INVALID", 2: "OSE_ERR_CUDA", 3: "OSE_ERR_NOMEM",
          4: "OSE_ERR_IO", 5: "OSE_ERR_UNSUPPORTED", 6: "OSE_ERR_STATE", 7: "OSE_ERR_NUMERIC",
          8: "OSE_ERR_TIMEOUT"}

# Every symbol include/ose3d.h declares.
EXPORTS = ["ose_default_params", "ose_padded_dims", "ose_create", "ose_create_from_file",
           "ose_destroy", "ose_last_error", "ose_get_derived", "ose_self_test_waits", "ose_reset_shot", "ose_step",
           "ose_run", "ose_run_record", "ose_run_timed", "ose_select_path", "ose_get_it", "ose_get_wavefield", "ose_set_wavefield",
           "ose_get_gather", "ose_get_wavelets", "ose_get_sponge", "ose_apply_operator",
           "ose_profile_step", "ose_write_outputs", "ose_version", "ose_apply_operator_noalloc",
           "ose_checkpoint_save", "ose_checkpoint_load", "ose_run_snapshots", "ose_write_su",
           "ose_write_segy", "ose_batch_create", "ose_batch_destroy", "ose_batch_last_error",
           "ose_batch_reset", "ose_batch_run", "ose_batch_run_timed", "ose_batch_info",
           "ose_batch_get_gather", "ose_batch_get_wavefield", "ose_batch_autotune",
           "ose_batch_get_tuning", "ose_set_precision", "ose_get_precision", "ose_set_corrector",
           "ose_state_box", "ose_corrector_param_count", "ose_corrector_create", "ose_corrector_destroy",
           "ose_corrector_last_error", "ose_corrector_info", "ose_corrector_set_params",
           "ose_corrector_get_params", "ose_corrector_get_grads", "ose_corrector_forward",
           "ose_corrector_apply", "ose_corrector_train_sample", "ose_corrector_adam", "ose_corrector_loss",
           "ose_rtm", "ose_batch_set_tuning", "ose_set_receivers"]
CORRECTOR_SHELL = 16   # OSE_CORRECTOR_SHELL

# void (*)(int it, const float* P, const float* Q, void* user)
SNAPSHOT_FN = ctypes.CFUNCTYPE(None, ctypes.c_int, ctypes.POINTER(ctypes.c_float),
                               ctypes.POINTER(ctypes.c_float), ctypes.c_void_p)


class OseError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class Params(ctypes.Structure):
    """ose_params (include/ose3d.h)."""

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


class Derived(ctypes.Structure):
    """ose_derived (include/ose3d.h)."""

    _fields_ = [
        ("nxb", ctypes.c_int), ("nyb", ctypes.c_int), ("nzb", ctypes.c_int),
        ("br", ctypes.c_int), ("bb", ctypes.c_int), ("bd", ctypes.c_int),
        ("ng", ctypes.c_int), ("M", ctypes.c_int), ("vmax", ctypes.c_float),
        ("R", ctypes.c_double), ("dtR", ctypes.c_double),
        ("dkx", ctypes.c_double), ("dky", ctypes.c_double), ("dkz", ctypes.c_double),
        ("bessel_tail", ctypes.c_double), ("device_bytes", ctypes.c_size_t),
        ("path", ctypes.c_int),
    ]


_lib = None


def load_library(path: str = LIB_PATH):
    """Load libose3d.so and declare every entry point.  Raises if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError(f"libose3d.so not built ({path}); run 3d-ose_gb300/build.py")
    L = ctypes.CDLL(path)
    P = ctypes.POINTER
    H = ctypes.c_void_p
    f32 = P(ctypes.c_float)
    sig = {
        "ose_default_params": ([P(Params)], ctypes.c_int),
        "ose_padded_dims": ([P(Params), P(ctypes.c_int), P(ctypes.c_int), P(ctypes.c_int)], ctypes.c_int),
        "ose_create": ([P(Params), f32, P(H)], ctypes.c_int),
        "ose_create_from_file": ([P(Params), ctypes.c_char_p, P(H)], ctypes.c_int),
        "ose_destroy": ([H], ctypes.c_int),
        "ose_last_error": ([H], ctypes.c_char_p),
        "ose_get_derived": ([H, P(Derived)], ctypes.c_int),
        "ose_self_test_waits": ([ctypes.c_double, P(ctypes.c_int)], ctypes.c_int),
        "ose_reset_shot": ([H, ctypes.c_int], ctypes.c_int),
        "ose_step": ([H], ctypes.c_int),
        "ose_run": ([H, ctypes.c_int, f32], ctypes.c_int),
        "ose_run_record": ([H, ctypes.c_int, f32], ctypes.c_int),
        "ose_run_timed": ([H, ctypes.c_int, f32], ctypes.c_int),
        "ose_select_path": ([H, ctypes.c_int], ctypes.c_int),
        "ose_set_precision": ([H, ctypes.c_int], ctypes.c_int),
        "ose_set_corrector": ([H, f32, ctypes.c_int], ctypes.c_int),
        "ose_rtm": ([H, f32, ctypes.c_int, ctypes.c_int, f32, f32], ctypes.c_int),
        "ose_set_receivers": ([H, ctypes.c_int, P(ctypes.c_int)], ctypes.c_int),
        "ose_state_box": ([H, ctypes.c_int, P(ctypes.c_int), ctypes.c_void_p, P(ctypes.c_int)], ctypes.c_int),
        "ose_corrector_param_count": ([], ctypes.c_size_t),
        "ose_corrector_create": ([ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, P(ctypes.c_int), P(H)],
                                 ctypes.c_int),
        "ose_corrector_destroy": ([H], ctypes.c_int),
        "ose_corrector_last_error": ([H], ctypes.c_char_p),
        "ose_corrector_info": ([H, P(ctypes.c_longlong), P(ctypes.c_longlong), P(ctypes.c_int)], ctypes.c_int),
        "ose_corrector_set_params": ([H, f32], ctypes.c_int),
        "ose_corrector_get_params": ([H, f32], ctypes.c_int),
        "ose_corrector_get_grads": ([H, f32], ctypes.c_int),
        "ose_corrector_forward": ([H, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, f32], ctypes.c_int),
        "ose_corrector_apply": ([H, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
        "ose_corrector_train_sample": ([H, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
        "ose_corrector_adam": ([H, ctypes.c_float, ctypes.c_int, f32], ctypes.c_int),
        "ose_corrector_loss": ([H, f32, ctypes.c_int], ctypes.c_int),
        "ose_get_precision": ([H, P(ctypes.c_int)], ctypes.c_int),
        "ose_get_it": ([H, P(ctypes.c_int)], ctypes.c_int),
        "ose_get_wavefield": ([H, ctypes.c_int, f32, ctypes.c_int], ctypes.c_int),
        "ose_set_wavefield": ([H, ctypes.c_int, f32, ctypes.c_int], ctypes.c_int),
        "ose_get_gather": ([H, f32], ctypes.c_int),
        "ose_get_wavelets": ([H, f32, f32], ctypes.c_int),
        "ose_get_sponge": ([H, f32, f32, f32], ctypes.c_int),
        "ose_apply_operator": ([H, f32, f32], ctypes.c_int),
        "ose_profile_step": ([H, ctypes.c_int, ctypes.c_int, P(ctypes.c_int), P(ctypes.c_char_p),
                              f32, P(ctypes.c_double), P(ctypes.c_int)], ctypes.c_int),
        "ose_write_outputs": ([H, ctypes.c_char_p, ctypes.c_char_p], ctypes.c_int),
        "ose_version": ([], ctypes.c_char_p),
        "ose_checkpoint_save": ([H, ctypes.c_char_p], ctypes.c_int),
        "ose_checkpoint_load": ([H, ctypes.c_char_p], ctypes.c_int),
        "ose_run_snapshots": ([H, ctypes.c_int, ctypes.c_int, ctypes.c_int, SNAPSHOT_FN, ctypes.c_void_p],
                              ctypes.c_int),
        "ose_write_su": ([H, ctypes.c_char_p], ctypes.c_int),
        "ose_write_segy": ([H, ctypes.c_char_p], ctypes.c_int),
        "ose_batch_create": ([P(Params), f32, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                              P(ShotWindow), P(H)], ctypes.c_int),
        "ose_batch_destroy": ([H], ctypes.c_int),
        "ose_batch_last_error": ([H], ctypes.c_char_p),
        "ose_batch_reset": ([H], ctypes.c_int),
        "ose_batch_run": ([H, ctypes.c_int], ctypes.c_int),
        "ose_batch_run_timed": ([H, ctypes.c_int, f32], ctypes.c_int),
        "ose_batch_info": ([H, ctypes.c_int, P(Derived), P(ctypes.c_longlong)], ctypes.c_int),
        "ose_batch_get_gather": ([H, ctypes.c_int, f32], ctypes.c_int),
        "ose_batch_get_wavefield": ([H, ctypes.c_int, ctypes.c_int, f32], ctypes.c_int),
        "ose_batch_autotune": ([H, ctypes.c_int, ctypes.c_char_p, f32], ctypes.c_int),
        "ose_batch_set_tuning": ([H] + [ctypes.c_int] * 6, ctypes.c_int),
        "ose_batch_get_tuning": ([H] + [P(ctypes.c_int)] * 6,
                                 ctypes.c_int),
        "ose_apply_operator_noalloc": ([ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                        ctypes.c_float, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def apply_operator_noalloc(nxb: int, nyb: int, nzb: int, dx: float, dy: float, dz: float, R: float,
                           vel_ptr: int, in_ptr: int, out_ptr: int, stream: int = 0) -> int:
    """ose_apply_operator_noalloc on device pointers (integers, e.g. from a
    framework tensor's data pointer); returns the ose_status.  For callers that
    cannot allocate device memory: the library allocates nothing here."""
    return load_library().ose_apply_operator_noalloc(
        nxb, nyb, nzb, dx, dy, dz, R, ctypes.c_void_p(vel_ptr), ctypes.c_void_p(in_ptr),
        ctypes.c_void_p(out_ptr), ctypes.c_void_p(stream) if stream else None)


def self_test_waits(limit_ms: float = 5.0) -> int:
    """ose_self_test_waits: run each bounded in-kernel wait (plane exchange,
    persistent-batch grid barrier, MMA completion) against something that
    never completes, with limit_ms instead of the production limit; returns
    the mask of waits that ran out and recorded it (7 = all three)."""
    L = load_library()
    out = ctypes.c_int(0)
    st = L.ose_self_test_waits(float(limit_ms), ctypes.byref(out))
    if st != 0:
        raise OseError(st, L.ose_last_error(None).decode())
    return out.value


def default_params(**kw) -> Params:
    """The reference main()'s hard-coded parameters (ose_3d.cu:75-118), overridden by keyword."""
    p = Params()
    load_library().ose_default_params(ctypes.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise KeyError(k)
        setattr(p, k, v)
    return p


def _f32(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class ShotWindow(ctypes.Structure):
    """ose_shot_window (include/ose3d.h)."""

    _fields_ = [(k, ctypes.c_int) for k in ("x0", "y0", "z0", "nx", "ny", "nz", "sx", "sy", "sz")]


def receiver_line(gxbeg: int, gybeg: int, gzbeg: int, jgx: int, jgy: int, jgz: int, n: int) -> np.ndarray:
    """The reference's receiver geometry (sg_init_device): receiver i at
    (gxbeg + i jgx, gybeg + i jgy, gzbeg + i jgz), i < n."""
    i = np.arange(n)
    return np.stack([gxbeg + i * jgx, gybeg + i * jgy, gzbeg + i * jgz], axis=1).astype(np.int32)


class Corrector:
    """Training object of the learned boundary corrector on one padded grid
    (ose_corrector_*).  Device buffers are passed as integer device pointers
    (e.g. torch's tensor.data_ptr()); work runs on the default stream."""

    def __init__(self, shape_zyx, sponge6, shell: int = CORRECTOR_SHELL):
        self._lib = load_library()
        nz, ny, nx = shape_zyx
        h = ctypes.c_void_p()
        sp = (ctypes.c_int * 6)(*[int(v) for v in sponge6])
        rc = self._lib.ose_corrector_create(nx, ny, nz, shell, sp, ctypes.byref(h))
        if rc != OK:
            raise OseError(rc, self._lib.ose_corrector_last_error(None).decode())
        self._h = h
        self.shape = tuple(shape_zyx)
        self.nparams = int(self._lib.ose_corrector_param_count())

    def _check(self, rc):
        if rc != OK:
            raise OseError(rc, self._lib.ose_corrector_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.ose_corrector_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        sc, wc, nt = ctypes.c_longlong(), ctypes.c_longlong(), ctypes.c_int()
        self._check(self._lib.ose_corrector_info(self._h, ctypes.byref(sc), ctypes.byref(wc), ctypes.byref(nt)))
        return dict(shell_cells=sc.value, write_cells=wc.value, tiles=nt.value)

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.nparams
        self._check(self._lib.ose_corrector_set_params(self._h, _f32(p)))

    def params(self) -> np.ndarray:
        p = np.zeros(self.nparams, np.float32)
        self._check(self._lib.ose_corrector_get_params(self._h, _f32(p)))
        return p

    def grads(self) -> np.ndarray:
        g = np.zeros(self.nparams, np.float32)
        self._check(self._lib.ose_corrector_get_grads(self._h, _f32(g)))
        return g

    def forward(self, state_ptr: int, vel_ptr: int, out_ptr: int | None = None) -> float:
        s = ctypes.c_float()
        self._check(self._lib.ose_corrector_forward(self._h, state_ptr, vel_ptr, out_ptr, ctypes.byref(s)))
        return s.value

    def apply(self, state_ptr: int, vel_ptr: int):
        self._check(self._lib.ose_corrector_apply(self._h, state_ptr, vel_ptr))

    def train_sample(self, state_ptr: int, vel_ptr: int, target_ptr: int):
        self._check(self._lib.ose_corrector_train_sample(self._h, state_ptr, vel_ptr, target_ptr))

    def adam(self, lr: float, batch: int) -> float:
        l = ctypes.c_float()
        self._check(self._lib.ose_corrector_adam(self._h, lr, batch, ctypes.byref(l)))
        return l.value

    def loss(self, reset: bool = False) -> float:
        l = ctypes.c_float()
        self._check(self._lib.ose_corrector_loss(self._h, ctypes.byref(l), int(reset)))
        return l.value


def corrector_param_count() -> int:
    return int(load_library().ose_corrector_param_count())


class Batch:
    """Many shots on windows of one model, advanced together (ose_batch_*)."""

    def __init__(self, params: Params, model_xyz: np.ndarray, windows):
        self._lib = load_library()
        m = np.ascontiguousarray(model_xyz, dtype=np.float32)
        if m.ndim != 3:
            raise ValueError("model must be a 3-D [x][y][z] array")
        arr = (ShotWindow * len(windows))()
        for i, w in enumerate(windows):
            for k in ("x0", "y0", "z0", "nx", "ny", "nz", "sx", "sy", "sz"):
                setattr(arr[i], k, int(w[k]))
        h = ctypes.c_void_p()
        st = self._lib.ose_batch_create(ctypes.byref(params), _f32(m), m.shape[0], m.shape[1], m.shape[2],
                                        len(windows), arr, ctypes.byref(h))
        if st != OK:
            raise OseError(st, self._lib.ose_batch_last_error(None).decode())
        self._h = h
        self.params = params
        self.nshots = len(windows)
        self.windows = [dict(w) for w in windows]

    def close(self):
        if getattr(self, "_h", None):
            self._lib.ose_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != OK:
            raise OseError(st, self._lib.ose_batch_last_error(self._h).decode())

    def reset(self):
        self._check(self._lib.ose_batch_reset(self._h))

    def run(self, nsteps: int):
        self._check(self._lib.ose_batch_run(self._h, nsteps))

    def run_timed(self, nsteps: int) -> float:
        ms = ctypes.c_float()
        self._check(self._lib.ose_batch_run_timed(self._h, nsteps, ctypes.byref(ms)))
        return ms.value

    def info(self, shot: int):
        d = Derived()
        cells = ctypes.c_longlong()
        self._check(self._lib.ose_batch_info(self._h, shot, ctypes.byref(d), ctypes.byref(cells)))
        return d, cells.value

    def gather(self, shot: int) -> np.ndarray:
        w = self.windows[shot]
        g = np.zeros((w["nx"] * w["ny"], self.params.nt), np.float32)
        self._check(self._lib.ose_batch_get_gather(self._h, shot, _f32(g)))
        return g

    def wavefield(self, shot: int, which: int = FIELD_Q) -> np.ndarray:
        d, _ = self.info(shot)
        out = np.zeros((d.nzb, d.nyb, d.nxb), np.float32)
        self._check(self._lib.ose_batch_get_wavefield(self._h, shot, which, _f32(out)))
        return out

    def autotune(self, steps: int = 3, cache_path: str | None = None) -> float:
        ms = ctypes.c_float()
        self._check(self._lib.ose_batch_autotune(self._h, steps, cache_path.encode() if cache_path else None,
                                                 ctypes.byref(ms)))
        return ms.value

    def set_tuning(self, rows_scale=2048, txy=16, txz=16, radix_order=0, group_mb=0, lanes=0):
        self._check(self._lib.ose_batch_set_tuning(self._h, rows_scale, txy, txz, radix_order, group_mb, lanes))

    def tuning(self):
        v = [ctypes.c_int() for _ in range(6)]
        self._check(self._lib.ose_batch_get_tuning(self._h, *[ctypes.byref(x) for x in v]))
        return dict(zip(("rows_scale", "txy", "txz", "radix_order", "group_mb", "lanes"), (x.value for x in v)))


class Modeler:
    """One shot-at-a-time OSE modeler on the current CUDA device."""

    def __init__(self, params: Params, vel_xyz: np.ndarray):
        self._lib = load_library()
        self.params = params
        v = np.ascontiguousarray(vel_xyz, dtype=np.float32)
        if v.size != params.nx * params.ny * params.nz:
            raise ValueError("velocity model must hold nx*ny*nz values ([x][y][z])")
        h = ctypes.c_void_p()
        st = self._lib.ose_create(ctypes.byref(params), _f32(v), ctypes.byref(h))
        if st != OK:
            raise OseError(st, self._lib.ose_last_error(None).decode())
        self._h = h
        self.derived = Derived()
        self._check(self._lib.ose_get_derived(self._h, ctypes.byref(self.derived)))
        d = self.derived
        self.shape = (d.nzb, d.nyb, d.nxb)

    # -- lifetime -----------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._lib.ose_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, st):
        if st != OK:
            raise OseError(st, self._lib.ose_last_error(self._h).decode())

    # -- time loop ----------------------------------------------------------
    def reset_shot(self, shot: int = 0):
        self._check(self._lib.ose_reset_shot(self._h, shot))

    def step(self):
        self._check(self._lib.ose_step(self._h))

    def run(self, nsteps: int, want_gather: bool = False):
        """nsteps steps by graph replay; returns the [ig][it] gather if asked."""
        if want_gather:
            g = np.zeros((self.derived.ng, self.params.nt), np.float32)
            self._check(self._lib.ose_run(self._h, nsteps, _f32(g)))
            return g
        self._check(self._lib.ose_run(self._h, nsteps, None))
        return None

    def run_record(self, nsteps: int, out: np.ndarray | None = None) -> np.ndarray:
        """nsteps steps, returning their receiver rows [it][ig] (copied every step)."""
        if out is None:
            out = np.zeros((nsteps, self.derived.ng), np.float32)
        self._check(self._lib.ose_run_record(self._h, nsteps, _f32(out)))
        return out

    def run_timed(self, nsteps: int) -> float:
        ms = ctypes.c_float()
        self._check(self._lib.ose_run_timed(self._h, nsteps, ctypes.byref(ms)))
        return ms.value

    def select_path(self, path: int):
        """PATH_PLANE (256^3 only) or PATH_GENERIC."""
        self._check(self._lib.ose_select_path(self._h, path))
        self._check(self._lib.ose_get_derived(self._h, ctypes.byref(self.derived)))

    @property
    def precision(self) -> int:
        """Arithmetic of the z-axis transforms (PRECISION_*)."""
        v = ctypes.c_int()
        self._check(self._lib.ose_get_precision(self._h, ctypes.byref(v)))
        return v.value

    @precision.setter
    def precision(self, mode):
        """PRECISION_FP32 (FFT kernels) or a tensor-core DFT-matmul z pass:
        PRECISION_TF32, PRECISION_TF32X3, PRECISION_BF16X3 (or their names)."""
        if isinstance(mode, str):
            mode = PRECISIONS[mode]
        self._check(self._lib.ose_set_precision(self._h, int(mode)))

    @property
    def it(self) -> int:
        v = ctypes.c_int()
        self._check(self._lib.ose_get_it(self._h, ctypes.byref(v)))
        return v.value

    # -- data in and out ----------------------------------------------------
    def gather(self) -> np.ndarray:
        """[ig][it], ng x nt (the qshot2.bin order)."""
        g = np.zeros((self.derived.ng, self.params.nt), np.float32)
        self._check(self._lib.ose_get_gather(self._h, _f32(g)))
        return g

    def wavefield(self, which: int = FIELD_Q, layout: int = LAYOUT_ZYX) -> np.ndarray:
        d = self.derived
        out = np.zeros(d.nxb * d.nyb * d.nzb, np.float32)
        self._check(self._lib.ose_get_wavefield(self._h, which, _f32(out), layout))
        return out.reshape(self.shape if layout == LAYOUT_ZYX else (d.nyb, d.nxb, d.nzb))

    def set_wavefield(self, which: int, data: np.ndarray, layout: int = LAYOUT_ZYX):
        a = np.ascontiguousarray(data, dtype=np.float32)
        self._check(self._lib.ose_set_wavefield(self._h, which, _f32(a), layout))

    def wavelets(self):
        nt = self.params.nt
        r, h = np.zeros(nt, np.float32), np.zeros(nt, np.float32)
        self._check(self._lib.ose_get_wavelets(self._h, _f32(r), _f32(h)))
        return r, h

    def sponge(self):
        d = self.derived
        ax, ay, az = (np.zeros(n, np.float32) for n in (d.nxb, d.nyb, d.nzb))
        self._check(self._lib.ose_get_sponge(self._h, _f32(ax), _f32(ay), _f32(az)))
        return ax, ay, az

    def set_corrector(self, params: np.ndarray | None, shell: int = CORRECTOR_SHELL):
        """Attach a trained learned-boundary corrector (None detaches)."""
        if params is None:
            self._check(self._lib.ose_set_corrector(self._h, None, shell))
            return
        p = np.ascontiguousarray(params, np.float32)
        self._check(self._lib.ose_set_corrector(self._h, _f32(p), shell))

    def set_receivers(self, xyz):
        """Receivers at explicit interior cells (n x 3 array of x, y, z), or
        None for the receiver plane at depth gzbeg."""
        if xyz is None or len(xyz) == 0:
            self._check(self._lib.ose_set_receivers(self._h, 0, None))
        else:
            a = np.ascontiguousarray(np.asarray(xyz, dtype=np.int32).reshape(-1, 3))
            self._check(self._lib.ose_set_receivers(self._h, a.shape[0],
                                                    a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))))
        self._check(self._lib.ose_get_derived(self._h, ctypes.byref(self.derived)))

    def rtm(self, rows: np.ndarray, every: int = 4):
        """Reverse-time migration of the current shot's observed receiver rows
        ([it][ig], as run_record returns them) with this modeler's velocity;
        returns the padded [z][y][x] image and source illumination."""
        r = np.ascontiguousarray(rows, np.float32)
        img = np.zeros(self.shape, np.float32)
        ill = np.zeros(self.shape, np.float32)
        self._check(self._lib.ose_rtm(self._h, _f32(r), r.shape[0], every, _f32(img), _f32(ill)))
        return img, ill

    def state_box(self, direction: int, box, buf_ptr: int, buf):
        """Copy a box of the state to (direction 0) or from (1) a device
        buffer: box = (x0, y0, z0, nx, ny, nz), buf = (bnx, bny, bx0, by0, bz0)."""
        b = (ctypes.c_int * 6)(*[int(v) for v in box])
        f = (ctypes.c_int * 5)(*[int(v) for v in buf])
        self._check(self._lib.ose_state_box(self._h, direction, b, buf_ptr, f))

    def apply_operator(self, x: np.ndarray) -> np.ndarray:
        """v * IFFT3(|k| FFT3(x)) / (R N) on a complex64 [nzb][nyb][nxb] field."""
        a = np.ascontiguousarray(x, dtype=np.complex64)
        out = np.zeros_like(a)
        self._check(self._lib.ose_apply_operator(self._h, _f32(a.view(np.float32)),
                                                 _f32(out.view(np.float32))))
        return out

    def profile_step(self, reps: int = 1):
        cap = 12
        count = ctypes.c_int()
        names = (ctypes.c_char_p * cap)()
        ms = np.zeros(cap, np.float32)
        by = np.zeros(cap, np.float64)
        launches = (ctypes.c_int * cap)()
        self._check(self._lib.ose_profile_step(self._h, reps, cap, ctypes.byref(count), names,
                                               _f32(ms), by.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                               launches))
        rows = [dict(name=names[i].decode(), ms=float(ms[i]), bytes=float(by[i]),
                     launches_per_step=int(launches[i])) for i in range(count.value)]
        return rows, sum(r["launches_per_step"] for r in rows)

    def checkpoint_save(self, path: str):
        self._check(self._lib.ose_checkpoint_save(self._h, path.encode()))

    def checkpoint_load(self, path: str):
        self._check(self._lib.ose_checkpoint_load(self._h, path.encode()))

    def run_snapshots(self, nsteps: int, every: int, callback, layout: int = LAYOUT_ZYX):
        """nsteps steps; callback(it, P, Q) after every `every` steps with numpy
        copies of the padded P and Q (shape of `layout`)."""
        d = self.derived
        shape = self.shape if layout == LAYOUT_ZYX else (d.nyb, d.nxb, d.nzb)
        n = d.nxb * d.nyb * d.nzb
        errors = []

        def tramp(it, p, q, _user):
            try:
                P = np.ctypeslib.as_array(p, shape=(n,)).copy().reshape(shape)
                Q = np.ctypeslib.as_array(q, shape=(n,)).copy().reshape(shape)
                callback(it, P, Q)
            except Exception as exc:   # keep going; report after the run
                errors.append(exc)

        fn = SNAPSHOT_FN(tramp)
        self._check(self._lib.ose_run_snapshots(self._h, nsteps, every, layout, fn, None))
        if errors:
            raise errors[0]

    def write_su(self, path: str):
        self._check(self._lib.ose_write_su(self._h, path.encode()))

    def write_segy(self, path: str):
        self._check(self._lib.ose_write_segy(self._h, path.encode()))

    def write_outputs(self, gather_path: str | None, par_path: str | None):
        self._check(self._lib.ose_write_outputs(
            self._h, gather_path.encode() if gather_path else None,
            par_path.encode() if par_path else None))
