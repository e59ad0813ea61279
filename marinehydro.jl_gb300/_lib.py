"""ctypes binding of libmarinehydro_cuda.so (the C-ABI in include/marinehydro_gb300.h).

There is no CPU fallback: if the library is missing or no CUDA device is usable,
every entry point raises.  Status codes map onto the exceptions the reference
throws: ``ArgumentError`` -> ``ValueError``, ``SingularException`` ->
``numpy.linalg.LinAlgError``, anything else -> ``MarineHydroError``.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "_build", "libmarinehydro_cuda.so")

MH_OK, MH_ERR_ARG, MH_ERR_UNSUPPORTED, MH_ERR_SINGULAR, MH_ERR_CUDA, MH_ERR_TIMEOUT, MH_ERR_NOT_CONVERGED, \
    MH_ERR_NOMEM = range(8)
MH_MEM_HOST, MH_MEM_DEVICE = 0, 1
MH_PREC_FP64, MH_PREC_MIXED, MH_PREC_FP64_TC = 0, 1, 2

GF_RANKINE = 1
GF_RANKINE_REFLECTED = 2
GF_RANKINE_REFLECTED_NEGATIVE = 4
GF_DELHOMMEAU_RANKINE = 8
GF_DELHOMMEAU_RANKINE_REFLECTED = 16
GF_WU = 32
GF_EXACT_DELHOMMEAU = 64
GF_SURROGATE = 128

# MH_ABI_VERSION of include/marinehydro_gb300.h that these bindings follow
ABI_VERSION = 2

# every symbol the header declares (checked by the CPU test suite)
EXPORTS = (
    "mh_abi_version", "mh_create", "mh_destroy", "mh_last_error", "mh_get_stream", "mh_set_stream",
    "mh_synchronize", "mh_launch_count", "mh_workspace_bytes", "mh_mesh_create", "mh_mesh_destroy",
    "mh_mesh_panels", "mh_mesh_set_lid", "mh_assemble_matrices", "mh_linsolve", "mh_solve", "mh_linsolve_adjoint",
    "mh_hydrodynamic_coefficients", "mh_wu_wave_terms", "mh_bessel01_points", "mh_fixpoint_points", "mh_exact_wave_terms", "mh_set_quadrature_tolerance",
    "mh_profile_enable", "mh_profile_reset", "mh_profile_read", "mh_probe_fma_peaks",
    "mh_assemble_matrices_noalloc", "mh_batch_hydrodynamic_coefficients", "mh_batch_release",
    "mh_hydro_gradient", "mh_surrogate_param_count", "mh_surrogate_train", "mh_surrogate_set",
    "mh_surrogate_wave_terms", "mh_surrogate_loss_grad", "mh_tile_table_set", "mh_tile_table_get", "mh_autotune",
    "mh_probe_wait_timeout", "mh_hydro_frequency_derivative", "mh_hydro_vjp", "mh_solve_pullback",
    "mh_surrogate_set_judge", "mh_surrogate_judge_read",
)


class MarineHydroError(RuntimeError):
    """A CUDA-side failure reported by libmarinehydro_cuda.so."""


_lock = threading.Lock()
_lib = None


def load(path: str | None = None):
    """Load (once) and type the shared library.  Raises if it has not been built."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise MarineHydroError(
                f"{p} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()'); "
                "there is no CPU fallback")
        L = ctypes.CDLL(p)
        vp = ctypes.c_void_p
        i64 = ctypes.c_int64
        D = ctypes.c_double
        I = ctypes.c_int
        u32 = ctypes.c_uint32
        L.mh_abi_version.restype = I
        L.mh_create.argtypes = [I, ctypes.POINTER(vp)]
        L.mh_destroy.argtypes = [vp]
        L.mh_last_error.argtypes = [vp]
        L.mh_last_error.restype = ctypes.c_char_p
        L.mh_get_stream.argtypes = [vp, ctypes.POINTER(vp)]
        L.mh_set_stream.argtypes = [vp, vp]
        L.mh_synchronize.argtypes = [vp]
        L.mh_launch_count.argtypes = [vp]
        L.mh_launch_count.restype = i64
        L.mh_workspace_bytes.argtypes = [vp]
        L.mh_workspace_bytes.restype = i64
        L.mh_mesh_create.argtypes = [vp, i64, vp, vp, vp, vp, vp, I, ctypes.POINTER(vp)]
        L.mh_mesh_destroy.argtypes = [vp]
        L.mh_mesh_panels.argtypes = [vp]
        L.mh_mesh_panels.restype = i64
        L.mh_mesh_set_lid.argtypes = [vp, i64]
        L.mh_assemble_matrices.argtypes = [vp, vp, D, u32, I, I, vp, vp, vp, I]
        L.mh_linsolve.argtypes = [vp, i64, i64, vp, vp, vp, I, I]
        L.mh_linsolve_adjoint.argtypes = [vp, i64, i64, vp, vp, vp, I, I]
        L.mh_solve.argtypes = [vp, i64, i64, vp, vp, vp, I, vp, vp, I, I]
        L.mh_hydrodynamic_coefficients.argtypes = [vp, vp, i64, vp, D, D, u32, I, i64, vp, i64, vp, i64, vp, i64, vp,
                                                   I, vp, vp, vp, vp, vp, I]
        L.mh_wu_wave_terms.argtypes = [vp, i64, vp, vp, vp, I]
        L.mh_bessel01_points.argtypes = [vp, i64, vp, vp, I]
        L.mh_fixpoint_points.argtypes = [vp, i64, vp, vp, I]
        L.mh_exact_wave_terms.argtypes = [vp, i64, vp, vp, D, D, vp, I]
        L.mh_set_quadrature_tolerance.argtypes = [vp, D, D]
        L.mh_profile_enable.argtypes = [vp, I]
        L.mh_profile_reset.argtypes = [vp]
        L.mh_profile_read.argtypes = [vp, i64, vp, vp, vp, ctypes.POINTER(i64)]
        L.mh_probe_fma_peaks.argtypes = [vp, ctypes.POINTER(D), ctypes.POINTER(D)]
        L.mh_batch_hydrodynamic_coefficients.argtypes = [vp, i64, vp, vp, vp, D, D, u32, I, i64, vp, i64, vp, i64,
                                                         vp, i64, vp, I, I, vp, vp, vp, vp, vp, I]
        L.mh_batch_release.argtypes = [vp]
        L.mh_probe_wait_timeout.argtypes = [vp, ctypes.c_uint32]
        L.mh_hydro_vjp.argtypes = [vp, vp, i64, vp, D, D, u32, I, i64, vp, i64, vp, i64, vp, i64, vp, vp, vp, vp, I,
                                   vp, vp, vp, vp, vp, vp, I]
        L.mh_solve_pullback.argtypes = [vp, i64, i64, vp, vp, vp, I, vp, vp, I, vp, vp, vp, vp, vp, I]
        L.mh_surrogate_set_judge.argtypes = [vp, i64, ctypes.c_uint64, D]
        L.mh_surrogate_judge_read.argtypes = [vp, i64, vp, vp]
        L.mh_hydro_frequency_derivative.argtypes = [vp, vp, i64, vp, D, D, u32, I, i64, vp, i64, vp, i64, vp, i64,
                                                    vp] + [vp] * 10 + [I]
        L.mh_tile_table_set.argtypes = [vp, i64, vp, vp]
        L.mh_tile_table_get.argtypes = [vp, i64, vp, vp, vp]
        L.mh_autotune.argtypes = [vp, I, i64, vp, i64, I, vp, vp]
        L.mh_hydro_gradient.argtypes = [vp, vp, i64, vp, D, D, u32, I, i64, vp, i64, vp, I, vp, vp, vp, vp, vp, vp, I]
        L.mh_surrogate_param_count.restype = I
        L.mh_surrogate_train.argtypes = [vp, i64, ctypes.c_uint64, I, I, D, vp, vp]
        L.mh_surrogate_set.argtypes = [vp, vp]
        L.mh_surrogate_wave_terms.argtypes = [vp, i64, vp, vp, vp, I]
        L.mh_surrogate_loss_grad.argtypes = [vp, vp, i64, vp, vp, vp, ctypes.POINTER(D)]
        L.mh_assemble_matrices_noalloc.argtypes = [vp, i64, vp, vp, vp, vp, vp, D, u32, I, I, vp, vp, vp]
        for name in EXPORTS:
            getattr(L, name)  # AttributeError if the build lacks a declared entry point
        if L.mh_abi_version() != ABI_VERSION:
            raise MarineHydroError(f"{p} reports ABI version {L.mh_abi_version()}, these bindings need "
                                   f"{ABI_VERSION}: rebuild the library")
        _lib = L
        return _lib


class Context:
    """One CUDA device, its stream and workspaces (mh_context)."""

    def __init__(self, device: int = 0):
        L = load()
        h = ctypes.c_void_p()
        rc = L.mh_create(int(device), ctypes.byref(h))
        if rc != MH_OK:
            raise MarineHydroError(f"mh_create(device={device}) failed with status {rc}: no usable CUDA device")
        self._h = h
        self.device = device
        self._L = L

    @property
    def handle(self):
        return self._h

    def check(self, rc: int, what: str = ""):
        if rc == MH_OK:
            return
        msg = self._L.mh_last_error(self._h).decode(errors="replace")
        text = f"{what}: {msg}" if what else msg
        if rc in (MH_ERR_ARG, MH_ERR_UNSUPPORTED):
            raise ValueError(text)
        if rc == MH_ERR_SINGULAR:
            raise np.linalg.LinAlgError(text)
        raise MarineHydroError(f"status {rc}: {text}")

    def stream(self) -> int:
        s = ctypes.c_void_p()
        self.check(self._L.mh_get_stream(self._h, ctypes.byref(s)), "mh_get_stream")
        return s.value or 0

    def set_stream(self, stream_ptr: int | None):
        self.check(self._L.mh_set_stream(self._h, ctypes.c_void_p(stream_ptr or 0)), "mh_set_stream")

    def synchronize(self):
        self.check(self._L.mh_synchronize(self._h), "mh_synchronize")

    def launch_count(self) -> int:
        return int(self._L.mh_launch_count(self._h))

    def workspace_bytes(self) -> int:
        return int(self._L.mh_workspace_bytes(self._h))

    def set_quadrature_tolerance(self, rtol: float, atol: float):
        self.check(self._L.mh_set_quadrature_tolerance(self._h, float(rtol), float(atol)), "quadrature tolerance")

    def profile(self, enable: bool = True):
        self.check(self._L.mh_profile_enable(self._h, int(bool(enable))), "mh_profile_enable")

    def profile_reset(self):
        self.check(self._L.mh_profile_reset(self._h), "mh_profile_reset")

    def profile_read(self) -> dict:
        """{kernel group: (total_ms, launches)} recorded since the last reset."""
        cap = 64
        names = ctypes.create_string_buffer(32 * cap)
        ms = (ctypes.c_double * cap)()
        cnt = (ctypes.c_int64 * cap)()
        n = ctypes.c_int64()
        self.check(self._L.mh_profile_read(self._h, cap, names, ms, cnt, ctypes.byref(n)), "mh_profile_read")
        out = {}
        for i in range(min(n.value, cap)):
            nm = names.raw[32 * i:32 * (i + 1)].split(b"\0", 1)[0].decode()
            out[nm] = (ms[i], int(cnt[i]))
        return out

    def surrogate_train(self, n_samples=10_000_000, seed=2026, epochs=8, batch=8192, lr=3e-3):
        """mh_surrogate_train: trains the learned wave-term surrogate on this context's device
        and installs it.  Returns (params float32 array, report dict)."""
        n = int(self._L.mh_surrogate_param_count())
        params = np.empty(n, dtype=np.float32)
        rep = np.zeros(10)
        self.check(self._L.mh_surrogate_train(self._h, int(n_samples), int(seed), int(epochs), int(batch), float(lr),
                                               params.ctypes.data, rep.ctypes.data), "mh_surrogate_train")
        keys = ("final_mse", "rms_rel_err_G", "max_rel_err_G", "wu_rms_rel_err_G", "wu_max_rel_err_G",
                "max_rel_err_dGdr", "wu_max_rel_err_dGdr", "sample_seconds", "train_seconds", "validation_points")
        return params, dict(zip(keys, rep.tolist()))

    def surrogate_set(self, params):
        p = np.ascontiguousarray(np.asarray(params, dtype=np.float32).ravel())
        n = int(self._L.mh_surrogate_param_count())
        if p.size != n:
            raise ValueError(f"the surrogate takes {n} parameters, got {p.size}")
        self.check(self._L.mh_surrogate_set(self._h, p.ctypes.data), "mh_surrogate_set")

    def surrogate_loss_grad(self, params, inputs, targets):
        """Loss and gradient from the training kernels (for checking them)."""
        p = np.ascontiguousarray(np.asarray(params, dtype=np.float32).ravel())
        x = np.ascontiguousarray(np.asarray(inputs, dtype=np.float32).reshape(-1, 2))
        y = np.ascontiguousarray(np.asarray(targets, dtype=np.float32).reshape(-1, 6))
        g = np.empty_like(p)
        loss = ctypes.c_double()
        self.check(self._L.mh_surrogate_loss_grad(self._h, p.ctypes.data, x.shape[0], x.ctypes.data, y.ctypes.data,
                                                  g.ctypes.data, ctypes.byref(loss)), "mh_surrogate_loss_grad")
        return loss.value, g

    def tile_table(self):
        """The launch-shape table: list of (n_max, oz_group, bx_group, cluster_f64, cluster_f32)."""
        n_max = np.zeros(16, dtype=np.int64)
        ch = np.zeros((16, 4), dtype=np.int32)
        cnt = ctypes.c_int64()
        self.check(self._L.mh_tile_table_get(self._h, 16, n_max.ctypes.data, ch.ctypes.data, ctypes.byref(cnt)),
                   "mh_tile_table_get")
        return [(int(n_max[q]),) + tuple(int(x) for x in ch[q]) for q in range(cnt.value)]

    def set_tile_table(self, entries):
        """Install a launch-shape table (entries as returned by tile_table(); [] = defaults)."""
        n_max = np.ascontiguousarray([e[0] for e in entries], dtype=np.int64)
        ch = np.ascontiguousarray([e[1:5] for e in entries], dtype=np.int32).reshape(-1, 4)
        self.check(self._L.mh_tile_table_set(self._h, len(entries), n_max.ctypes.data if len(entries) else None,
                                             ch.ctypes.data if len(entries) else None), "mh_tile_table_set")

    def autotune(self, precision, sizes, batch=16, reps=3):
        """mh_autotune: time the candidate launch shapes of the batched LU for `precision`
        at each order in `sizes` and install the fastest; returns (best ms, default ms)."""
        sz = np.ascontiguousarray(sizes, dtype=np.int64)
        best = np.zeros(sz.size)
        dflt = np.zeros(sz.size)
        self.check(self._L.mh_autotune(self._h, int(precision), sz.size, sz.ctypes.data, int(batch), int(reps),
                                       best.ctypes.data, dflt.ctypes.data), "mh_autotune")
        return best, dflt

    def probe_fma_peaks(self):
        """(fp64, fp32) FMA throughput in TFLOP/s measured on this device."""
        a = ctypes.c_double()
        b = ctypes.c_double()
        self.check(self._L.mh_probe_fma_peaks(self._h, ctypes.byref(a), ctypes.byref(b)), "mh_probe_fma_peaks")
        return a.value, b.value

    def close(self):
        if getattr(self, "_h", None) is not None and self._h.value:
            self._L.mh_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_ctx = {}


def default_context(device: int = 0) -> Context:
    with _lock:
        c = _ctx.get(device)
    if c is None:
        c = Context(device)
        with _lock:
            _ctx[device] = c
    return c


def ptr_and_mem(a):
    """(pointer, memory kind) of a numpy array (host) or an object exposing
    __cuda_array_interface__ (device; e.g. a CUDA torch tensor)."""
    if a is None:
        return None, MH_MEM_HOST
    cai = getattr(a, "__cuda_array_interface__", None)
    if cai is not None:
        return ctypes.c_void_p(cai["data"][0]), MH_MEM_DEVICE
    if isinstance(a, np.ndarray):
        return ctypes.c_void_p(a.ctypes.data), MH_MEM_HOST
    raise TypeError(f"expected a numpy array or a CUDA array, got {type(a)!r}")
