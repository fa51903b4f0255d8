"""dc_gb300 -- Python host side of the GB300-native Fletcher TTI propagator.

The compute path is libdc_gb300.so (hand-written sm_103a CUDA behind a C
ABI declared in include/dc_gb300.h).  This module only binds that ABI with
ctypes:

* ``lib()``            -- the loaded library; raises if it was not built.
* ``Process`` / ``device_data_init`` ... -- the reference's entry points
  (include/device_data.h, include/propagate.h, include/precomp.h,
  include/boundary.h, include/calculate_source.h) with the reference's
  argument meaning, callable from Python the way src/worker.c calls them.
* ``Simulation``       -- the library's own status-returning API
  (dc_gb300_*): graph-captured multi-step runs, fused source, sponge,
  receivers, energy.

There is no CPU fallback: every call that computes goes to the GPU, and a
missing library or device raises ``DcError``.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "libdc_gb300.so"
HEADER = PKG_DIR.parent / "include" / "dc_gb300.h"

OK, ERR_ARG, ERR_CUDA, ERR_NOMEM, ERR_DEVICE, ERR_TIMEOUT, ERR_STATE = range(7)
KERNEL_FAST, KERNEL_EXACT = 0, 1
MEDIUM_PRECOMP, MEDIUM_VPZ_VSV, MEDIUM_PRECOMP_F16, MEDIUM_PRECOMP_BF16 = 0, 1, 2, 3
MAX_LAYERS, MAX_FEATURES = 32, 128

# dc_precomp_vars field order (include/precomp.h:6-17)
COEF_NAMES = ("ch1dxx", "ch1dyy", "ch1dzz", "ch1dxy", "ch1dyz", "ch1dxz",
              "v2px", "v2pz", "v2sz", "v2pn")
ANISO_NAMES = ("theta", "phi", "vsv", "vpz", "epsilon", "delta")


class DcError(RuntimeError):
    """A dc_gb300 call failed (status code + the library's message)."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"dc_gb300 error {code}: {msg}")
        self.code = code


_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)


class PrecompVars(C.Structure):
    _fields_ = [(n, _fp) for n in COEF_NAMES]


class Anisotropy(C.Structure):
    _fields_ = [(n, _fp) for n in ANISO_NAMES]


class ProcessT(C.Structure):
    """dc_process_t, include/dc_process.h:7-21."""
    _fields_ = [
        ("rank", C.c_int),
        ("coordinates", C.c_int * 3),
        ("neighbours", C.c_int * 27),
        ("topology", C.c_int * 3),
        ("iterations", C.c_uint),
        ("source_index", C.c_int),
        ("dx", C.c_float), ("dy", C.c_float), ("dz", C.c_float), ("dt", C.c_float),
        ("sizes", C.c_size_t * 3),
        ("anisotropy_vars", Anisotropy),
        ("precomp_vars", PrecompVars),
        ("pp", _fp), ("pc", _fp), ("qp", _fp), ("qc", _fp),
        ("hostnames", C.c_char_p),
        ("num_workers", C.c_size_t),
    ]


class DeviceData(C.Structure):
    """dc_device_data, include/device_data.h:11-15 (device pointers)."""
    _fields_ = [("pp", _fp), ("pc", _fp), ("qp", _fp), ("qc", _fp),
                ("vpz", _fp), ("vsv", _fp), ("precomp_vars", PrecompVars)]


class Config(C.Structure):
    _fields_ = [("sx", C.c_long), ("sy", C.c_long), ("sz", C.c_long),
                ("dx", C.c_float), ("dy", C.c_float), ("dz", C.c_float), ("dt", C.c_float),
                ("kernel", C.c_int), ("medium", C.c_int), ("device", C.c_int)]


class LayeredSpec(C.Structure):
    _fields_ = [
        ("nlayers", C.c_int),
        ("layer_top", C.c_float * MAX_LAYERS),
        ("vp", C.c_float * MAX_LAYERS),
        ("epsilon", C.c_float * MAX_LAYERS),
        ("delta", C.c_float * MAX_LAYERS),
        ("vp_noise", C.c_float),
        ("theta_lo", C.c_float), ("theta_hi", C.c_float),
        ("phi_lo", C.c_float), ("phi_hi", C.c_float),
        ("sigma_ratio", C.c_float),
        ("n_noise", C.c_int), ("n_theta", C.c_int), ("n_phi", C.c_int),
        ("k_noise", (C.c_float * 4) * MAX_FEATURES),
        ("k_theta", (C.c_float * 4) * MAX_FEATURES),
        ("k_phi", (C.c_float * 4) * MAX_FEATURES),
        ("ox", C.c_long), ("oy", C.c_long), ("oz", C.c_long),
    ]


class BatchConfig(C.Structure):
    _fields_ = [("mx", C.c_long), ("my", C.c_long), ("mz", C.c_long),
                ("dx", C.c_float), ("dy", C.c_float), ("dz", C.c_float), ("dt", C.c_float),
                ("medium", C.c_int), ("device", C.c_int), ("max_steps", C.c_int)]


class Shot(C.Structure):
    _fields_ = [("sx", C.c_long), ("sy", C.c_long), ("sz", C.c_long),
                ("ox", C.c_long), ("oy", C.c_long), ("oz", C.c_long),
                ("src_x", C.c_long), ("src_y", C.c_long), ("src_z", C.c_long),
                ("fcut", C.c_double), ("absorb", C.c_long), ("kappa", C.c_double)]


_sz3 = C.c_size_t * 3
_i3 = C.c_int * 3

# Every entry point declared in include/dc_gb300.h: (name, restype, argtypes)
SIGNATURES = [
    # reference ABI
    ("dc_propagate", None, [C.POINTER(C.c_size_t), C.POINTER(C.c_size_t), C.POINTER(C.c_size_t),
                            C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_void_p,
                            C.c_float, C.c_float, C.c_float, C.c_float]),
    ("dc_device_data_init", C.c_void_p, [C.POINTER(ProcessT)]),
    ("dc_device_data_free", None, [C.c_void_p]),
    ("dc_device_data_get_results", None, [C.POINTER(ProcessT), C.c_void_p]),
    ("dc_device_swap_arrays", None, [C.c_void_p]),
    ("dc_device_add_source", None, [C.c_void_p, C.c_size_t, C.c_float]),
    ("dc_device_extract_halo_face", None, [C.c_void_p, _fp, C.POINTER(C.c_size_t),
                                           C.POINTER(C.c_size_t), C.POINTER(C.c_size_t), _fp]),
    ("dc_device_insert_halo_face", None, [C.c_void_p, _fp, C.POINTER(C.c_size_t),
                                          C.POINTER(C.c_size_t), C.POINTER(C.c_size_t), _fp]),
    ("dc_compute_precomp_vars", PrecompVars, [C.c_int, C.c_int, C.c_int, Anisotropy]),
    ("dc_compute_anisotropy_vars", Anisotropy, [C.c_int, C.c_int, C.c_int]),
    ("dc_free_precomp_vars", None, [C.POINTER(PrecompVars)]),
    ("dc_free_anisotropy_vars", None, [C.POINTER(Anisotropy)]),
    ("randomVelocityBoundaryPartition", None, [C.c_int] * 14 + [_fp, _fp, C.POINTER(C.c_uint)]),
    ("dc_calculate_source", C.c_float, [C.c_float, C.c_int]),
    # library API
    ("dc_gb300_last_error", C.c_char_p, []),
    ("dc_gb300_version", C.c_char_p, []),
    ("dc_gb300_create", C.c_int, [C.POINTER(Config), C.POINTER(C.c_void_p)]),
    ("dc_gb300_destroy", None, [C.c_void_p]),
    ("dc_gb300_device_data", C.c_void_p, [C.c_void_p]),
    ("dc_gb300_from_device_data", C.c_void_p, [C.c_void_p]),
    ("dc_gb300_device_pitch", C.c_long, [C.c_void_p]),
    ("dc_gb300_set_precomp", C.c_int, [C.c_void_p, C.POINTER(PrecompVars)]),
    ("dc_gb300_set_vpz_vsv", C.c_int, [C.c_void_p, _fp, _fp]),
    ("dc_gb300_set_anisotropy", C.c_int, [C.c_void_p, C.POINTER(Anisotropy)]),
    ("dc_gb300_get_precomp", C.c_int, [C.c_void_p, C.POINTER(PrecompVars)]),
    ("dc_gb300_get_vpz_vsv", C.c_int, [C.c_void_p, _fp, _fp]),
    ("dc_gb300_generate_layered", C.c_int, [C.c_void_p, C.POINTER(LayeredSpec)]),
    ("dc_gb300_generate_reference", C.c_int, [C.c_void_p, C.c_long, C.c_long, C.c_long,
                                              C.c_long, C.c_uint]),
    ("dc_gb300_set_fields", C.c_int, [C.c_void_p, _fp, _fp, _fp, _fp]),
    ("dc_gb300_get_fields", C.c_int, [C.c_void_p, _fp, _fp, _fp, _fp]),
    ("dc_gb300_set_source", C.c_int, [C.c_void_p, C.c_long, _fp, C.c_int]),
    ("dc_gb300_set_sponge", C.c_int, [C.c_void_p, _fp, _fp, _fp]),
    ("dc_gb300_set_receivers", C.c_int, [C.c_void_p, C.POINTER(C.c_long), C.c_int, C.c_int]),
    ("dc_gb300_get_traces", C.c_int, [C.c_void_p, _fp, C.c_int]),
    ("dc_gb300_enable_energy", C.c_int, [C.c_void_p, C.c_int]),
    ("dc_gb300_get_energy", C.c_int, [C.c_void_p, _dp, C.c_int]),
    ("dc_gb300_run", C.c_int, [C.c_void_p, C.c_int]),
    ("dc_gb300_synchronize", C.c_int, [C.c_void_p]),
    ("dc_gb300_steps_done", C.c_long, [C.c_void_p]),
    ("dc_gb300_propagate_box", C.c_int, [C.c_void_p, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]),
    ("dc_gb300_save_checkpoint", C.c_int, [C.c_void_p, C.c_char_p]),
    ("dc_gb300_load_checkpoint", C.c_int, [C.c_void_p, C.c_char_p]),
    ("dc_gb300_kernel_launches", C.c_long, [C.c_void_p]),
    ("dc_gb300_stream", C.c_void_p, [C.c_void_p]),
    ("dc_gb300_batch_create", C.c_int, [C.POINTER(BatchConfig), C.POINTER(C.c_void_p)]),
    ("dc_gb300_batch_destroy", C.c_int, [C.c_void_p]),
    ("dc_gb300_batch_generate_layered", C.c_int, [C.c_void_p, C.POINTER(LayeredSpec)]),
    ("dc_gb300_batch_set_precomp", C.c_int, [C.c_void_p, C.POINTER(PrecompVars)]),
    ("dc_gb300_batch_add_shot", C.c_int, [C.c_void_p, C.POINTER(Shot), C.POINTER(C.c_int)]),
    ("dc_gb300_batch_set_receivers", C.c_int,
     [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_long)]),
    ("dc_gb300_batch_set_learned_layer", C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    ("dc_gb300_batch_set_tiles", C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    ("dc_gb300_batch_tiles", C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("dc_gb300_batch_set_grid", C.c_int, [C.c_void_p, C.c_int]),
    ("dc_gb300_batch_grid", C.c_int, [C.c_void_p]),
    ("dc_gb300_batch_autotune", C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_int),
                                          C.POINTER(C.c_int), _fp]),
    ("dc_gb300_batch_run", C.c_int, [C.c_void_p, C.c_int]),
    ("dc_gb300_batch_synchronize", C.c_int, [C.c_void_p]),
    ("dc_gb300_batch_get_fields", C.c_int, [C.c_void_p, C.c_int, _fp, _fp, _fp, _fp]),
    ("dc_gb300_batch_get_traces", C.c_int, [C.c_void_p, C.c_int, C.c_int, _fp]),
    ("dc_gb300_batch_steps_done", C.c_int, [C.c_void_p]),
    ("dc_gb300_batch_kernel_launches", C.c_long, [C.c_void_p]),
    ("dc_gb300_batch_stream", C.c_void_p, [C.c_void_p]),
    ("dc_gb300_batch_points", C.c_longlong, [C.c_void_p]),
    ("dc_gb300_mlp_create", C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    ("dc_gb300_mlp_destroy", C.c_int, [C.c_void_p]),
    ("dc_gb300_mlp_init", C.c_int, [C.c_void_p, C.c_uint]),
    ("dc_gb300_mlp_set_params", C.c_int, [C.c_void_p, _fp]),
    ("dc_gb300_mlp_get_params", C.c_int, [C.c_void_p, _fp]),
    ("dc_gb300_mlp_device_params", C.c_void_p, [C.c_void_p]),
    ("dc_gb300_mlp_forward", C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong, C.c_void_p]),
    ("dc_gb300_mlp_gradient", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong, _fp,
                                        _dp]),
    ("dc_gb300_mlp_train", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_longlong, C.c_int,
                                     C.c_int, C.c_float, C.c_ulonglong, _fp]),
    ("dc_gb300_layer_cells", C.c_longlong, [C.c_long, C.c_long, C.c_long, C.c_int,
                                           C.POINTER(C.c_int), C.c_longlong]),
    ("dc_gb300_layer_plan", C.c_int, [C.c_long, C.c_long, C.c_long, C.c_int,
                                      C.POINTER(C.c_int), C.c_longlong, C.POINTER(C.c_int),
                                      C.c_longlong, C.POINTER(C.c_longlong),
                                      C.POINTER(C.c_longlong)]),
    ("dc_gb300_set_learned_layer",C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    ("dc_gb300_lb_sample", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_long), C.c_int,
                                     C.c_void_p, C.c_void_p, C.c_longlong,
                                     C.POINTER(C.c_longlong)]),
    ("dc_gb300_lb_rollout", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_long), C.c_int,
                                      C.c_void_p, C.c_void_p, C.c_longlong,
                                      C.POINTER(C.c_longlong)]),
    ("dc_gb300_exact_steps_noalloc", C.c_int,
     [C.c_void_p, C.POINTER(C.c_void_p), C.c_void_p, C.c_int, _dp, C.c_void_p]),
    ("dc_gb300_source", C.c_float, [C.c_float, C.c_int, C.c_double]),
    ("dc_gb300_sponge_profile", None, [C.c_long, C.c_long, C.c_double, _fp]),
]

_LIB = None


def build(force: bool = False) -> Path:
    from importlib import util
    spec = util.spec_from_file_location("_dc_gb300_build", PKG_DIR / "build.py")
    mod = util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(force=force)


def lib() -> C.CDLL:
    """The loaded libdc_gb300.so.  Raises DcError if it has not been built."""
    global _LIB
    if _LIB is None:
        if not LIB_PATH.exists():
            raise DcError(ERR_STATE, f"{LIB_PATH.name} is not built; call build() first")
        L = C.CDLL(str(LIB_PATH))
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def last_error() -> str:
    msg = lib().dc_gb300_last_error()
    return msg.decode() if msg else ""


def check(code: int) -> None:
    if code != OK:
        raise DcError(code, last_error())


def fptr(a: np.ndarray | None):
    if a is None:
        return None
    if a.dtype != np.float32 or not a.flags.c_contiguous:
        raise TypeError("expected a C-contiguous float32 array")
    return a.ctypes.data_as(_fp)


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float32)


# ---------------------------------------------------------------------------
# The reference's entry points
# ---------------------------------------------------------------------------

class Process:
    """Owns a dc_process_t and the numpy arrays it points at (the state that
    src/main.c:146-172 builds for one rank).  Arrays are shape (sz, sy, sx).
    """

    def __init__(self, sizes, d=(1.0, 1.0, 1.0), dt=1.0, pp=None, pc=None, qp=None, qc=None,
                 anisotropy=None, precomp=None, iterations=0, source_index=-1):
        sx, sy, sz = (int(v) for v in sizes)
        shape = (sz, sy, sx)
        self.shape = shape
        self._keep = {}
        p = ProcessT()
        p.rank = 0
        p.topology[:] = [1, 1, 1]
        p.iterations = iterations
        p.source_index = source_index
        p.dx, p.dy, p.dz = d
        p.dt = dt
        p.sizes[:] = [sx, sy, sz]
        for name, arr in (("pp", pp), ("pc", pc), ("qp", qp), ("qc", qc)):
            a = _f32(arr if arr is not None else np.zeros(shape, np.float32)).reshape(shape).copy()
            self._keep[name] = a
            setattr(p, name, fptr(a))
        if anisotropy is not None:
            # names left out stay NULL (the vpz/vsv medium reads only those two)
            for n in ANISO_NAMES:
                if anisotropy.get(n) is None:
                    continue
                a = _f32(anisotropy[n]).reshape(shape)
                self._keep["a_" + n] = a
                setattr(p.anisotropy_vars, n, fptr(a))
        if precomp is not None:
            for n, arr in zip(COEF_NAMES, precomp):
                a = _f32(arr).reshape(shape)
                self._keep["c_" + n] = a
                setattr(p.precomp_vars, n, fptr(a))
        p.num_workers = 1
        self.proc = p

    def field(self, name: str) -> np.ndarray:
        return self._keep[name]


def device_data_init(process: Process) -> int:
    """dc_device_data_init; returns the dc_device_data* as an int."""
    return lib().dc_device_data_init(C.byref(process.proc))


def device_data_free(data: int) -> None:
    lib().dc_device_data_free(data)


def device_data_get_results(process: Process, data: int) -> None:
    lib().dc_device_data_get_results(C.byref(process.proc), data)


def device_swap_arrays(data: int) -> None:
    lib().dc_device_swap_arrays(data)


def device_add_source(data: int, index: int, source: float) -> None:
    lib().dc_device_add_source(data, index, source)


def propagate(start, end, sizes, data: int, dx, dy, dz, dt, process_coordinates=(0, 0, 0),
              topology=(1, 1, 1)) -> None:
    """dc_propagate over the half-open box [start, end)."""
    lib().dc_propagate(_sz3(*start), _sz3(*end), _sz3(*sizes), _i3(*process_coordinates),
                       _i3(*topology), data, dx, dy, dz, dt)


def device_view(data: int) -> DeviceData:
    return DeviceData.from_address(data)


def extract_halo_face(data: int, start, end, sizes, from_array) -> np.ndarray:
    w = [int(e) - int(s) for s, e in zip(start, end)]
    buf = np.zeros((w[2], w[1], w[0]), np.float32)
    lib().dc_device_extract_halo_face(data, fptr(buf), _sz3(*start), _sz3(*end), _sz3(*sizes),
                                      from_array)
    return buf


def insert_halo_face(data: int, buffer: np.ndarray, start, end, sizes, to_array) -> None:
    buf = _f32(buffer)
    lib().dc_device_insert_halo_face(data, fptr(buf), _sz3(*start), _sz3(*end), _sz3(*sizes),
                                     to_array)


def compute_anisotropy_vars(sizes) -> dict:
    """dc_compute_anisotropy_vars, copied into numpy (arrays freed)."""
    sx, sy, sz = sizes
    a = lib().dc_compute_anisotropy_vars(sx, sy, sz)
    n = sx * sy * sz
    out = {k: np.ctypeslib.as_array(getattr(a, k), (n,)).reshape(sz, sy, sx).copy()
           for k in ANISO_NAMES}
    lib().dc_free_anisotropy_vars(C.byref(a))
    return out


def compute_precomp_vars(sizes, aniso: dict) -> list[np.ndarray]:
    """dc_compute_precomp_vars (FP64 trig on the GPU), as numpy arrays in
    dc_precomp_vars order."""
    sx, sy, sz = sizes
    keep = {k: _f32(aniso[k]) for k in ANISO_NAMES}
    a = Anisotropy(*[fptr(keep[k]) for k in ANISO_NAMES])
    v = lib().dc_compute_precomp_vars(sx, sy, sz, a)
    n = sx * sy * sz
    out = [np.ctypeslib.as_array(getattr(v, k), (n,)).reshape(sz, sy, sx).copy()
           for k in COEF_NAMES]
    lib().dc_free_precomp_vars(C.byref(v))
    return out


def random_velocity_boundary(local, glob, start, n, bord, absorb, vpz, vsv, seed=0) -> int:
    s = C.c_uint(seed)
    lib().randomVelocityBoundaryPartition(*local, *glob, *start, *n, bord, absorb, fptr(vpz),
                                          fptr(vsv), C.byref(s))
    return s.value


def calculate_source(dt: float, it: int) -> float:
    return float(lib().dc_calculate_source(dt, it))


def source(dt: float, it: int, fcut: float = 40.0) -> float:
    return float(lib().dc_gb300_source(dt, it, fcut))


def source_table(dt: float, steps: int, fcut: float = 40.0) -> np.ndarray:
    return np.array([source(dt, i, fcut) for i in range(steps)], np.float32)


def sponge_profile(s: int, a: int, kappa: float) -> np.ndarray:
    g = np.empty(s, np.float32)
    lib().dc_gb300_sponge_profile(s, a, kappa, fptr(g))
    return g


# ---------------------------------------------------------------------------
# The library's own API
# ---------------------------------------------------------------------------

class Simulation:
    """One propagator on one GPU (dc_gb300_create ... dc_gb300_destroy)."""

    def __init__(self, sizes, d=(12.5, 12.5, 12.5), dt=1e-3, kernel=KERNEL_FAST,
                 medium=MEDIUM_PRECOMP, device=-1):
        self.sizes = tuple(int(v) for v in sizes)
        sx, sy, sz = self.sizes
        self.shape = (sz, sy, sx)
        cfg = Config(sx, sy, sz, d[0], d[1], d[2], dt, kernel, medium, device)
        h = C.c_void_p()
        check(lib().dc_gb300_create(C.byref(cfg), C.byref(h)))
        self.h = h.value
        self.kernel = kernel
        self.medium = medium
        self.nrec = 0

    def close(self):
        if getattr(self, "h", None):
            lib().dc_gb300_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # medium ------------------------------------------------------------------
    def set_precomp(self, coef) -> None:
        keep = [_f32(c).reshape(self.shape) for c in coef]
        pv = PrecompVars(*[fptr(c) for c in keep])
        check(lib().dc_gb300_set_precomp(self.h, C.byref(pv)))

    def set_vpz_vsv(self, vpz, vsv) -> None:
        a, b = _f32(vpz), _f32(vsv)
        check(lib().dc_gb300_set_vpz_vsv(self.h, fptr(a), fptr(b)))

    def set_anisotropy(self, aniso: dict) -> None:
        keep = {k: _f32(aniso[k]).reshape(self.shape) for k in ANISO_NAMES}
        a = Anisotropy(*[fptr(keep[k]) for k in ANISO_NAMES])
        check(lib().dc_gb300_set_anisotropy(self.h, C.byref(a)))

    def get_precomp(self, out=None) -> list[np.ndarray]:
        """The device coefficients as dense arrays (dc_precomp_vars order);
        ``out`` may supply the ten destination arrays (e.g. pinned)."""
        out = out if out is not None else [np.empty(self.shape, np.float32) for _ in range(10)]
        pv = PrecompVars(*[fptr(a) for a in out])
        check(lib().dc_gb300_get_precomp(self.h, C.byref(pv)))
        return out

    def get_vpz_vsv(self):
        a, b = np.empty(self.shape, np.float32), np.empty(self.shape, np.float32)
        check(lib().dc_gb300_get_vpz_vsv(self.h, fptr(a), fptr(b)))
        return a, b

    def generate_reference(self, n, absorb: int, seed: int = 0) -> None:
        """The reference's default medium + random velocity boundary +
        precompute, on the GPU (sizes must be n + 2*absorb + 8)."""
        check(lib().dc_gb300_generate_reference(self.h, int(n[0]), int(n[1]), int(n[2]),
                                                int(absorb), int(seed)))

    def generate_layered(self, spec: LayeredSpec) -> None:
        check(lib().dc_gb300_generate_layered(self.h, C.byref(spec)))

    # fields ----------------------------------------------------------------
    def set_fields(self, pp=None, pc=None, qp=None, qc=None) -> None:
        arrs = [None if a is None else _f32(a).reshape(self.shape) for a in (pp, pc, qp, qc)]
        check(lib().dc_gb300_set_fields(self.h, *[fptr(a) for a in arrs]))

    def get_fields(self):
        out = [np.empty(self.shape, np.float32) for _ in range(4)]
        check(lib().dc_gb300_get_fields(self.h, *[fptr(a) for a in out]))
        return dict(zip(("pp", "pc", "qp", "qc"), out))

    def get_pc(self) -> np.ndarray:
        """The current p field alone (dense)."""
        out = np.empty(self.shape, np.float32)
        check(lib().dc_gb300_get_fields(self.h, None, fptr(out), None, None))
        return out

    def set_source(self, index: int, amplitudes) -> None:
        if index is None or index < 0:
            check(lib().dc_gb300_set_source(self.h, -1, None, 0))
            return
        a = _f32(amplitudes)
        check(lib().dc_gb300_set_source(self.h, int(index), fptr(a), int(a.size)))

    def set_sponge(self, gx=None, gy=None, gz=None) -> None:
        if gx is None:
            check(lib().dc_gb300_set_sponge(self.h, None, None, None))
            return
        g = [_f32(v) for v in (gx, gy, gz)]
        check(lib().dc_gb300_set_sponge(self.h, *[fptr(v) for v in g]))

    def set_receivers(self, index, max_steps: int) -> None:
        idx = np.ascontiguousarray(index, np.int64)
        arr = (C.c_long * max(1, idx.size))(*idx.tolist())
        check(lib().dc_gb300_set_receivers(self.h, arr, int(idx.size), int(max_steps)))
        self.nrec = int(idx.size)

    def traces(self, steps: int) -> np.ndarray:
        out = np.empty((steps, self.nrec), np.float32)
        check(lib().dc_gb300_get_traces(self.h, fptr(out), steps))
        return out

    def enable_energy(self, max_steps: int) -> None:
        check(lib().dc_gb300_enable_energy(self.h, int(max_steps)))

    def energy(self, steps: int) -> np.ndarray:
        out = np.empty(steps, np.float64)
        check(lib().dc_gb300_get_energy(self.h, out.ctypes.data_as(_dp), steps))
        return out

    # time loop ---------------------------------------------------------------
    def run(self, steps: int) -> None:
        check(lib().dc_gb300_run(self.h, int(steps)))

    def synchronize(self) -> None:
        check(lib().dc_gb300_synchronize(self.h))

    def propagate_box(self, start, end) -> None:
        check(lib().dc_gb300_propagate_box(self.h, _sz3(*start), _sz3(*end)))

    def save_checkpoint(self, path) -> None:
        check(lib().dc_gb300_save_checkpoint(self.h, str(path).encode()))

    def load_checkpoint(self, path) -> None:
        check(lib().dc_gb300_load_checkpoint(self.h, str(path).encode()))

    @property
    def steps_done(self) -> int:
        return int(lib().dc_gb300_steps_done(self.h))

    @property
    def launches(self) -> int:
        return int(lib().dc_gb300_kernel_launches(self.h))

    @property
    def stream(self) -> int:
        return int(lib().dc_gb300_stream(self.h) or 0)

    @property
    def pitch(self) -> int:
        return int(lib().dc_gb300_device_pitch(self.h))

    @property
    def device_data(self) -> int:
        return int(lib().dc_gb300_device_data(self.h))


class Batch:
    """Shots cropped out of one shared medium, advanced together
    (dc_gb300_batch_create ... dc_gb300_batch_destroy).

    ``medium_sizes`` are the medium box's (mx, my, mz); a shot is
    ``add_shot(sizes, origin, src, fcut, absorb, kappa)`` with its padded box
    sizes, the medium position of its point (0, 0, 0) (x a multiple of 4) and
    its source in box coordinates."""

    def __init__(self, medium_sizes, d=(12.5, 12.5, 12.5), dt=1e-3, medium=MEDIUM_PRECOMP,
                 device=-1, max_steps=1000):
        self.medium_sizes = tuple(int(v) for v in medium_sizes)
        cfg = BatchConfig(*self.medium_sizes, d[0], d[1], d[2], dt, medium, device,
                          int(max_steps))
        h = C.c_void_p()
        check(lib().dc_gb300_batch_create(C.byref(cfg), C.byref(h)))
        self.h = h.value
        self.shots = []
        self.nrec = []

    def close(self):
        if getattr(self, "h", None):
            lib().dc_gb300_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def generate_layered(self, spec: LayeredSpec) -> None:
        check(lib().dc_gb300_batch_generate_layered(self.h, C.byref(spec)))

    def set_precomp(self, coef) -> None:
        mx, my, mz = self.medium_sizes
        keep = [_f32(c).reshape(mz, my, mx) for c in coef]
        pv = PrecompVars(*[fptr(c) for c in keep])
        check(lib().dc_gb300_batch_set_precomp(self.h, C.byref(pv)))

    def add_shot(self, sizes, origin, src, fcut=40.0, absorb=0, kappa=0.0) -> int:
        sh = Shot(*[int(v) for v in sizes], *[int(v) for v in origin], *[int(v) for v in src],
                  float(fcut), int(absorb), float(kappa))
        idx = C.c_int(-1)
        check(lib().dc_gb300_batch_add_shot(self.h, C.byref(sh), C.byref(idx)))
        self.shots.append(tuple(int(v) for v in sizes))
        self.nrec.append(0)
        return idx.value

    def set_receivers(self, shot: int, xyz) -> None:
        a = np.ascontiguousarray(xyz, np.int64).reshape(-1, 3)
        arr = (C.c_long * max(1, a.size))(*a.reshape(-1).tolist())
        check(lib().dc_gb300_batch_set_receivers(self.h, int(shot), int(a.shape[0]), arr))
        self.nrec[shot] = int(a.shape[0])

    def set_learned_layer(self, mlp: "MLP | None", layer: int) -> None:
        """Every shot reads the network at every step: the batch keeps a
        reference to ``mlp`` for as long as the layer is set."""
        check(lib().dc_gb300_batch_set_learned_layer(self.h, mlp.h if mlp is not None else None,
                                                     int(layer)))
        self._mlp = mlp if layer > 0 else None

    def set_tiles(self, ty: int, zsplit: int) -> None:
        check(lib().dc_gb300_batch_set_tiles(self.h, int(ty), int(zsplit)))

    def tiles(self):
        ty, zs = C.c_int(), C.c_int()
        check(lib().dc_gb300_batch_tiles(self.h, C.byref(ty), C.byref(zs)))
        return ty.value, zs.value

    def set_grid(self, persistent: bool) -> None:
        check(lib().dc_gb300_batch_set_grid(self.h, 1 if persistent else 0))

    @property
    def persistent(self) -> bool:
        return lib().dc_gb300_batch_grid(self.h) == 1

    def autotune(self, steps: int = 4):
        """(ty, zsplit, ms per step) of the fastest tile candidate; leaves
        the batch at step 0 with zero wavefields."""
        ty, zs, ms = C.c_int(), C.c_int(), C.c_float()
        check(lib().dc_gb300_batch_autotune(self.h, int(steps), C.byref(ty), C.byref(zs),
                                            C.byref(ms)))
        return ty.value, zs.value, ms.value

    def run(self, steps: int) -> None:
        check(lib().dc_gb300_batch_run(self.h, int(steps)))

    def synchronize(self) -> None:
        check(lib().dc_gb300_batch_synchronize(self.h))

    def get_fields(self, shot: int):
        sx, sy, sz = self.shots[shot]
        out = [np.empty((sz, sy, sx), np.float32) for _ in range(4)]
        check(lib().dc_gb300_batch_get_fields(self.h, int(shot), *[fptr(a) for a in out]))
        return dict(zip(("pp", "pc", "qp", "qc"), out))

    def traces(self, shot: int, steps: int) -> np.ndarray:
        out = np.empty((steps, self.nrec[shot]), np.float32)
        check(lib().dc_gb300_batch_get_traces(self.h, int(shot), int(steps), fptr(out)))
        return out

    @property
    def steps_done(self) -> int:
        return int(lib().dc_gb300_batch_steps_done(self.h))

    @property
    def launches(self) -> int:
        return int(lib().dc_gb300_batch_kernel_launches(self.h))

    @property
    def stream(self) -> int:
        return int(lib().dc_gb300_batch_stream(self.h) or 0)

    @property
    def points(self) -> int:
        return int(lib().dc_gb300_batch_points(self.h))


MLP_PARAMS = 32 * 32 + 16 * 32 + 32 * 32 + 32 + 2 * 32 + 2
MLP_DEPTHS = 16
SAMPLE_STRIDE = 33


class MLP:
    """The learned layer's network (dc_gb300_mlp_*).  Sample and target
    arrays are device pointers (ints), e.g. torch tensors' data_ptr()."""

    def __init__(self, device=-1, seed=None, params=None):
        h = C.c_void_p()
        check(lib().dc_gb300_mlp_create(int(device), C.byref(h)))
        self.h = h.value
        if params is not None:
            self.set_params(params)
        elif seed is not None:
            check(lib().dc_gb300_mlp_init(self.h, int(seed)))

    def close(self):
        if getattr(self, "h", None):
            lib().dc_gb300_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_params(self, params) -> None:
        a = _f32(params).reshape(-1)
        if a.size != MLP_PARAMS:
            raise ValueError(f"expected {MLP_PARAMS} parameters")
        check(lib().dc_gb300_mlp_set_params(self.h, fptr(a)))

    def params(self) -> np.ndarray:
        out = np.empty(MLP_PARAMS, np.float32)
        check(lib().dc_gb300_mlp_get_params(self.h, fptr(out)))
        return out

    def forward(self, samples_ptr: int, n: int, out_ptr: int) -> None:
        check(lib().dc_gb300_mlp_forward(self.h, samples_ptr, int(n), out_ptr))

    def gradient(self, samples_ptr: int, targets_ptr: int, n: int):
        g = np.empty(MLP_PARAMS, np.float32)
        loss = (C.c_double * 2)()
        check(lib().dc_gb300_mlp_gradient(self.h, samples_ptr, targets_ptr, int(n), fptr(g), loss))
        return g, (loss[0], loss[1])

    def train(self, samples_ptr: int, targets_ptr: int, n: int, steps: int, batch: int,
              lr: float, seed: int = 0) -> np.ndarray:
        hist = np.empty(max(1, steps), np.float32)
        check(lib().dc_gb300_mlp_train(self.h, samples_ptr, targets_ptr, int(n), int(steps),
                                       int(batch), float(lr), int(seed), fptr(hist)))
        return hist[:steps]


def layer_cells(sizes, layer: int) -> np.ndarray:
    """[n][4] table (x, y, z, axis | side << 2 | depth << 3) of the layer cells."""
    n = lib().dc_gb300_layer_cells(*[int(v) for v in sizes], int(layer), None, 0)
    if n < 0:
        raise DcError(ERR_ARG, last_error())
    out = np.empty((n, 4), np.int32)
    lib().dc_gb300_layer_cells(*[int(v) for v in sizes], int(layer),
                               out.ctypes.data_as(C.POINTER(C.c_int)), n)
    return out


def layer_plan(sizes, layer: int):
    """(lines, edge): the face lines ([n][4]: x, y, z of the outermost cell,
    axis | side << 2), corrected in place by one fused pass, and the edge
    cells ([m][4], ``layer_cells`` entries), corrected through a buffer."""
    nl, ne = C.c_longlong(), C.c_longlong()
    dims = [int(v) for v in sizes]
    check(lib().dc_gb300_layer_plan(*dims, int(layer), None, 0, None, 0, C.byref(nl),
                                    C.byref(ne)))
    lines = np.empty((nl.value, 4), np.int32)
    edge = np.empty((ne.value, 4), np.int32)
    ip = C.POINTER(C.c_int)
    check(lib().dc_gb300_layer_plan(*dims, int(layer), lines.ctypes.data_as(ip), nl.value,
                                    edge.ctypes.data_as(ip), ne.value, C.byref(nl), C.byref(ne)))
    return lines, edge


def set_learned_layer(sim: "Simulation", mlp: "MLP | None", layer: int) -> None:
    """The simulation reads the network's parameters at every step: it keeps
    a reference to ``mlp`` for as long as the layer is set."""
    check(lib().dc_gb300_set_learned_layer(sim.h, mlp.h if mlp is not None else None, int(layer)))
    sim._mlp = mlp if layer > 0 else None


def lb_sample(wide: "Simulation", thin: "Simulation", offset, layer: int, samples_ptr: int,
              targets_ptr: int, cap: int) -> int:
    n = C.c_longlong()
    check(lib().dc_gb300_lb_sample(wide.h, thin.h, (C.c_long * 3)(*[int(v) for v in offset]),
                                   int(layer), samples_ptr, targets_ptr, int(cap), C.byref(n)))
    return n.value


def lb_rollout(wide: "Simulation", thin: "Simulation", offset, steps: int, samples_ptr: int,
               targets_ptr: int, cap: int) -> int:
    n = C.c_longlong()
    check(lib().dc_gb300_lb_rollout(wide.h, thin.h, (C.c_long * 3)(*[int(v) for v in offset]),
                                    int(steps), samples_ptr, targets_ptr, int(cap), C.byref(n)))
    return n.value


def header_symbols() -> list[str]:
    """Function names declared in include/dc_gb300.h."""
    import re
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\(", text)
    skip = {"if", "sizeof", "defined", "struct"}
    return sorted({n for n in names if n not in skip and (n.startswith("dc_") or n == "randomVelocityBoundaryPartition")})
