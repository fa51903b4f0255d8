"""ctypes bindings for the CPU oracle (TEST INFRASTRUCTURE ONLY).

``Port`` wraps our C restatement (oracle/dc_oracle.c); ``Reference`` wraps
the reference's own sources compiled into oracle/_ref/ (present only where
the reference checkout or its staged copy exists).  Only tests/, the smoke check and
bench.py's CPU-baseline leg import this module -- it is the checker, never
the product.

Arrays are numpy, x fastest, shape (sz, sy, sx) C-order, i.e. index
``x + y*sx + z*sx*sy`` as in the reference (include/indexing.h:15-21).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

from . import build_oracle

NCOEF = 10
COEF_NAMES = ("ch1dxx", "ch1dyy", "ch1dzz", "ch1dxy", "ch1dyz", "ch1dxz",
              "v2px", "v2pz", "v2sz", "v2pn")
KIND_F32, KIND_F32_REFCUDA, KIND_F64, KIND_F64_SEP = 0, 1, 2, 3
STORE_F32, STORE_F16, STORE_BF16 = 0, 1, 2

_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)
_lp = C.POINTER(C.c_long)


def _f(a):
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(_fp)


def _vp(a):
    assert a.flags.c_contiguous
    return C.c_void_p(a.ctypes.data)


class _RunCfg(C.Structure):
    _fields_ = [
        ("kind", C.c_int),
        ("sx", C.c_long), ("sy", C.c_long), ("sz", C.c_long),
        ("dx", C.c_float), ("dy", C.c_float), ("dz", C.c_float), ("dt", C.c_float),
        ("steps", C.c_int),
        ("src_index", C.c_long),
        ("src", _fp),
        ("coef", _fp * NCOEF),
        ("vpz", _fp), ("vsv", _fp),
        ("sponge", _fp * 3),
        ("nrec", C.c_long),
        ("rec", _lp),
        ("traces", _dp),
        ("energy", _dp),
        ("nthreads", C.c_int),
        ("store", C.c_int),
        ("store_exp", C.c_int * 2),
    ]


@dataclass
class RunResult:
    pp: np.ndarray
    pc: np.ndarray
    qp: np.ndarray
    qc: np.ndarray
    traces: np.ndarray | None = None
    energy: np.ndarray | None = None


def default_threads() -> int:
    return max(1, os.cpu_count() or 1)


class Port:
    """Our C restatement of the reference path."""

    def __init__(self):
        so = build_oracle.build_port()
        lib = C.CDLL(str(so))
        lib.o_default_anisotropy.argtypes = [C.c_long] + [_fp] * 6
        lib.o_precomp.argtypes = [C.c_long] + [_fp] * 6 + [_fp * NCOEF]
        lib.o_random_velocity_boundary.argtypes = [C.c_int] * 14 + [_fp, _fp, C.POINTER(C.c_uint)]
        lib.o_source.argtypes = [C.c_float, C.c_int, C.c_double]
        lib.o_source.restype = C.c_float
        lib.o_sponge_profile.argtypes = [C.c_long, C.c_long, C.c_double, _fp]
        lib.o_step.argtypes = [C.c_int, C.c_long, C.c_long, C.c_long, _lp, _lp,
                               C.c_float, C.c_float, C.c_float, C.c_float,
                               C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                               _fp * NCOEF, _fp, _fp, C.c_void_p, C.c_int]
        lib.o_step.restype = C.c_int
        lib.o_run.argtypes = [C.POINTER(_RunCfg)] + [C.c_void_p] * 4
        lib.o_run.restype = C.c_int
        self.lib = lib

    # ---- medium ----------------------------------------------------------
    def default_anisotropy(self, shape):
        n = int(np.prod(shape))
        arrs = {k: np.empty(shape, np.float32) for k in ("vpz", "vsv", "epsilon", "delta", "phi", "theta")}
        self.lib.o_default_anisotropy(n, _f(arrs["vpz"]), _f(arrs["vsv"]), _f(arrs["epsilon"]),
                                      _f(arrs["delta"]), _f(arrs["phi"]), _f(arrs["theta"]))
        return arrs

    def precomp(self, aniso) -> list[np.ndarray]:
        shape = aniso["vpz"].shape
        n = int(np.prod(shape))
        out = [np.empty(shape, np.float32) for _ in range(NCOEF)]
        arr = (_fp * NCOEF)(*[_f(o) for o in out])
        self.lib.o_precomp(n, _f(aniso["theta"]), _f(aniso["phi"]), _f(aniso["vsv"]),
                           _f(aniso["vpz"]), _f(aniso["epsilon"]), _f(aniso["delta"]), arr)
        return out

    def random_velocity_boundary(self, local, glob, start, n, bord, absorb, vpz, vsv, seed=0):
        s = C.c_uint(seed)
        self.lib.o_random_velocity_boundary(*local, *glob, *start, *n, bord, absorb,
                                            _f(vpz), _f(vsv), C.byref(s))
        return s.value

    def source(self, dt, it, fcut=40.0) -> float:
        return float(self.lib.o_source(dt, it, fcut))

    def source_table(self, dt, steps, fcut=40.0) -> np.ndarray:
        return np.array([self.source(dt, i, fcut) for i in range(steps)], np.float32)

    def sponge_profile(self, s, a, kappa) -> np.ndarray:
        g = np.empty(s, np.float32)
        self.lib.o_sponge_profile(s, a, kappa, _f(g))
        return g

    # ---- stencil -----------------------------------------------------------
    def step(self, kind, sizes, b0, b1, d, dt, pc, qc, pp, qp, coef=None, vpz=None, vsv=None,
             sponge=None, nthreads=None):
        sx, sy, sz = sizes
        cp = (_fp * NCOEF)(*([_f(c) for c in coef] if coef is not None else [None] * NCOEF))
        sp = None
        if sponge is not None:
            sp_arr = (_fp * 3)(*[_f(g) for g in sponge])
            sp = C.cast(sp_arr, C.c_void_p)
        lb0 = (C.c_long * 3)(*b0)
        lb1 = (C.c_long * 3)(*b1)
        rc = self.lib.o_step(kind, sx, sy, sz, lb0, lb1, d[0], d[1], d[2], dt,
                             _vp(pc), _vp(qc), _vp(pp), _vp(qp), cp,
                             _f(vpz), _f(vsv), sp, nthreads or default_threads())
        if rc != 0:
            raise ValueError("box outside the compute region")

    def run(self, kind, sizes, d, dt, steps, pp, pc, qp, qc, coef=None, vpz=None, vsv=None,
            src_index=-1, src=None, sponge=None, rec=None, energy=False, nthreads=None,
            store=0, store_exp=(0, 0)) -> RunResult:
        """Time loop; field arrays are updated in place (copies are the
        caller's business).  Returns the final fields and optional
        traces [steps, nrec] and energy [steps]."""
        dtype = np.float64 if kind in (KIND_F64, KIND_F64_SEP) else np.float32
        for a in (pp, pc, qp, qc):
            assert a.dtype == dtype and a.flags.c_contiguous
        cfg = _RunCfg()
        cfg.kind = kind
        cfg.sx, cfg.sy, cfg.sz = sizes
        cfg.dx, cfg.dy, cfg.dz = d
        cfg.dt = dt
        cfg.steps = steps
        cfg.src_index = src_index
        src_arr = None
        if src is not None:
            src_arr = np.ascontiguousarray(src, np.float32)
            assert src_arr.size >= steps
            cfg.src = _f(src_arr)
        if coef is not None:
            for k in range(NCOEF):
                cfg.coef[k] = _f(coef[k])
        cfg.vpz, cfg.vsv = _f(vpz), _f(vsv)
        if sponge is not None:
            for k in range(3):
                cfg.sponge[k] = _f(sponge[k])
        traces = en = rec_arr = None
        if rec is not None:
            rec_arr = np.ascontiguousarray(rec, np.int64)
            traces = np.zeros((steps, rec_arr.size), np.float64)
            cfg.nrec = rec_arr.size
            cfg.rec = rec_arr.ctypes.data_as(_lp)
            cfg.traces = traces.ctypes.data_as(_dp)
        if energy:
            en = np.zeros(steps, np.float64)
            cfg.energy = en.ctypes.data_as(_dp)
        cfg.nthreads = nthreads or default_threads()
        cfg.store = store
        cfg.store_exp[0], cfg.store_exp[1] = store_exp
        rc = self.lib.o_run(C.byref(cfg), _vp(pp), _vp(pc), _vp(qp), _vp(qc))
        if rc != 0:
            raise RuntimeError("oracle run failed")
        return RunResult(pp, pc, qp, qc, traces, en)


class Reference:
    """The reference's own sources, compiled from the reference checkout or
    its staged copy (oracle/build_oracle.py).  Raises FileNotFoundError when
    unavailable.

    variant "pin":    OpenMP backend, contraction off (bit-exact to the
                      golden fixtures);
    variant "native": OpenMP backend with the reference's own flags (the
                      timed CPU baseline);
    variant "cuda":   the reference's CUDA backend (needs a GPU to run).
    """

    BUILDERS = {"pin": "build_ref", "native": "build_ref_native", "cuda": "build_ref_cuda"}

    def __init__(self, variant: str = "pin"):
        so = getattr(build_oracle, self.BUILDERS[variant])()
        if so is None:
            raise FileNotFoundError(f"reference build '{variant}' not available")
        self.variant = variant
        self.path = so
        lib = C.CDLL(str(so))
        lib.dc_calculate_source.argtypes = [C.c_float, C.c_int]
        lib.dc_calculate_source.restype = C.c_float
        lib.randomVelocityBoundaryPartition.argtypes = [C.c_int] * 14 + [_fp, _fp, C.POINTER(C.c_uint)]
        run_args = [C.c_int, C.c_long, C.c_long, C.c_long, C.c_float, C.c_float,
                    C.c_float, C.c_float, C.c_int, C.c_long, _fp, C.POINTER(_fp),
                    _fp, _fp, _fp, _fp, _fp, _fp, C.POINTER(_fp), C.POINTER(_fp)]
        lib.ref_run.argtypes = run_args
        lib.ref_run.restype = C.c_int
        lib.ref_run_timed.argtypes = run_args + [_dp]
        lib.ref_run_timed.restype = C.c_int
        lib.ref_max_threads.restype = C.c_int
        self.lib = lib

    def threads(self) -> int:
        """OpenMP threads of the backend's parallel regions."""
        return int(self.lib.ref_max_threads())

    def source(self, dt, it) -> float:
        return float(self.lib.dc_calculate_source(dt, it))

    def random_velocity_boundary(self, local, glob, start, n, bord, absorb, vpz, vsv, seed=0):
        s = C.c_uint(seed)
        self.lib.randomVelocityBoundaryPartition(*local, *glob, *start, *n, bord, absorb,
                                                 _f(vpz), _f(vsv), C.byref(s))
        return s.value

    def default_anisotropy(self, shape):
        """dc_compute_anisotropy_vars, copied out of the malloc'd arrays."""
        sx, sy, sz = shape[2], shape[1], shape[0]
        n = sx * sy * sz

        class Aniso(C.Structure):
            _fields_ = [(k, _fp) for k in ("theta", "phi", "vsv", "vpz", "epsilon", "delta")]

        self.lib.dc_compute_anisotropy_vars.argtypes = [C.c_int] * 3
        self.lib.dc_compute_anisotropy_vars.restype = Aniso
        self.lib.dc_free_anisotropy_vars.argtypes = [C.POINTER(Aniso)]
        a = self.lib.dc_compute_anisotropy_vars(sx, sy, sz)
        out = {k: np.ctypeslib.as_array(getattr(a, k), (n,)).reshape(shape).copy()
               for k, _ in Aniso._fields_}
        self.lib.dc_free_anisotropy_vars(C.byref(a))
        return out

    def precomp(self, aniso) -> list[np.ndarray]:
        """dc_compute_precomp_vars on the given anisotropy arrays."""
        shape = aniso["vpz"].shape
        sx, sy, sz = shape[2], shape[1], shape[0]
        n = sx * sy * sz

        class Aniso(C.Structure):
            _fields_ = [(k, _fp) for k in ("theta", "phi", "vsv", "vpz", "epsilon", "delta")]

        class Pre(C.Structure):
            _fields_ = [(k, _fp) for k in COEF_NAMES]

        keep = {k: np.ascontiguousarray(aniso[k], np.float32) for k, _ in Aniso._fields_}
        a = Aniso(*[_f(keep[k]) for k, _ in Aniso._fields_])
        self.lib.dc_compute_precomp_vars.argtypes = [C.c_int] * 3 + [Aniso]
        self.lib.dc_compute_precomp_vars.restype = Pre
        self.lib.dc_free_precomp_vars.argtypes = [C.POINTER(Pre)]
        p = self.lib.dc_compute_precomp_vars(sx, sy, sz, a)
        out = [np.ctypeslib.as_array(getattr(p, k), (n,)).reshape(shape).copy() for k in COEF_NAMES]
        self.lib.dc_free_precomp_vars(C.byref(p))
        return out

    def run(self, kind, sizes, d, dt, steps, pp, pc, qp, qc, coef=None, vpz=None, vsv=None,
            src_index=-1, src=None, timed=False):
        """ref_run: the reference loop through the linked backend's
        dc_propagate (kind 0: the OpenMP path with `coef`, or in the "cuda"
        variant the reference's GPU path with vpz/vsv) or the reference CUDA
        arithmetic replayed on the host (kind 1).  Returns (pc, qc) copies of
        the final fields, and the time loop's wall seconds when `timed`."""
        sx, sy, sz = sizes
        cp = (_fp * NCOEF)(*[_f(c) for c in coef]) if coef is not None else None
        out_pc, out_qc = _fp(), _fp()
        sec = C.c_double(0.0)
        src_arr = np.ascontiguousarray(src, np.float32) if src is not None else None
        rc = self.lib.ref_run_timed(kind, sx, sy, sz, d[0], d[1], d[2], dt, steps, src_index,
                                    _f(src_arr), cp, _f(vpz), _f(vsv), _f(pp), _f(pc), _f(qp),
                                    _f(qc), C.byref(out_pc), C.byref(out_qc), C.byref(sec))
        if rc != 0:
            raise ValueError(f"kind {kind} is not available in the '{self.variant}' build")
        n = sx * sy * sz
        res_pc = np.ctypeslib.as_array(out_pc, (n,)).reshape(pc.shape).copy()
        res_qc = np.ctypeslib.as_array(out_qc, (n,)).reshape(qc.shape).copy()
        if timed:
            return res_pc, res_qc, sec.value
        return res_pc, res_qc


@dataclass
class Geometry:
    """Padded cube of the reference CLI: s = n + 2a + 8 per axis
    (src/main.c:94-99); the source sits at the global centre s//2
    (src/coordinator.c:11-16)."""
    n: tuple[int, int, int]              # interior (x, y, z)
    absorb: int
    sizes: tuple[int, int, int] = field(init=False)

    def __post_init__(self):
        self.sizes = tuple(int(v) + 2 * self.absorb + 8 for v in self.n)

    @property
    def shape(self):
        sx, sy, sz = self.sizes
        return (sz, sy, sx)

    @property
    def count(self):
        return int(np.prod(self.sizes))

    def index(self, x, y, z):
        sx, sy, _ = self.sizes
        return int(x + y * sx + z * sx * sy)

    @property
    def source_index(self):
        sx, sy, sz = self.sizes
        return self.index(sx // 2, sy // 2, sz // 2)

    @property
    def compute_points(self):
        sx, sy, sz = self.sizes
        return (sx - 8) * (sy - 8) * (sz - 8)


def reference_medium(lib, geom: Geometry, seed: int = 0):
    """Reference default medium + random velocity boundary + precompute, the
    set-up of src/main.c:158-172 for one rank.  ``lib`` is Port() or
    Reference(); both must give identical arrays."""
    aniso = lib.default_anisotropy(geom.shape)
    sx, sy, sz = geom.sizes
    lib.random_velocity_boundary((sx, sy, sz), (sx, sy, sz), (0, 0, 0), geom.n, 4, geom.absorb,
                                 aniso["vpz"], aniso["vsv"], seed)
    coef = lib.precomp(aniso)
    return aniso, coef


def _round_bf16(a):
    u = np.asarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


def fixed16(c):
    """An angle term in the GPU's 16-bit medium: c x 2^15 rounded to nearest
    even, clamped to [-32768, 32767], scaled back (exact)."""
    q = np.clip(np.rint(np.asarray(c, np.float32) * np.float32(32768.0)), -32768, 32767)
    return (q / 32768.0).astype(np.float32)


def row_referenced16(v, ratio: str = "f16"):
    """A velocity term in the GPU's 16-bit medium: per row (the last axis)
    the base b is the midrange of the row's non-zero values (float), the
    stored value d = v / b - 1 rounded to FP16 (ratio "f16", what the GPU
    stores) or BF16 (ratio "bf16", a measured alternative), read back as
    b + b * d with a single rounding."""
    v = np.asarray(v, np.float32)
    nz = v != 0
    mn = np.where(nz, v, np.float32(np.inf)).min(axis=-1, keepdims=True).astype(np.float32)
    mx = np.where(nz, v, np.float32(-np.inf)).max(axis=-1, keepdims=True).astype(np.float32)
    with np.errstate(invalid="ignore", over="ignore"):
        mid = (np.float32(0.5) * (mn + mx)).astype(np.float32)
    base = np.where(mn <= mx, mid, np.float32(0.0)).astype(np.float32)
    safe = np.where(base != 0, base, np.float32(1.0)).astype(np.float32)
    d = np.where(base != 0, (v / safe).astype(np.float32) - np.float32(1.0),
                 np.float32(0.0)).astype(np.float32)
    d16 = (d.astype(np.float16) if ratio == "f16" else _round_bf16(d)).astype(np.float64)
    b64 = base.astype(np.float64)
    return (b64 * d16 + b64).astype(np.float32)


def narrow_medium(coef, fmt: str):
    """The ten coefficients (dc_precomp_vars order, arrays (sz, sy, sx)) as
    the fast kernel reads its 16-bit medium copy.

    "f16":  the six angle terms as 16-bit fixed point (fixed16), the four
            velocity terms as FP16 ratios to a per-row FP32 base
            (row_referenced16);
    "bf16": all ten rounded to BF16, the velocity terms scaled by 2^-vexp
            (max below 2^14) before rounding and scaled back;
    "bf16_rowref": the "f16" encoding with BF16 velocity ratios (not a GPU
            form: the measured reason the BF16 copy cannot borrow it)."""
    if fmt == "f16":
        return [fixed16(c) for c in coef[:6]] + [row_referenced16(c) for c in coef[6:]]
    if fmt == "bf16_rowref":
        return [fixed16(c) for c in coef[:6]] + [row_referenced16(c, "bf16") for c in coef[6:]]
    vmax = max(float(np.abs(c).max()) for c in coef[6:])
    vexp = int(np.frexp(vmax)[1]) - 14 if vmax > 0 else 0
    out = [_round_bf16(c) for c in coef[:6]]
    out += [(_round_bf16(np.asarray(c, np.float32) * np.float32(2.0 ** -vexp))
             * np.float32(2.0 ** vexp)).astype(np.float32) for c in coef[6:]]
    return out


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    den = np.linalg.norm(b)
    num = np.linalg.norm(a - b)
    return float(num / den) if den > 0 else float(num)
