"""omega2d_gb300 -- GB300 (sm_103a) direct Biot-Savart engine for Omega2D's influence path.

Python front-end over the C ABI in ``include/omega2d_gb300.h`` (``libomega2d_gb300.so``).
It mirrors the reference's operator interface for this path:

* element containers ``Points`` / ``Surfaces`` (structure-of-arrays, src/Points.h,
  src/Surfaces.h) holding positions, radii/strengths and accumulated velocities;
* the drivers ``points_affect_points``, ``panels_affect_points``, ``points_affect_panels``
  (src/Influence.h), ``panels_on_panels_coeff`` (src/Coefficients.h), ``vels_to_rhs_panels``
  (src/RHS.h), ``finalize_vels`` (src/ElementBase.h) and the BEM solve (src/BEM.h);
* ``ResultsType`` values (src/ResultsType.h) and an ``ExecEnv`` that carries the core function
  and accumulation mode the reference fixes at compile time.

Influence sums accumulate into the targets' velocity arrays, unscaled, exactly like the
reference drivers; ``finalize_vels`` applies fs + u/(2 pi).

The compute path is the CUDA library only: importing this package fails loudly if the library
has not been built, and every call raises ``EngineError`` on a non-zero status.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass, field

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libomega2d_gb300.so")

# ---- enums (include/omega2d_gb300.h)
CORE_RM, CORE_GAUSSIAN, CORE_V2, CORE_WL, CORE_V3, CORE_SINGULAR, CORE_COMPACT_EXP = 1, 2, 3, 4, 5, 6, 7
VELONLY, VELANDGRAD, PSIONLY, VELANDVORT, VELANDSHEAR = 1, 2, 3, 4, 5
PLAIN_F32, COMPENSATED = 0, 1
FLAG_FINALIZE = 1

STATUS = {0: "ok", -1: "invalid argument", -2: "allocation failed", -3: "CUDA runtime error",
          -4: "device wait timed out", -5: "no usable CUDA device", -6: "singular matrix",
          -7: "unsupported combination"}


class EngineError(RuntimeError):
    def __init__(self, status: int, what: str):
        super().__init__(f"{what}: status {status} ({STATUS.get(status, 'unknown')})")
        self.status = status


_lib = None


def lib() -> ctypes.CDLL:
    """The loaded engine library (raises if it was never built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"engine library missing ({LIB_PATH}); build it with __graft_entry__.build()")
        L = ctypes.CDLL(LIB_PATH)
        L.obs_launch_count.restype = ctypes.c_longlong
        L.obs_status_string.restype = ctypes.c_char_p
        for f in ("external_vel_solver_f_", "external_vel_solver_tr_f_", "external_vel_solver_d_"):
            getattr(L, f).restype = ctypes.c_float
        _lib = L
    return _lib


def _check(status: int, what: str):
    if status != 0:
        raise EngineError(status, what)


def _f32(a):
    if a is None:
        return None
    return np.ascontiguousarray(a, dtype=np.float32)


def _ptr(a):
    if a is None:
        return None
    if hasattr(a, "data_ptr"):           # torch tensor on the device
        return ctypes.c_void_p(a.data_ptr())
    return a.ctypes.data_as(ctypes.c_void_p)


class Context:
    """An engine context: device binding, stream and device work buffers (obs_context)."""

    def __init__(self, device: int = 0):
        self._h = ctypes.c_void_p()
        _check(lib().obs_create(ctypes.byref(self._h), ctypes.c_int(device)), "obs_create")

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h:
            lib().obs_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr: int | None):
        """Use the given cudaStream_t handle (0 = legacy default stream); None = own stream."""
        if stream_ptr is None:
            _check(lib().obs_use_own_stream(self._h), "obs_use_own_stream")
        else:
            _check(lib().obs_set_stream(self._h, ctypes.c_void_p(stream_ptr)), "obs_set_stream")

    def synchronize(self):
        _check(lib().obs_synchronize(self._h), "obs_synchronize")

    def enable_timing(self, on: bool = True):
        _check(lib().obs_enable_timing(self._h, ctypes.c_int(1 if on else 0)), "obs_enable_timing")

    def last_timing(self):
        m, c = ctypes.c_float(), ctypes.c_float()
        _check(lib().obs_last_timing(self._h, ctypes.byref(m), ctypes.byref(c)), "obs_last_timing")
        return m.value, c.value

    @property
    def launches(self) -> int:
        return int(lib().obs_launch_count(self._h))


_default_ctx: Context | None = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


# ---------------------------------------------------------------- reference-mirroring types

class ResultsType:
    """src/ResultsType.h: which outputs a driver computes."""

    def __init__(self, rtype: int = VELONLY):
        self.rtype = rtype

    def compute_vel(self):
        return self.rtype != PSIONLY

    def compute_grad(self):
        return self.rtype == VELANDGRAD

    def compute_psi(self):
        return self.rtype == PSIONLY

    def compute_vort(self):
        return self.rtype == VELANDVORT

    def compute_shear(self):
        return self.rtype == VELANDSHEAR


@dataclass
class ExecEnv:
    """src/ExecEnv.h, with the accel_t::gpu_cuda choice made concrete: the core function and
    the accumulation mode (the reference fixes the core at compile time, src/CoreFunc.h:35-39)."""
    core: int = CORE_V2
    accum: int = COMPENSATED
    context: Context | None = None

    def ctx(self) -> Context:
        return self.context or default_context()


@dataclass
class Points:
    """0-D elements (src/Points.h): vortex particles (radius given) or field points (r=None)."""
    x: np.ndarray
    y: np.ndarray
    r: np.ndarray | None = None
    s: np.ndarray | None = None
    u: np.ndarray = field(default=None)
    v: np.ndarray = field(default=None)
    vort: np.ndarray | None = None
    shear: np.ndarray | None = None
    psi: np.ndarray | None = None
    grad: list | None = None   # [du/dx, dv/dx, du/dy, dv/dy]

    def __post_init__(self):
        self.x, self.y = _f32(self.x), _f32(self.y)
        self.r, self.s = _f32(self.r), _f32(self.s)
        n = self.x.size
        if self.u is None:
            self.u = np.zeros(n, np.float32)
        if self.v is None:
            self.v = np.zeros(n, np.float32)

    @property
    def n(self) -> int:
        return self.x.size

    def is_inert(self) -> bool:
        return self.r is None

    def zero_vels(self):
        """ElementBase::zero_vels (src/ElementBase.h:200-212)."""
        self.u[:] = 0
        self.v[:] = 0
        for a in (self.vort, self.shear, self.psi):
            if a is not None:
                a[:] = 0
        if self.grad is not None:
            for g in self.grad:
                g[:] = 0

    def finalize_vels(self, fs=(0.0, 0.0)):
        """ElementBase::finalize_vels (src/ElementBase.h:215-234): u = fs + u/(2 pi)."""
        f = 0.5 / np.pi
        self.u[:] = (fs[0] + self.u.astype(np.float64) * f).astype(np.float32)
        self.v[:] = (fs[1] + self.v.astype(np.float64) * f).astype(np.float32)
        for a in (self.vort, self.shear):
            if a is not None:
                a[:] = (a.astype(np.float64) * f).astype(np.float32)


def points_affect_points(src: Points, targ: Points, restype: ResultsType | int = VELONLY,
                         env: ExecEnv | None = None, finalize: bool = False, fs=(0.0, 0.0)) -> float:
    """points_affect_points (src/Influence.h:56-416): accumulate the influence of the source
    particles on the targets (thick targets when ``targ.r`` is set, field points otherwise).
    Returns the reference's flop count for the call."""
    env = env or ExecEnv()
    rt = restype.rtype if isinstance(restype, ResultsType) else int(restype)
    nt = targ.n
    ex = [None] * 4
    if rt == VELANDGRAD:
        if targ.grad is None:
            targ.grad = [np.zeros(nt, np.float32) for _ in range(4)]
        ex = list(targ.grad)
    elif rt == VELANDVORT:
        if targ.vort is None:
            targ.vort = np.zeros(nt, np.float32)
        ex[0] = targ.vort
    elif rt == VELANDSHEAR:
        if targ.shear is None:
            targ.shear = np.zeros(nt, np.float32)
        ex[0] = targ.shear
    elif rt == PSIONLY:
        if targ.psi is None:
            targ.psi = np.zeros(nt, np.float32)
        ex[0] = targ.psi
    flops = ctypes.c_double()
    st = lib().obs_points_affect_points(
        env.ctx().handle, ctypes.c_int(env.core), ctypes.c_int(rt), ctypes.c_int(env.accum),
        ctypes.c_int(FLAG_FINALIZE if finalize else 0), ctypes.c_double(fs[0]), ctypes.c_double(fs[1]),
        ctypes.c_int(src.n), _ptr(src.x), _ptr(src.y), _ptr(src.r), _ptr(src.s),
        ctypes.c_int(nt), _ptr(targ.x), _ptr(targ.y), _ptr(targ.r),
        _ptr(targ.u), _ptr(targ.v), *[_ptr(e) for e in ex], ctypes.byref(flops))
    _check(st, "obs_points_affect_points")
    return flops.value


def points_affect_points_dev(ctx: Context, core: int, result: int, accum: int, sx, sy, sr, ss,
                             tx, ty, tr, tu, tv, extra=(None, None, None, None), finalize=False,
                             fs=(0.0, 0.0)) -> float:
    """Device-resident variant: all arrays are CUDA tensors (or objects with data_ptr());
    asynchronous on the context's stream."""
    flops = ctypes.c_double()
    extra = list(extra) + [None] * (4 - len(extra))
    ns, nt = sx.numel(), tx.numel()
    for name, t, need in (("sy", sy, ns), ("sr", sr, ns), ("ss", ss, ns), ("ty", ty, nt), ("tr", tr, nt),
                          ("tu", tu, nt), ("tv", tv, nt), *[(f"extra{k}", e, nt) for k, e in enumerate(extra)]):
        if t is not None and t.numel() < need:
            raise ValueError(f"{name} has {t.numel()} elements, the call needs {need}")
    st = lib().obs_points_affect_points_dev(
        ctx.handle, ctypes.c_int(core), ctypes.c_int(result), ctypes.c_int(accum),
        ctypes.c_int(FLAG_FINALIZE if finalize else 0), ctypes.c_double(fs[0]), ctypes.c_double(fs[1]),
        ctypes.c_int(sx.numel()), _ptr(sx), _ptr(sy), _ptr(sr), _ptr(ss),
        ctypes.c_int(tx.numel()), _ptr(tx), _ptr(ty), _ptr(tr), _ptr(tu), _ptr(tv),
        *[_ptr(e) for e in extra], ctypes.byref(flops))
    _check(st, "obs_points_affect_points_dev")
    return flops.value


def flops_per_pair(core: int, result: int = VELONLY, thick: bool = True) -> int:
    return int(lib().obs_flops_per_pair(ctypes.c_int(core), ctypes.c_int(result), ctypes.c_int(1 if thick else 0)))
