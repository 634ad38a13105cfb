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
VARIANT_AUTO, VARIANT_GENERIC, VARIANT_PACKED2, VARIANT_PACKED3, VARIANT_PACKED4 = 0, 1, 2, 3, 4
ORDER_AUTO, ORDER_INPUT, ORDER_BINNED, ORDER_BINNED_TARGETS = 0, 1, 2, 3

STATUS = {0: "ok", -1: "invalid argument", -2: "allocation failed", -3: "CUDA runtime error",
          -4: "device wait timed out", -5: "no usable CUDA device", -6: "singular matrix",
          -7: "unsupported combination", -8: "size exceeds the no-allocation scratch",
          -9: "iterative solve did not reach its tolerance"}


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


def _own32(a):
    """A float32 copy owned by the container (the reference's containers copy their inputs,
    src/Points.h:75-104), so in-place updates never write through to the caller's arrays."""
    if a is None:
        return None
    return np.array(a, dtype=np.float32, copy=True, order="C")


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

    def set_kernel_variant(self, variant: int):
        """VARIANT_AUTO (packed FP32 kernels where available), VARIANT_GENERIC, PACKED2/PACKED4."""
        _check(lib().obs_set_kernel_variant(self._h, ctypes.c_int(variant)), "obs_set_kernel_variant")

    def set_target_order(self, order: int):
        """ORDER_AUTO, ORDER_INPUT, ORDER_BINNED (targets and sources) or ORDER_BINNED_TARGETS: the
        processing order of packed Gaussian velocity sums (results stay in the caller's order)."""
        _check(lib().obs_set_target_order(self._h, ctypes.c_int(order)), "obs_set_target_order")

    @property
    def launches(self) -> int:
        return int(lib().obs_launch_count(self._h))

    def last_failure(self):
        """(bits, code, v1, v2) of the last device-side failure record a synchronizing call read."""
        w = [ctypes.c_int() for _ in range(4)]
        _check(lib().obs_last_failure(self._h, *[ctypes.byref(v) for v in w]), "obs_last_failure")
        return tuple(v.value for v in w)

    def selftest_bounded_wait(self, which: int, max_polls: int = 64) -> int:
        """Run a bounded wait that nothing completes (0: mbarrier, 1: grid barrier) and return the
        status the host reads afterwards (OBS_ERR_TIMEOUT when it gave up as designed)."""
        return int(lib().obs_selftest_bounded_wait(self._h, ctypes.c_int(which), ctypes.c_int(max_polls)))


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
        self.x, self.y = _own32(self.x), _own32(self.y)
        self.r, self.s = _own32(self.r), _own32(self.s)
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


TREE_THETA_DEFAULT = 0.5
TREE_ORDER_DEFAULT = 24
SUMMATION_DIRECT, SUMMATION_TREE = 1, 2      # summation_t direct, barneshut (src/ExecEnv.h:26-31)


def points_affect_points_tree(src: Points, targ: Points, env: ExecEnv | None = None, theta: float = 0.0,
                              order: int = 0, finalize: bool = False, fs=(0.0, 0.0)) -> float:
    """Velocity of the source particles at the targets by treecode (the reference's
    summation_t barneshut slot, src/ExecEnv.h:26-31): accumulated into targ.u, targ.v like
    points_affect_points with VELONLY.  theta (0: 0.5) and order (0: 24 terms) set the
    multipole acceptance and truncation.  Returns the direct-sum flop count of the call."""
    env = env or ExecEnv()
    flops = ctypes.c_double()
    st = lib().obs_points_affect_points_tree(
        env.ctx().handle, ctypes.c_int(env.core), ctypes.c_int(FLAG_FINALIZE if finalize else 0),
        ctypes.c_double(fs[0]), ctypes.c_double(fs[1]), ctypes.c_double(theta), ctypes.c_int(order),
        ctypes.c_int(src.n), _ptr(src.x), _ptr(src.y), _ptr(src.r), _ptr(src.s),
        ctypes.c_int(targ.n), _ptr(targ.x), _ptr(targ.y), _ptr(targ.r), _ptr(targ.u), _ptr(targ.v),
        ctypes.byref(flops))
    _check(st, "obs_points_affect_points_tree")
    return flops.value


def points_affect_points_tree_dev(ctx: "Context", core: int, sx, sy, sr, ss, tx, ty, tr, tu, tv,
                                  theta: float = 0.0, order: int = 0, finalize: bool = False,
                                  fs=(0.0, 0.0)) -> float:
    """Device-resident treecode velocity (CUDA tensors); asynchronous on the context's stream."""
    ns, nt = sx.numel(), tx.numel()
    for name, t, need in (("sy", sy, ns), ("sr", sr, ns), ("ss", ss, ns), ("ty", ty, nt), ("tr", tr, nt),
                          ("tu", tu, nt), ("tv", tv, nt)):
        if t is not None and t.numel() < need:
            raise ValueError(f"{name} has {t.numel()} elements, the call needs {need}")
    flops = ctypes.c_double()
    st = lib().obs_points_affect_points_tree_dev(
        ctx.handle, ctypes.c_int(core), ctypes.c_int(FLAG_FINALIZE if finalize else 0),
        ctypes.c_double(fs[0]), ctypes.c_double(fs[1]), ctypes.c_double(theta), ctypes.c_int(order),
        ctypes.c_int(ns), _ptr(sx), _ptr(sy), _ptr(sr), _ptr(ss),
        ctypes.c_int(nt), _ptr(tx), _ptr(ty), _ptr(tr), _ptr(tu), _ptr(tv), ctypes.byref(flops))
    _check(st, "obs_points_affect_points_tree_dev")
    return flops.value


def points_affect_points_vorticity(src: Points, targ: Points, env: ExecEnv | None = None,
                                   finalize: bool = False) -> None:
    """points_affect_points_vorticity (src/InfluenceVort.h:47-126): accumulate the Gaussian-blob
    vorticity of the source particles at the targets (field points) into ``targ.vort``.  The
    core is always the Gaussian blob; env supplies the context and accumulation mode."""
    env = env or ExecEnv()
    if targ.vort is None:
        targ.vort = np.zeros(targ.n, np.float32)
    st = lib().obs_points_affect_points_vorticity(
        env.ctx().handle, ctypes.c_int(env.accum), ctypes.c_int(FLAG_FINALIZE if finalize else 0),
        ctypes.c_int(src.n), _ptr(src.x), _ptr(src.y), _ptr(src.r), _ptr(src.s),
        ctypes.c_int(targ.n), _ptr(targ.x), _ptr(targ.y), _ptr(targ.vort))
    _check(st, "obs_points_affect_points_vorticity")


def points_affect_points_vorticity_dev(ctx: Context, accum: int, sx, sy, sr, ss, tx, ty, tw, finalize=False):
    _check(lib().obs_points_affect_points_vorticity_dev(
        ctx.handle, ctypes.c_int(accum), ctypes.c_int(FLAG_FINALIZE if finalize else 0),
        ctypes.c_int(sx.numel()), _ptr(sx), _ptr(sy), _ptr(sr), _ptr(ss),
        ctypes.c_int(tx.numel()), _ptr(tx), _ptr(ty), _ptr(tw)), "obs_points_affect_points_vorticity_dev")


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


def morton_order_dev(ctx: Context, x, y, perm):
    """Stable Morton-cell order of n points (CUDA tensors x, y; int32 tensor perm receives it)."""
    n = x.numel()
    if y.numel() < n or perm.numel() < n:
        raise ValueError("y and perm need at least x.numel() elements")
    _check(lib().obs_morton_order_dev(ctx.handle, ctypes.c_int(n), _ptr(x), _ptr(y), _ptr(perm)),
           "obs_morton_order_dev")


def flops_per_pair(core: int, result: int = VELONLY, thick: bool = True) -> int:
    return int(lib().obs_flops_per_pair(ctypes.c_int(core), ctypes.c_int(result), ctypes.c_int(1 if thick else 0)))


# ---------------------------------------------------------------- panels (src/Surfaces.h)

def _u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


@dataclass
class Surfaces:
    """1-D elements (src/Surfaces.h): straight panels between nodes (nx, ny) with node-index
    pairs idx[2k], idx[2k+1]; the fluid is to the left walking node0 -> node1.  vs / ss are the
    vortex / source sheet strengths, bcn the normal-velocity boundary condition, (pu, pv) the
    panel-centre velocities; omega the body's rotation rate after a rotation-augmented solve."""
    nx: np.ndarray
    ny: np.ndarray
    idx: np.ndarray
    vs: np.ndarray | None = None
    ss: np.ndarray | None = None
    bcn: np.ndarray | None = None
    pu: np.ndarray = field(default=None)
    pv: np.ndarray = field(default=None)
    omega: float | None = None   # rotation rate from an augmented solve (solve_bem_bodies)

    def __post_init__(self):
        self.nx, self.ny = _own32(self.nx), _own32(self.ny)
        self.idx = np.array(self.idx, dtype=np.uint32, copy=True)
        self.vs, self.ss, self.bcn = _own32(self.vs), _own32(self.ss), _own32(self.bcn)
        if self.pu is None:
            self.pu = np.zeros(self.npan, np.float32)
        if self.pv is None:
            self.pv = np.zeros(self.npan, np.float32)

    @property
    def npan(self) -> int:
        return self.idx.size // 2

    @property
    def nnodes(self) -> int:
        return self.nx.size

    def zero_vels(self):
        self.pu[:] = 0
        self.pv[:] = 0

    def finalize_vels(self, fs=(0.0, 0.0)):
        """Surfaces::finalize_vels (src/Surfaces.h:764-774) on the panel-centre velocities."""
        f = 0.5 / np.pi
        self.pu[:] = (fs[0] + self.pu.astype(np.float64) * f).astype(np.float32)
        self.pv[:] = (fs[1] + self.pv.astype(np.float64) * f).astype(np.float32)

    def _geo(self):
        return (ctypes.c_int(self.nnodes), _ptr(self.nx), _ptr(self.ny), ctypes.c_int(self.npan), _ptr(self.idx))


def circle_panels(npan: int, diameter: float = 1.0, center=(0.0, 0.0)) -> Surfaces:
    """Closed circle of npan straight panels, nodes at theta_i = -2 pi i / npan (clockwise, so
    the fluid is outside), as SolidCircle lays them out (src/BoundaryFeature.cpp:489-531)."""
    th = -2.0 * np.pi * np.arange(npan) / npan
    nx = center[0] + 0.5 * diameter * np.cos(th)
    ny = center[1] + 0.5 * diameter * np.sin(th)
    idx = np.stack([np.arange(npan), (np.arange(npan) + 1) % npan], 1).ravel()
    return Surfaces(nx, ny, idx)


def join_surfaces(bodies) -> tuple[Surfaces, np.ndarray]:
    """Several bodies as one panel set: nodes and panels concatenated in body order, node
    indices offset, strengths / boundary conditions / velocities carried along where every body
    has them.  Returns the joined Surfaces and the panel offsets (len(bodies) + 1).

    The reference assembles a multi-body BEM system block by block (src/BEMHelper.h:166-221),
    block (t, s) being panels_on_panels_coeff of body s on body t with the self term only on
    the diagonal blocks (src/Coefficients.h:389-401, `&src == &targ`); since the off-diagonal
    pair formula is the same as within one body, that matrix equals the coefficients of the
    joined panel set bit for bit in the reference's own arithmetic."""
    bodies = list(bodies)
    if not bodies:
        raise ValueError("join_surfaces: no bodies")
    offs = np.zeros(len(bodies) + 1, np.int64)
    node0 = 0
    nx, ny, idx = [], [], []
    for k, b in enumerate(bodies):
        nx.append(b.nx)
        ny.append(b.ny)
        idx.append(b.idx.astype(np.int64) + node0)
        node0 += b.nnodes
        offs[k + 1] = offs[k] + b.npan

    def cat(name):
        vals = [getattr(b, name) for b in bodies]
        return None if any(v is None for v in vals) else np.concatenate(vals)

    j = Surfaces(np.concatenate(nx), np.concatenate(ny), np.concatenate(idx), vs=cat("vs"), ss=cat("ss"),
                 bcn=cat("bcn"), pu=cat("pu"), pv=cat("pv"))
    return j, offs


def panels_affect_points(src: Surfaces, targ: Points, env: ExecEnv | None = None, vortex_only: bool = False,
                         finalize: bool = False, fs=(0.0, 0.0)):
    """panels_affect_points (src/Influence.h:422-614): accumulate the panels' influence on the
    points.  The reference always uses the vortex+source kernel for active panels; vortex_only
    selects kernelu_1v_0p."""
    env = env or ExecEnv()
    ss = None if (vortex_only or src.ss is None) else src.ss
    vs = src.vs if src.vs is not None else np.zeros(src.npan, np.float32)
    st = lib().obs_panels_affect_points(env.ctx().handle, ctypes.c_int(env.accum),
                                        ctypes.c_int(FLAG_FINALIZE if finalize else 0),
                                        ctypes.c_double(fs[0]), ctypes.c_double(fs[1]), *src._geo(),
                                        _ptr(vs), _ptr(ss), ctypes.c_int(targ.n), _ptr(targ.x), _ptr(targ.y),
                                        _ptr(targ.u), _ptr(targ.v))
    _check(st, "obs_panels_affect_points")


def panels_affect_points_vjp(src: Surfaces, targ: Points, lu, lv, env: ExecEnv | None = None):
    """Reverse mode of panels_affect_points with respect to the panel strengths: for cotangents
    (lu, lv) of the finalized point velocities returns (dL/d vortex strengths, dL/d source
    strengths), one value per panel (no counterpart in the reference)."""
    env = env or ExecEnv()
    gv = np.zeros(src.npan, np.float32)
    gs = np.zeros(src.npan, np.float32)
    lu, lv = _own32(lu), _own32(lv)
    st = lib().obs_panels_affect_points_vjp(env.ctx().handle, ctypes.c_int(env.accum), *src._geo(),
                                            ctypes.c_int(targ.n), _ptr(targ.x), _ptr(targ.y), _ptr(lu), _ptr(lv),
                                            _ptr(gv), _ptr(gs))
    _check(st, "obs_panels_affect_points_vjp")
    return gv, gs


def panels_affect_points_vjp_dev(ctx: Context, accum: int, nx, ny, idx, tx, ty, lu, lv, gvs, gss=None):
    """Device-resident panel-strength VJP (CUDA tensors), asynchronous; gvs, gss accumulate."""
    _check(lib().obs_panels_affect_points_vjp_dev(ctx.handle, ctypes.c_int(accum), ctypes.c_int(nx.numel()), _ptr(nx),
                                                  _ptr(ny), ctypes.c_int(idx.numel() // 2), _ptr(idx),
                                                  ctypes.c_int(tx.numel()), _ptr(tx), _ptr(ty), _ptr(lu), _ptr(lv),
                                                  _ptr(gvs), _ptr(gss)), "obs_panels_affect_points_vjp_dev")


def points_affect_panels(src: Points, targ: Surfaces, env: ExecEnv | None = None,
                         finalize: bool = False, fs=(0.0, 0.0)):
    """points_affect_panels (src/Influence.h:633-771): mean velocity over each panel due to the
    particles (treated as point vortices, as in the reference), accumulated into targ.pu/pv."""
    env = env or ExecEnv()
    st = lib().obs_points_affect_panels(env.ctx().handle, ctypes.c_int(env.accum),
                                        ctypes.c_int(FLAG_FINALIZE if finalize else 0),
                                        ctypes.c_double(fs[0]), ctypes.c_double(fs[1]),
                                        ctypes.c_int(src.n), _ptr(src.x), _ptr(src.y), _ptr(src.s),
                                        *targ._geo(), _ptr(targ.pu), _ptr(targ.pv))
    _check(st, "obs_points_affect_panels")


def panels_affect_panels(src: Surfaces, targ: Surfaces, env: ExecEnv | None = None, finalize: bool = False,
                         fs=(0.0, 0.0)):
    """panels_affect_panels (src/Influence.h:774-795): accumulate the source panels' influence
    on the target panels' centre velocities (targ.pu, targ.pv) through the reference's
    collocation points 1e-4 off the target panels."""
    env = env or ExecEnv()
    vs = src.vs if src.vs is not None else np.zeros(src.npan, np.float32)
    st = lib().obs_panels_affect_panels(env.ctx().handle, ctypes.c_int(env.accum),
                                        ctypes.c_int(FLAG_FINALIZE if finalize else 0),
                                        ctypes.c_double(fs[0]), ctypes.c_double(fs[1]), *src._geo(),
                                        _ptr(vs), _ptr(src.ss), *targ._geo(), _ptr(targ.pu), _ptr(targ.pv))
    _check(st, "obs_panels_affect_panels")


def panels_on_panels_coeff(src: Surfaces, targ: Surfaces | None = None, nunk: int = 2, fp64: bool = False,
                           context: Context | None = None) -> np.ndarray:
    """panels_on_panels_coeff (src/Coefficients.h:155-427): the (nunk*ntarg, nunk*nsrc)
    influence block (targets are rows); targ None means the self block of src."""
    ctx = context or default_context()
    same = targ is None
    targ = src if same else targ
    nel = src.npan * nunk * targ.npan * nunk
    out = np.zeros(nel, np.float64 if fp64 else np.float32)
    st = lib().obs_panels_on_panels_coeff(ctx.handle, ctypes.c_int(nunk), ctypes.c_int(1 if same else 0),
                                          *src._geo(), *targ._geo(),
                                          None if fp64 else _ptr(out), _ptr(out) if fp64 else None)
    _check(st, "obs_panels_on_panels_coeff")
    return out.reshape(src.npan * nunk, targ.npan * nunk).T.copy()   # column-major -> (rows, cols)


def vels_to_rhs_panels(targ: Surfaces, nunk: int = 2, fp64: bool = False, context: Context | None = None):
    """vels_to_rhs_panels (src/RHS.h:54-115) from targ.pu/pv and targ.bcn."""
    ctx = context or default_context()
    out = np.zeros(targ.npan * nunk, np.float64 if fp64 else np.float32)
    st = lib().obs_vels_to_rhs_panels(ctx.handle, ctypes.c_int(nunk), *targ._geo(), _ptr(targ.pu), _ptr(targ.pv),
                                      _ptr(targ.bcn), None if fp64 else _ptr(out), _ptr(out) if fp64 else None)
    _check(st, "obs_vels_to_rhs_panels")
    return out


def solve_dense_f64(A: np.ndarray, b: np.ndarray, context: Context | None = None):
    """FP64 LU solve of A x = b on the GPU; returns (x, ||A x - b|| / ||b||)."""
    ctx = context or default_context()
    A = np.asarray(A, np.float64)
    n = A.shape[0]
    Ac = np.asfortranarray(A).ravel(order="K") if A.flags.f_contiguous else np.ascontiguousarray(A.T).ravel()
    b = np.ascontiguousarray(b, np.float64)
    x = np.zeros(n)
    rel = ctypes.c_double()
    _check(lib().obs_solve_dense_f64(ctx.handle, ctypes.c_int(n), _ptr(Ac), _ptr(b), _ptr(x), ctypes.byref(rel)),
           "obs_solve_dense_f64")
    return x, rel.value


def solve_gmres_f64(A: np.ndarray, b: np.ndarray, x0=None, tol: float = 1e-13, restart: int = 60,
                    maxiter: int | None = None, context: Context | None = None):
    """FP64 GMRES on the GPU; returns (x, iterations, ||b - A x|| / ||b||)."""
    ctx = context or default_context()
    A = np.asarray(A, np.float64)
    n = A.shape[0]
    Ac = np.ascontiguousarray(A.T).ravel()            # column-major
    b = np.ascontiguousarray(b, np.float64)
    x = np.zeros(n) if x0 is None else np.array(x0, np.float64)
    it, rel = ctypes.c_int(), ctypes.c_double()
    _check(lib().obs_solve_gmres_f64(ctx.handle, ctypes.c_int(n), _ptr(Ac), _ptr(b), _ptr(x), ctypes.c_double(tol),
                                     ctypes.c_int(restart), ctypes.c_int(maxiter or 2 * n), ctypes.byref(it),
                                     ctypes.byref(rel)), "obs_solve_gmres_f64")
    return x, it.value, rel.value


def solve_gmres_f64_dev(ctx: Context, A, b, x, tol: float = 1e-13, restart: int = 60, maxiter: int | None = None):
    """Device FP64 GMRES (A column-major, x = initial guess in, solution out); returns
    (iterations, relative residual)."""
    it, rel = ctypes.c_int(), ctypes.c_double()
    n = b.numel()
    _check(lib().obs_solve_gmres_f64_dev(ctx.handle, ctypes.c_int(n), _ptr(A), _ptr(b), _ptr(x), ctypes.c_double(tol),
                                         ctypes.c_int(restart), ctypes.c_int(maxiter or 2 * n), ctypes.byref(it),
                                         ctypes.byref(rel)), "obs_solve_gmres_f64_dev")
    return it.value, rel.value


def solve_bem(vort: Points, bdry: Surfaces, fs=(0.0, 0.0), nunk: int = 2, env: ExecEnv | None = None,
              reuse_matrix: bool = False, direct_lu: bool = False) -> float:
    """solve_bem for one fixed body (src/BEMHelper.h:43-260): sets bdry.vs (and bdry.ss for
    nunk == 2) from the particles' velocity and the freestream; returns the relative residual."""
    env = env or ExecEnv()
    vs = np.zeros(bdry.npan, np.float32)
    ss = np.zeros(bdry.npan, np.float32) if nunk == 2 else None
    rel = ctypes.c_double()
    st = lib().obs_solve_bem(env.ctx().handle, ctypes.c_int(nunk), ctypes.c_int(env.accum),
                             ctypes.c_int((2 if reuse_matrix else 0) | (4 if direct_lu else 0)),
                             ctypes.c_double(fs[0]), ctypes.c_double(fs[1]),
                             ctypes.c_int(vort.n), _ptr(vort.x), _ptr(vort.y), _ptr(vort.s), *bdry._geo(),
                             _ptr(bdry.bcn), _ptr(vs), _ptr(ss), ctypes.byref(rel))
    _check(st, "obs_solve_bem")
    bdry.vs = vs
    if ss is not None:
        bdry.ss = ss
    return rel.value


def solve_bem_bodies(vort: Points, bodies, fs=(0.0, 0.0), nunk: int = 2, env: ExecEnv | None = None,
                     reuse_matrix: bool = False, direct_lu: bool = False, augmented=None, circ_rhs=None) -> float:
    """solve_bem for several bodies (src/BEMHelper.h:43-260 over a list of boundary
    collections): one system over the joined panel set (join_surfaces), whose matrix is the
    reference's block assembly; sets each body's vs (and ss for nunk == 2) and returns the
    relative residual.  augmented[k] makes body k rotate (src/Coefficients.h:429-572): its
    rotation row takes circ_rhs[k] as right-hand side and its rotation rate is set as
    bodies[k].omega.  The reference rebuilds only the blocks of bodies in relative motion
    (:147-193); here the whole matrix is rebuilt unless reuse_matrix (no body moved, none
    rotating), since assembling it costs about 2 % of a BEM step (4096 unknowns: 0.05 ms of
    2.5 ms)."""
    bodies = list(bodies)
    joined, offs = join_surfaces(bodies)
    if augmented is None or not any(augmented):
        rel = solve_bem(vort, joined, fs=fs, nunk=nunk, env=env, reuse_matrix=reuse_matrix, direct_lu=direct_lu)
        omegas = None
    else:
        env = env or ExecEnv()
        aug = np.ascontiguousarray([1 if a else 0 for a in augmented], np.int32)
        circ = np.ascontiguousarray(np.zeros(len(bodies)) if circ_rhs is None else circ_rhs, np.float64)
        if aug.size != len(bodies) or circ.size != len(bodies):
            raise ValueError("solve_bem_bodies: one augmented flag and one circulation per body")
        vs = np.zeros(joined.npan, np.float32)
        ss = np.zeros(joined.npan, np.float32) if nunk == 2 else None
        omegas = np.zeros(len(bodies))
        off32 = np.ascontiguousarray(offs, np.int32)
        rel_c = ctypes.c_double()
        _check(lib().obs_solve_bem_bodies(env.ctx().handle, ctypes.c_int(nunk), ctypes.c_int(env.accum),
                                          ctypes.c_int(4 if direct_lu else 0), ctypes.c_double(fs[0]),
                                          ctypes.c_double(fs[1]), ctypes.c_int(vort.n), _ptr(vort.x), _ptr(vort.y),
                                          _ptr(vort.s), *joined._geo(), _ptr(joined.bcn), ctypes.c_int(len(bodies)),
                                          _ptr(off32), _ptr(aug), _ptr(circ), _ptr(vs), _ptr(ss), _ptr(omegas),
                                          ctypes.byref(rel_c)), "obs_solve_bem_bodies")
        joined.vs, joined.ss, rel = vs, ss, rel_c.value
    for k, b in enumerate(bodies):
        b.vs = joined.vs[offs[k]:offs[k + 1]].copy()
        if nunk == 2:
            b.ss = joined.ss[offs[k]:offs[k + 1]].copy()
        if omegas is not None and augmented[k]:
            b.omega = float(omegas[k])
    return rel


def panels_on_panels_coeff_bodies(bodies, augmented, nunk: int = 2, accum: int = COMPENSATED,
                                  context: Context | None = None):
    """The BEM matrix of several bodies, some rotating (augmented[k]), over their joined panel
    set: panel unknowns first, then one rotation unknown per rotating body.  Returns the FP64
    (rows, cols) array and (area, centroid x, centroid y) per body (rotating bodies)."""
    ctx = context or default_context()
    bodies = list(bodies)
    joined, offs = join_surfaces(bodies)
    aug = np.ascontiguousarray([1 if a else 0 for a in augmented], np.int32)
    m = joined.npan * nunk + int(aug.sum())
    out = np.zeros(m * m)
    geom = np.zeros(3 * len(bodies))
    _check(lib().obs_panels_on_panels_coeff_bodies(ctx.handle, ctypes.c_int(nunk), ctypes.c_int(accum),
                                                   *joined._geo(), ctypes.c_int(len(bodies)),
                                                   _ptr(np.ascontiguousarray(offs, np.int32)), _ptr(aug), _ptr(out),
                                                   _ptr(geom)), "obs_panels_on_panels_coeff_bodies")
    return out.reshape(m, m).T.copy(), geom.reshape(len(bodies), 3)


# Convection.h:301-302's cutoff factor for clear_inner_layer
CLEAR_CUTOFF = float(0.5 / np.sqrt(2.0 * np.pi))


def clear_inner_layer(pts: Points, body: Surfaces, ips: float, method: int = 0, cutoff_mult: float = CLEAR_CUTOFF,
                      env: ExecEnv | None = None) -> tuple[float, int]:
    """clear_inner_layer for one body (src/Reflect.h:733-760 over clear_inner_panp2, :491-729):
    method 0 crops the particles inside the cutoff layer (strengths scaled, points shifted
    outward by the cut tables), method 1 pushes points (particles, or field points without
    radii) onto the layer.  Updates pts.x, pts.y (and pts.s) in place; returns (circulation
    removed, number of modifications)."""
    env = env or ExecEnv()
    circ, nc = ctypes.c_double(), ctypes.c_longlong()
    st = lib().obs_clear_inner_layer(env.ctx().handle, ctypes.c_int(method), ctypes.c_float(cutoff_mult),
                                     ctypes.c_float(ips), *body._geo(), ctypes.c_int(pts.n), _ptr(pts.x), _ptr(pts.y),
                                     _ptr(pts.s), _ptr(pts.r), ctypes.byref(circ), ctypes.byref(nc))
    _check(st, "obs_clear_inner_layer")
    return circ.value, nc.value


def clear_inner_layer_dev(ctx: Context, method: int, cutoff_mult: float, ips: float, nx, ny, idx, x, y, s=None,
                          r=None) -> tuple[float, int]:
    """Device-resident clear_inner_layer (CUDA tensors, updated in place); synchronizes and
    returns (circulation removed, number of modifications)."""
    circ, nc = ctypes.c_double(), ctypes.c_longlong()
    _check(lib().obs_clear_inner_layer_dev(ctx.handle, ctypes.c_int(method), ctypes.c_float(cutoff_mult),
                                           ctypes.c_float(ips), ctypes.c_int(nx.numel()), _ptr(nx), _ptr(ny),
                                           ctypes.c_int(idx.numel() // 2), _ptr(idx), ctypes.c_int(x.numel()),
                                           _ptr(x), _ptr(y), _ptr(s), _ptr(r), ctypes.byref(circ), ctypes.byref(nc)),
           "obs_clear_inner_layer_dev")
    return circ.value, nc.value


# ---------------------------------------------------------------- device-resident panel calls
# All arrays are CUDA tensors (node coordinates float32, idx int32/uint32 pairs); asynchronous
# on the context's stream, same semantics as the host calls above.

def points_affect_panels_dev(ctx: Context, accum: int, sx, sy, ss, nx, ny, idx, pu, pv, finalize=False,
                             fs=(0.0, 0.0)):
    _check(lib().obs_points_affect_panels_dev(ctx.handle, ctypes.c_int(accum),
                                              ctypes.c_int(FLAG_FINALIZE if finalize else 0),
                                              ctypes.c_double(fs[0]), ctypes.c_double(fs[1]),
                                              ctypes.c_int(sx.numel()), _ptr(sx), _ptr(sy), _ptr(ss),
                                              ctypes.c_int(nx.numel()), _ptr(nx), _ptr(ny),
                                              ctypes.c_int(idx.numel() // 2), _ptr(idx), _ptr(pu), _ptr(pv)),
           "obs_points_affect_panels_dev")


def panels_affect_points_dev(ctx: Context, accum: int, nx, ny, idx, vs, ss, tx, ty, tu, tv, finalize=False,
                             fs=(0.0, 0.0)):
    _check(lib().obs_panels_affect_points_dev(ctx.handle, ctypes.c_int(accum),
                                              ctypes.c_int(FLAG_FINALIZE if finalize else 0),
                                              ctypes.c_double(fs[0]), ctypes.c_double(fs[1]),
                                              ctypes.c_int(nx.numel()), _ptr(nx), _ptr(ny),
                                              ctypes.c_int(idx.numel() // 2), _ptr(idx), _ptr(vs), _ptr(ss),
                                              ctypes.c_int(tx.numel()), _ptr(tx), _ptr(ty), _ptr(tu), _ptr(tv)),
           "obs_panels_affect_points_dev")


def panels_affect_panels_dev(ctx: Context, accum: int, snx, sny, sidx, vs, ss, tnx, tny, tidx, pu, pv,
                             finalize=False, fs=(0.0, 0.0)):
    _check(lib().obs_panels_affect_panels_dev(ctx.handle, ctypes.c_int(accum),
                                              ctypes.c_int(FLAG_FINALIZE if finalize else 0),
                                              ctypes.c_double(fs[0]), ctypes.c_double(fs[1]),
                                              ctypes.c_int(snx.numel()), _ptr(snx), _ptr(sny),
                                              ctypes.c_int(sidx.numel() // 2), _ptr(sidx), _ptr(vs), _ptr(ss),
                                              ctypes.c_int(tnx.numel()), _ptr(tnx), _ptr(tny),
                                              ctypes.c_int(tidx.numel() // 2), _ptr(tidx), _ptr(pu), _ptr(pv)),
           "obs_panels_affect_panels_dev")


def panels_on_panels_coeff_dev(ctx: Context, nunk: int, nx, ny, idx, A32=None, A64=None):
    """Self block of one body into device buffers (column-major, (nunk*npan)^2 elements)."""
    geo = (ctypes.c_int(nx.numel()), _ptr(nx), _ptr(ny), ctypes.c_int(idx.numel() // 2), _ptr(idx))
    _check(lib().obs_panels_on_panels_coeff_dev(ctx.handle, ctypes.c_int(nunk), ctypes.c_int(1), *geo, *geo,
                                                _ptr(A32), _ptr(A64)), "obs_panels_on_panels_coeff_dev")


def vels_to_rhs_panels_dev(ctx: Context, nunk: int, nx, ny, idx, pu, pv, bcn=None, rhs32=None, rhs64=None):
    _check(lib().obs_vels_to_rhs_panels_dev(ctx.handle, ctypes.c_int(nunk), ctypes.c_int(nx.numel()), _ptr(nx),
                                            _ptr(ny), ctypes.c_int(idx.numel() // 2), _ptr(idx), _ptr(pu), _ptr(pv),
                                            _ptr(bcn), _ptr(rhs32), _ptr(rhs64)), "obs_vels_to_rhs_panels_dev")


def solve_dense_f64_dev(ctx: Context, A, b, x) -> float:
    """FP64 LU solve on device arrays (A column-major n x n); returns ||A x - b|| / ||b||."""
    rel = ctypes.c_double()
    _check(lib().obs_solve_dense_f64_dev(ctx.handle, ctypes.c_int(b.numel()), _ptr(A), _ptr(b), _ptr(x),
                                         ctypes.byref(rel)), "obs_solve_dense_f64_dev")
    return rel.value


def panels_on_panels_coeff_augmented(body: Surfaces, nunk: int = 2, accum: int = COMPENSATED,
                                     context: Context | None = None):
    """The rotation-augmented self block of one body (src/Coefficients.h:429-572) as an
    (nunk*npan+1)^2 (rows, cols) FP64 array, and (area, centroid x, centroid y)."""
    ctx = context or default_context()
    m = body.npan * nunk + 1
    out = np.zeros(m * m)
    geom = np.zeros(3)
    _check(lib().obs_panels_on_panels_coeff_augmented(ctx.handle, ctypes.c_int(nunk), ctypes.c_int(accum),
                                                      *body._geo(), _ptr(out), _ptr(geom)),
           "obs_panels_on_panels_coeff_augmented")
    return out.reshape(m, m).T.copy(), tuple(geom)


def solve_bem_augmented(vort: Points, bdry: Surfaces, circ_rhs: float = 0.0, fs=(0.0, 0.0), nunk: int = 2,
                        env: ExecEnv | None = None, direct_lu: bool = False):
    """solve_bem with the rotation augmentation (src/BEMHelper.h:114-135): sets bdry.vs (and
    bdry.ss) and returns (rotation rate, relative residual)."""
    env = env or ExecEnv()
    vs = np.zeros(bdry.npan, np.float32)
    ss = np.zeros(bdry.npan, np.float32) if nunk == 2 else None
    om, rel = ctypes.c_double(), ctypes.c_double()
    _check(lib().obs_solve_bem_augmented(env.ctx().handle, ctypes.c_int(nunk), ctypes.c_int(env.accum),
                                         ctypes.c_int(4 if direct_lu else 0), ctypes.c_double(fs[0]),
                                         ctypes.c_double(fs[1]), ctypes.c_int(vort.n), _ptr(vort.x), _ptr(vort.y),
                                         _ptr(vort.s), *bdry._geo(), _ptr(bdry.bcn), ctypes.c_double(circ_rhs),
                                         _ptr(vs), _ptr(ss), ctypes.byref(om), ctypes.byref(rel)),
           "obs_solve_bem_augmented")
    bdry.vs = vs
    if ss is not None:
        bdry.ss = ss
    return om.value, rel.value


# ---------------------------------------------------------------- reverse mode and time stepping

def points_affect_points_vjp(src: Points, targ: Points, lu, lv, env: ExecEnv | None = None,
                             want_targets: bool = False):
    """Backward of the finalized velocity at a separate target set: given cotangents (lu, lv) on
    targ's velocities, return dL/d(src x, y, s) and, if asked, dL/d(targ x, y)."""
    env = env or ExecEnv()
    lu, lv = _f32(lu), _f32(lv)
    gsx, gsy, gss = (np.zeros(src.n, np.float32) for _ in range(3))
    gtx = np.zeros(targ.n, np.float32) if want_targets else None
    gty = np.zeros(targ.n, np.float32) if want_targets else None
    st = lib().obs_points_affect_points_vjp(env.ctx().handle, ctypes.c_int(env.core), ctypes.c_int(env.accum),
                                            ctypes.c_int(src.n), _ptr(src.x), _ptr(src.y), _ptr(src.r), _ptr(src.s),
                                            ctypes.c_int(targ.n), _ptr(targ.x), _ptr(targ.y), _ptr(targ.r),
                                            _ptr(lu), _ptr(lv), _ptr(gsx), _ptr(gsy), _ptr(gss), _ptr(gtx), _ptr(gty))
    _check(st, "obs_points_affect_points_vjp")
    return (gsx, gsy, gss, gtx, gty) if want_targets else (gsx, gsy, gss)


def points_affect_points_vjp_self(p: Points, lu, lv, env: ExecEnv | None = None):
    """Backward of the particles' own finalized velocity: returns dL/dx, dL/dy, dL/ds."""
    env = env or ExecEnv()
    lu, lv = _f32(lu), _f32(lv)
    gx, gy, gs = (np.zeros(p.n, np.float32) for _ in range(3))
    st = lib().obs_points_affect_points_vjp_self(env.ctx().handle, ctypes.c_int(env.core), ctypes.c_int(env.accum),
                                                 ctypes.c_int(p.n), _ptr(p.x), _ptr(p.y), _ptr(p.r), _ptr(p.s),
                                                 _ptr(lu), _ptr(lv), _ptr(gx), _ptr(gy), _ptr(gs))
    _check(st, "obs_points_affect_points_vjp_self")
    return gx, gy, gs


def points_affect_points_vjp_self_dev(ctx: Context, core: int, accum: int, x, y, r, s, lu, lv, gx=None, gy=None,
                                      gs=None):
    """Device-resident self-interaction backward (CUDA tensors), asynchronous; outputs accumulate."""
    _check(lib().obs_points_affect_points_vjp_self_dev(ctx.handle, ctypes.c_int(core), ctypes.c_int(accum),
                                                       ctypes.c_int(x.numel()), _ptr(x), _ptr(y), _ptr(r), _ptr(s),
                                                       _ptr(lu), _ptr(lv), _ptr(gx), _ptr(gy), _ptr(gs)),
           "obs_points_affect_points_vjp_self_dev")


def advect(p: Points, fs=(0.0, 0.0), dt: float = 0.01, nsteps: int = 1, order: int = 2,
           env: ExecEnv | None = None):
    """Convection::advect_1st (order 1), advect_2nd_ralston (2), advect_3rd (3) or
    advect_2nd_heun (4) without bodies (src/Convection.h:274-598): moves p.x, p.y in place."""
    env = env or ExecEnv()
    st = lib().obs_advect(env.ctx().handle, ctypes.c_int(env.core), ctypes.c_int(env.accum), ctypes.c_int(order),
                          ctypes.c_int(p.n), _ptr(p.x), _ptr(p.y), _ptr(p.r), _ptr(p.s),
                          ctypes.c_double(fs[0]), ctypes.c_double(fs[1]), ctypes.c_double(dt), ctypes.c_int(nsteps))
    _check(st, "obs_advect")


def advect_vjp(p0: Points, lx, ly, fs=(0.0, 0.0), dt: float = 0.01, nsteps: int = 1, order: int = 2,
               checkpoint_every: int = 0, env: ExecEnv | None = None):
    """Backward of advect from the initial state p0: given dL/d(final x, y), returns
    (dL/ds, dL/dx0, dL/dy0, engine device bytes)."""
    env = env or ExecEnv()
    lx, ly = _f32(lx), _f32(ly)
    gs, gx, gy = (np.zeros(p0.n, np.float32) for _ in range(3))
    peak = ctypes.c_longlong()
    st = lib().obs_advect_vjp(env.ctx().handle, ctypes.c_int(env.core), ctypes.c_int(env.accum), ctypes.c_int(order),
                              ctypes.c_int(p0.n), _ptr(p0.x), _ptr(p0.y), _ptr(p0.r), _ptr(p0.s),
                              ctypes.c_double(fs[0]), ctypes.c_double(fs[1]), ctypes.c_double(dt),
                              ctypes.c_int(nsteps), ctypes.c_int(checkpoint_every), _ptr(lx), _ptr(ly),
                              _ptr(gs), _ptr(gx), _ptr(gy), ctypes.byref(peak))
    _check(st, "obs_advect_vjp")
    return gs, gx, gy, peak.value


def points_affect_points_vjp_dev(ctx: Context, core: int, accum: int, sx, sy, sr, ss, tx, ty, tr, lu, lv,
                                 gsx=None, gsy=None, gss=None, gtx=None, gty=None):
    """Device-resident backward (CUDA tensors), asynchronous on the context's stream."""
    st = lib().obs_points_affect_points_vjp_dev(ctx.handle, ctypes.c_int(core), ctypes.c_int(accum),
                                                ctypes.c_int(sx.numel()), _ptr(sx), _ptr(sy), _ptr(sr), _ptr(ss),
                                                ctypes.c_int(tx.numel()), _ptr(tx), _ptr(ty), _ptr(tr), _ptr(lu),
                                                _ptr(lv), _ptr(gsx), _ptr(gsy), _ptr(gss), _ptr(gtx), _ptr(gty))
    _check(st, "obs_points_affect_points_vjp_dev")


def advect_dev(ctx: Context, core: int, accum: int, order: int, x, y, r, s, fs, dt, nsteps):
    st = lib().obs_advect_dev(ctx.handle, ctypes.c_int(core), ctypes.c_int(accum), ctypes.c_int(order),
                              ctypes.c_int(x.numel()), _ptr(x), _ptr(y), _ptr(r), _ptr(s), ctypes.c_double(fs[0]),
                              ctypes.c_double(fs[1]), ctypes.c_double(dt), ctypes.c_int(nsteps))
    _check(st, "obs_advect_dev")


ADVECT_EULER, ADVECT_RK2_RALSTON, ADVECT_RK3, ADVECT_RK2_HEUN = 1, 2, 3, 4
# checkpoint_every value that keeps every step's positions and stage positions (no recompute)
TAPE_ALL = -1


def advect_record_dev(ctx: Context, core: int, accum: int, order: int, x, y, r, s, fs, dt, nsteps,
                      checkpoint_every: int = 0):
    """advect_dev that keeps checkpoints in the context for advect_vjp_tape_dev."""
    _check(lib().obs_advect_record_dev(ctx.handle, ctypes.c_int(core), ctypes.c_int(accum), ctypes.c_int(order),
                                       ctypes.c_int(x.numel()), _ptr(x), _ptr(y), _ptr(r), _ptr(s),
                                       ctypes.c_double(fs[0]), ctypes.c_double(fs[1]), ctypes.c_double(dt),
                                       ctypes.c_int(nsteps), ctypes.c_int(checkpoint_every)), "obs_advect_record_dev")


def advect_vjp_tape_dev(ctx: Context, lx, ly, gs=None, gx0=None, gy0=None) -> int:
    """Backward of the last advect_record_dev on this context; returns the engine's device bytes."""
    peak = ctypes.c_longlong()
    _check(lib().obs_advect_vjp_tape_dev(ctx.handle, _ptr(lx), _ptr(ly), _ptr(gs), _ptr(gx0), _ptr(gy0),
                                         ctypes.byref(peak)), "obs_advect_vjp_tape_dev")
    return peak.value


def advect_vjp_dev(ctx: Context, core: int, accum: int, order: int, x0, y0, r, s, fs, dt, nsteps,
                   checkpoint_every, lx, ly, gs=None, gx0=None, gy0=None) -> int:
    peak = ctypes.c_longlong()
    st = lib().obs_advect_vjp_dev(ctx.handle, ctypes.c_int(core), ctypes.c_int(accum), ctypes.c_int(order),
                                  ctypes.c_int(x0.numel()), _ptr(x0), _ptr(y0), _ptr(r), _ptr(s),
                                  ctypes.c_double(fs[0]), ctypes.c_double(fs[1]), ctypes.c_double(dt),
                                  ctypes.c_int(nsteps), ctypes.c_int(checkpoint_every), _ptr(lx), _ptr(ly),
                                  _ptr(gs), _ptr(gx0), _ptr(gy0), ctypes.byref(peak))
    _check(st, "obs_advect_vjp_dev")
    return peak.value
