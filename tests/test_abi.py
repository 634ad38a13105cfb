"""CPU tests of the C ABI surface: the engine library loads, exports every function declared in
include/*.h, and rejects bad arguments without touching a GPU."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from conftest import ROOT


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", text, flags=re.M):
            name = m.group(1)
            if name not in ("if", "defined"):
                names.add(name)
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("obs_create", "obs_points_affect_points", "external_vel_solver_f_",
                 "external_vel_solver_tr_f_", "external_vel_solver_d_"):
        assert must in names


def test_library_exports_every_declared_symbol(engine_lib):
    missing = [n for n in declared_functions() if not hasattr(engine_lib, n)]
    assert not missing, missing


def test_status_strings(engine_lib):
    engine_lib.obs_status_string.restype = ctypes.c_char_p
    assert engine_lib.obs_status_string(0) == b"ok"
    assert engine_lib.obs_status_string(-1) == b"invalid argument"
    assert engine_lib.obs_status_string(-4) == b"device wait timed out"


def test_null_context_is_rejected(engine_lib):
    assert engine_lib.obs_destroy(None) == -1
    assert engine_lib.obs_synchronize(None) == -1
    z = np.zeros(4, np.float32)
    p = z.ctypes.data_as(ctypes.c_void_p)
    st = engine_lib.obs_points_affect_points(None, 1, 1, 0, 0, ctypes.c_double(0), ctypes.c_double(0),
                                             4, p, p, p, p, 4, p, p, None, p, p, None, None, None, None, None)
    assert st == -1


def test_create_without_device_reports_no_device(engine_lib):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    h = ctypes.c_void_p()
    assert engine_lib.obs_create(ctypes.byref(h), 0) == -5


def test_flops_per_pair_matches_reference_counts(engine_lib, golden):
    g = golden("p2p")
    # thick-target velocity, field-point velocity, thick-target gradient (src/Kernels.h flops*)
    for name, core in (("rm", 1), ("exp", 2), ("v2", 3), ("wl", 4), ("v3", 5)):
        ref = list(g[f"{name}_flops"])
        assert engine_lib.obs_flops_per_pair(core, 1, 1) == ref[0]
        assert engine_lib.obs_flops_per_pair(core, 1, 0) == ref[1]
        assert engine_lib.obs_flops_per_pair(core, 2, 1) == ref[2]
        assert engine_lib.obs_flops_per_pair(core, 4, 1) == ref[3]
        assert engine_lib.obs_flops_per_pair(core, 5, 1) == ref[4]


def test_external_solver_rejects_null_counts(engine_lib):
    engine_lib.external_vel_solver_f_.restype = ctypes.c_float
    assert engine_lib.external_vel_solver_f_(None, None, None, None, None, None, None, None, None, None) < 0


def test_python_constants_mirror_header_defines():
    """Every OBS_<NAME> integer #define that the Python module also names as <NAME> has the same
    value there (result types, cores, accumulation modes, schemes, flags, tape modes)."""
    import omega2d_gb300 as og
    seen = 0
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        for m in re.finditer(r"^#define\s+OBS_(\w+)\s+\(?(-?\d+)\)?\s*$", open(h).read(), flags=re.M):
            name, val = m.group(1), int(m.group(2))
            if hasattr(og, name):
                assert getattr(og, name) == val, name
                seen += 1
    assert seen >= 10 and og.TAPE_ALL == -1


def test_clear_inner_layer_rejects_bad_arguments_without_a_device(engine_lib):
    """obs_clear_inner_layer validates before it binds a device: a null context, an unknown
    method, a non-positive ips and cropping without radii are OBS_ERR_ARG."""
    f = engine_lib.obs_clear_inner_layer
    z = np.zeros(4, np.float32)
    p = z.ctypes.data_as(ctypes.c_void_p)
    idx = np.array([0, 1, 1, 0], np.uint32).ctypes.data_as(ctypes.c_void_p)
    C, F = ctypes.c_int, ctypes.c_float

    def call(ctx, method, ips, r):
        return f(ctx, C(method), F(0.2), F(ips), C(2), p, p, C(2), idx, C(4), p, p, p, r, None, None)
    assert call(None, 0, 0.02, p) == -1
    h = ctypes.c_void_p(1)                      # never dereferenced: the checks come first
    assert call(h, 2, 0.02, p) == -1
    assert call(h, 1, 0.0, p) == -1
    assert call(h, 0, 0.02, None) == -1


def test_tree_entry_points_check_arguments(engine_lib):
    """The treecode entry points reject a null context, theta outside (0, 1), an order beyond 32
    and missing arrays before touching a device; the external hook's summation switch rejects
    unknown summations."""
    z = np.zeros(4, np.float32)
    p = z.ctypes.data_as(ctypes.c_void_p)
    for fn in (engine_lib.obs_points_affect_points_tree, engine_lib.obs_points_affect_points_tree_dev):
        args = lambda theta, order, sr=p: (None, 2, 0, ctypes.c_double(0), ctypes.c_double(0), ctypes.c_double(theta),
                                           ctypes.c_int(order), 4, p, p, sr, p, 4, p, p, None, p, p, None)
        assert fn(*args(0.5, 24)) == -1                     # null context
    sw = engine_lib.obs_external_configure_summation
    assert sw(3, ctypes.c_double(0.5), 24) == -1
    assert sw(2, ctypes.c_double(1.0), 24) == -1
    assert sw(2, ctypes.c_double(0.5), 33) == -1
    assert sw(2, ctypes.c_double(0.0), 0) == 0             # defaults
    assert sw(1, ctypes.c_double(0.0), 0) == 0             # back to direct sums


def test_bodies_entry_points_check_arguments(engine_lib):
    """obs_panels_on_panels_coeff_bodies and obs_solve_bem_bodies reject a null context, panel
    offsets that do not start at 0, end at npan and increase, and missing body arrays, before
    they bind a device."""
    nx = np.array([1, 0, -1, 0, 3, 2, 3], np.float32)
    ny = np.array([0, -1, 0, 1, 0, 0, 1], np.float32)
    idx = np.array([0, 1, 1, 2, 2, 3, 3, 0, 4, 5, 5, 6, 6, 4], np.uint32)
    out = np.zeros(64, np.float64)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    aug = np.array([1, 1], np.int32)
    h = ctypes.c_void_p(1)                      # never dereferenced: the checks come first
    coeff = engine_lib.obs_panels_on_panels_coeff_bodies

    def call(ctx, off, augp=P(aug)):
        return coeff(ctx, 2, 1, 7, P(nx), P(ny), 7, P(idx), 2, P(off), augp, P(out), None)
    good = np.array([0, 4, 7], np.int32)
    assert call(None, good) == -1
    for bad in ([1, 4, 7], [0, 4, 6], [0, 4, 4], [0, 8, 7]):
        assert call(h, np.array(bad, np.int32)) == -1, bad
    assert call(h, good, None) == -1
    solve = engine_lib.obs_solve_bem_bodies
    z = np.zeros(8, np.float32)
    circ = np.zeros(2, np.float64)
    D = ctypes.c_double
    assert solve(None, 2, 1, 0, D(0), D(0), 0, None, None, None, 7, P(nx), P(ny), 7, P(idx), None, 2, P(good),
                 P(aug), P(circ), P(z), P(z), P(circ), None) == -1
    assert solve(h, 2, 1, 0, D(0), D(0), 0, None, None, None, 7, P(nx), P(ny), 7, P(idx), None, 2,
                 P(np.array([0, 7, 7], np.int32)), P(aug), P(circ), P(z), P(z), P(circ), None) == -1
