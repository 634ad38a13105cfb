"""GPU test of obs_points_affect_points_noalloc, the entry point for callers that cannot
allocate device memory (framework-owned allocators, FFI callers with finished buffers).

It must give the same velocities as the allocating entry point, on two calls in a row (the
second call reuses the fixed scratch the first one left behind), and reject source counts
beyond its fixed scratch.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

import omega2d_gb300 as og
from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL = {og.PLAIN_F32: 2e-5, og.COMPENSATED: 2e-6}


def _noalloc(core, result, accum, sx, sy, sr, ss, tx, ty, tr, tu, tv, extra=(None, None, None, None)):
    L = og.lib()
    P = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())
    return L.obs_points_affect_points_noalloc(
        None, ctypes.c_int(core), ctypes.c_int(result), ctypes.c_int(accum), ctypes.c_int(0),
        ctypes.c_double(0.0), ctypes.c_double(0.0),
        ctypes.c_int(sx.numel()), P(sx), P(sy), P(sr), P(ss),
        ctypes.c_int(tx.numel()), P(tx), P(ty), P(tr), P(tu), P(tv), *[P(e) for e in extra])


def _cloud(rng, n, torch, dev):
    x, y = rng.uniform(-1, 1, (2, n)).astype(np.float32)
    r = rng.uniform(0.01, 0.03, n).astype(np.float32)
    s = rng.normal(0, 1 / np.sqrt(n), n).astype(np.float32)
    return [torch.from_numpy(a).to(dev) for a in (x, y, r, s)]


@pytest.mark.parametrize("core,result,accum", [
    (og.CORE_GAUSSIAN, og.VELONLY, og.COMPENSATED),
    (og.CORE_RM, og.VELANDGRAD, og.PLAIN_F32),
])
def test_noalloc_matches_allocating_entry_point_twice(core, result, accum):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(77)
    ctx = og.Context(0)
    ctx.set_stream(0)          # legacy default stream, like the no-allocation call below
    try:
        # two calls in a row with different sizes: the second must not see the first's data
        for ns, nt in ((60_000, 30_000), (9_000, 45_000)):
            sx, sy, sr, ss = _cloud(rng, ns, torch, dev)
            tx, ty, tr, _ = _cloud(rng, nt, torch, dev)
            nex = 4 if result == og.VELANDGRAD else 0
            ref_uv = [torch.zeros(nt, device=dev) for _ in range(2 + nex)]
            got_uv = [torch.zeros(nt, device=dev) for _ in range(2 + nex)]
            ex_ref = ref_uv[2:] + [None] * (4 - nex)
            ex_got = got_uv[2:] + [None] * (4 - nex)
            og.points_affect_points_dev(ctx, core, result, accum, sx, sy, sr, ss, tx, ty, tr,
                                        ref_uv[0], ref_uv[1], extra=ex_ref)
            ctx.synchronize()
            st = _noalloc(core, result, accum, sx, sy, sr, ss, tx, ty, tr, got_uv[0], got_uv[1], ex_got)
            assert st == 0, og.STATUS.get(st, st)
            torch.cuda.synchronize()
            for a, b in zip(ref_uv, got_uv):
                a, b = a.cpu().numpy(), b.cpu().numpy()
                assert np.isfinite(b).all()
                assert rel_err(a, b) < TOL[accum]
    finally:
        ctx.close()


def test_noalloc_rejects_sources_beyond_its_scratch():
    L = og.lib()
    limit = 262144
    assert L.obs_points_affect_points_noalloc(None, 2, 1, 1, 0, ctypes.c_double(0), ctypes.c_double(0),
                                              limit + 1, None, None, None, None, 10, None, None, None,
                                              None, None, None, None, None, None) == -8
    L.obs_status_string.restype = ctypes.c_char_p
    assert b"no-allocation" in L.obs_status_string(-8)


def test_noalloc_allocates_no_device_memory():
    """After one warm-up pass (the first launch of each kernel loads its code onto the GPU),
    further calls of several sizes -- velocity, streamfunction (PSIONLY) and field-point
    (tr == NULL) calls -- leave the device's free memory and torch's allocator unchanged, and
    match the allocating entry point."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(78)
    configs = [(og.CORE_GAUSSIAN, og.VELONLY, og.COMPENSATED, True),
               (og.CORE_V2, og.PSIONLY, og.COMPENSATED, True),
               (og.CORE_RM, og.VELONLY, og.PLAIN_F32, False)]
    sizes = [(60_000, 30_000), (200_000, 3_000), (5_000, 100_000)]
    cases = []
    ctx = og.Context(0)
    ctx.set_stream(0)
    try:
        for core, result, accum, thick in configs:
            for ns, nt in sizes:
                sx, sy, sr, ss = _cloud(rng, ns, torch, dev)
                tx, ty, tr, _ = _cloud(rng, nt, torch, dev)
                tr = tr if thick else None
                ref = [torch.zeros(nt, device=dev) for _ in range(3)]
                ex_ref = [ref[2], None, None, None] if result == og.PSIONLY else [None] * 4
                og.points_affect_points_dev(ctx, core, result, accum, sx, sy, sr, ss, tx, ty, tr,
                                            ref[0], ref[1], extra=ex_ref)
                got = [torch.zeros(nt, device=dev) for _ in range(3)]
                cases.append((core, result, accum, sx, sy, sr, ss, tx, ty, tr, ref, got))
        ctx.synchronize()
    finally:
        ctx.close()

    def call(c):
        core, result, accum, sx, sy, sr, ss, tx, ty, tr, _, got = c
        for t in got:
            t.zero_()
        psi = result == og.PSIONLY
        st = _noalloc(core, result, accum, sx, sy, sr, ss, tx, ty, tr, None if psi else got[0],
                      None if psi else got[1], (got[2] if psi else None, None, None, None))
        assert st == 0, og.STATUS.get(st, st)

    for c in cases:               # warm-up: every kernel of every path launched once
        call(c)
    torch.cuda.synchronize()
    free0, alloc0 = torch.cuda.mem_get_info(dev)[0], torch.cuda.memory_allocated(dev)
    for c in cases:
        call(c)
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info(dev)[0] == free0
        assert torch.cuda.memory_allocated(dev) == alloc0
    for core, result, accum, *_, ref, got in cases:     # results checked after the measured calls
        pairs = [(ref[2], got[2])] if result == og.PSIONLY else [(ref[0], got[0]), (ref[1], got[1])]
        for a, b in pairs:
            a, b = a.cpu().numpy(), b.cpu().numpy()
            assert np.isfinite(b).all()
            assert rel_err(a, b) < TOL[accum]
        if result == og.PSIONLY:
            assert not got[0].cpu().numpy().any() and not got[1].cpu().numpy().any()   # velocity untouched


@pytest.mark.filterwarnings("ignore:The CUDA Graph is empty")
def test_noalloc_refuses_a_capturing_stream():
    """Every call ends by synchronizing its stream, which a stream capture does not allow: on a
    stream that is being captured the call does nothing and returns OBS_ERR_UNSUPPORTED."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(79)
    sx, sy, sr, ss = _cloud(rng, 4_000, torch, dev)
    tx, ty, tr, _ = _cloud(rng, 2_000, torch, dev)
    tu, tv = torch.zeros(2_000, device=dev), torch.zeros(2_000, device=dev)
    L = og.lib()
    P = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    torch.cuda.synchronize()
    with torch.cuda.stream(s):
        g.capture_begin()
        try:
            st = L.obs_points_affect_points_noalloc(
                ctypes.c_void_p(s.cuda_stream), ctypes.c_int(og.CORE_GAUSSIAN), ctypes.c_int(og.VELONLY),
                ctypes.c_int(og.COMPENSATED), ctypes.c_int(0), ctypes.c_double(0.0), ctypes.c_double(0.0),
                ctypes.c_int(sx.numel()), P(sx), P(sy), P(sr), P(ss),
                ctypes.c_int(tx.numel()), P(tx), P(ty), P(tr), P(tu), P(tv), None, None, None, None)
        finally:
            g.capture_end()
    torch.cuda.synchronize()
    assert st == -7, og.STATUS.get(st, st)
    assert not bool(tu.any()) and not bool(tv.any())
