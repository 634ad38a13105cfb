"""CPU checks of bench.py's host-side workload construction."""
import numpy as np

import bench


def test_workload_follows_requested_size(monkeypatch):
    monkeypatch.setattr(bench, "N", 4096)
    x, y, r, s = bench.make_workload()
    assert x.size == y.size == r.size == s.size == 4096
    assert abs(float(s.astype(np.float64).sum()) - 1.0) < 1e-5
    assert np.all(r == bench.SIGMA)


def test_workload_is_seeded():
    a = bench.make_workload(7, 1000)
    b = bench.make_workload(7, 1000)
    for u, v in zip(a, b):
        np.testing.assert_array_equal(u, v)


def test_reference_arm_prints_the_contract_line():
    """`bench.py --impl reference` (CPU only) prints one JSON line with the engine arm's metric,
    a cpu_baseline describing the run and an e2e object without transfers."""
    import json
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0", "--n", "20000", "--cpu-sample", "256"],
                         capture_output=True, text=True, timeout=300, cwd=root)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["value"] > 0 and d["higher_is_better"] is True and d["steps"] == 1
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert d["cpu_baseline"]["kind"] in ("reference", "port")
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_rk2_workload_options_reach_the_run(monkeypatch):
    """--rk-steps and --checkpoint-every (-1: the full tape) are handed to the RK2 adjoint run."""
    import sys
    seen = {}
    monkeypatch.setattr(bench, "run_rk2adjoint2M", lambda args: seen.update(vars(args)))
    monkeypatch.setattr(sys, "argv", ["bench.py", "--workload", "rk2adjoint2M", "--rk-steps", "4",
                                      "--checkpoint-every", "-1"])
    bench.main()
    assert seen["rk_steps"] == 4 and seen["checkpoint_every"] == -1
    monkeypatch.setattr(sys, "argv", ["bench.py", "--workload", "rk2adjoint2M"])
    bench.main()
    assert seen["rk_steps"] == 64 and seen["checkpoint_every"] == 8
