"""The header-only C++ adapters (include/omega2d_gb300_influence.hpp) compile against element
containers shaped like the reference's (src/Points.h, src/Surfaces.h accessors; the non-const
get_pos / get_str that clear_inner_panp2 writes through) and link against the engine library.  Without a GPU the first call reports the missing device through
the adapter's exception, which the program prints."""
import os
import shutil
import subprocess

import pytest

import omega2d_gb300 as og

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <array>
#include <cstdio>
#include <cstdint>
#include <stdexcept>
#include <vector>
#include "omega2d_gb300_influence.hpp"

template <class T> using Vector = std::vector<T>;
using Int = std::uint32_t;

// the accessors the reference's Points<float> offers (src/ElementBase.h, src/Points.h)
struct Points {
  std::array<Vector<float>, 2> x, u;
  Vector<float> r, s, vort, shear;
  bool inert = false;
  size_t get_n() const { return x[0].size(); }
  bool is_inert() const { return inert; }
  const std::array<Vector<float>, 2>& get_pos() const { return x; }
  std::array<Vector<float>, 2>& get_pos() { return x; }
  const Vector<float>& get_rad() const { return r; }
  const Vector<float>& get_str() const { return s; }
  Vector<float>& get_str() { return s; }
  std::array<Vector<float>, 2>& get_vel() { return u; }
  Vector<float>& get_vort() { return vort; }
  Vector<float>& get_shear() { return shear; }
};

// the accessors the reference's Surfaces<float> offers (src/Surfaces.h:231-252)
struct Surfaces {
  std::array<Vector<float>, 2> x, pu;
  std::vector<Int> idx;
  Vector<float> vs, ss;
  size_t get_npanels() const { return idx.size() / 2; }
  const std::array<Vector<float>, 2>& get_pos() const { return x; }
  const std::vector<Int>& get_idx() const { return idx; }
  const Vector<float>& get_str() const { return vs; }
  bool have_src_str() const { return !ss.empty(); }
  const Vector<float>& get_src_str() const { return ss; }
  std::array<Vector<float>, 2>& get_vel() { return pu; }
};

int main() {
  Points p;
  p.x = {Vector<float>{0.1f, 0.3f}, Vector<float>{0.2f, 0.25f}};   // inside the triangle, off its panels
  p.u = {Vector<float>(2, 0.f), Vector<float>(2, 0.f)};
  p.r = {0.1f, 0.1f};
  p.s = {1.f, -1.f};
  Surfaces b;
  b.x = {Vector<float>{1.f, 0.f, -1.f}, Vector<float>{0.f, 1.f, 0.f}};
  b.idx = {0, 1, 1, 2, 2, 0};
  b.vs = {1.f, 1.f, 1.f};
  b.pu = {Vector<float>(3, 0.f), Vector<float>(3, 0.f)};
  // compiled and linked here; the engine call behind it is tested through the Python binding
  float (*clear)(int, const Surfaces&, Points&, float, float) = &omega2d_gb300::clear_inner_panp2<Surfaces, Points>;
  (void)clear;
  try {
    omega2d_gb300::points_affect_points(p, p, OBS_VELONLY);
    omega2d_gb300::panels_affect_points(b, p);
    omega2d_gb300::points_affect_panels(p, b);
    std::printf("ran %g %g\n", p.u[0][0], b.pu[0][0]);
  } catch (const std::exception& e) {
    std::printf("caught %s\n", e.what());
  }
  return 0;
}
"""


def _build_and_run(tmp_path):
    lib = og.LIB_PATH
    if not os.path.exists(lib):
        pytest.skip("engine library not built")
    src = tmp_path / "adapter.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "adapter"
    cmd = ["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src), lib,
           "-Wl,-rpath," + os.path.dirname(lib), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    return out.stdout


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_adapter_compiles_and_links(tmp_path):
    out = _build_and_run(tmp_path)
    # with a GPU the three calls run; without one the first reports the missing device
    assert out.startswith("ran ") or "obs_create" in out, out


@pytest.mark.gpu
@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_adapter_runs_on_gpu(tmp_path):
    out = _build_and_run(tmp_path)
    assert out.startswith("ran "), out
    vals = [float(v) for v in out.split()[1:]]
    assert all(v == v and abs(v) < 1e6 for v in vals) and any(v != 0.0 for v in vals)
