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


# ---- the same adapters inside the reference's own drivers, with its real containers

GPU_BRANCH = {
    "void points_affect_points (const Points<S>& src, Points<S>& targ, const ResultsType& restype, const ExecEnv& env) {":
        "omega2d_gb300::points_affect_points(src, targ, restype.get_type());",
    "void panels_affect_points (const Surfaces<S>& src, Points<S>& targ, const ResultsType& restype, const ExecEnv& env) {":
        "omega2d_gb300::panels_affect_points(src, targ);",
    "void points_affect_panels (const Points<S>& src, Surfaces<S>& targ, const ResultsType& restype, const ExecEnv& env) {":
        "omega2d_gb300::points_affect_panels(src, targ);",
}

REF_PROGRAM = r"""
#include "Omega2D.h"
#include "Collection.h"
#include "Influence.h"
#include "Reflect.h"
#include <cstdio>
#include <stdexcept>

int main() {
  // two particles and a triangle, built the way the reference builds its elements
  std::vector<float> xy = {0.1f, 0.2f, 0.3f, 0.25f};
  std::vector<float> str = {1.f, -1.f};
  ElementPacket<float> pk(xy, std::vector<Int>(), str, 2, 0);
  Points<float> p(pk, active, lagrangian, nullptr, 1.0f);
  p.get_rad()[0] = 0.1f;
  p.get_rad()[1] = 0.1f;
  std::vector<float> nxy = {1.f, 0.f, 0.f, 1.f, -1.f, 0.f};
  std::vector<Int> idx = {0, 1, 1, 2, 2, 0};
  std::vector<float> val = {1.f, 0.f, 1.f, 0.f, 1.f, 0.f};
  ElementPacket<float> bk(nxy, idx, val, 3, 1);
  Surfaces<float> b(bk, reactive, fixed, nullptr);
  const ExecEnv env(true, direct, gpu_cuda);
  try {
    points_affect_points<float, double>(p, p, ResultsType(velonly), env);
    panels_affect_points<float, double>(b, p, ResultsType(velonly), env);
    points_affect_panels<float, double>(p, b, ResultsType(velonly), env);
    const float lost = omega2d_gb300::clear_inner_panp2(0, b, p, 0.2f, 0.02f);
    std::printf("ran %g %g %g\n", p.get_vel()[0][0], b.get_vel()[0][0], lost);
  } catch (const std::exception& e) {
    std::printf("caught %s\n", e.what());
  }
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_adapter_inside_reference_drivers(tmp_path):
    """A temporary copy of the reference's src/Influence.h with the gpu_cuda branch of the
    integration guide inserted at the top of points_affect_points, panels_affect_points and
    points_affect_panels (src/Influence.h:57, :423, :634), compiled with the reference's real
    Points<float> / Surfaces<float> (src/Points.h, src/Surfaces.h) and linked against the
    engine.  The reference tree is read in place; only the patched header is written, under the
    test's temporary directory."""
    from oracle import build_ref
    if not build_ref.available():
        pytest.skip("reference tree not present")
    lib = og.LIB_PATH
    if not os.path.exists(lib):
        pytest.skip("engine library not built")
    ref_src = os.path.join(build_ref.REF_ROOT, "src")
    inc = tmp_path / "inc"
    inc.mkdir()
    for name in os.listdir(ref_src):
        if name != "Influence.h":
            os.symlink(os.path.join(ref_src, name), inc / name)
    text = open(os.path.join(ref_src, "Influence.h")).read()
    text = text.replace("#include <cassert>\n", "#include <cassert>\n#include <type_traits>\n"
                        "#include \"omega2d_gb300_influence.hpp\"\n", 1)
    for head, call in GPU_BRANCH.items():
        assert text.count(head) == 1, head
        text = text.replace(head, head + "\n  if constexpr (std::is_same<S, float>::value) {\n"
                            "    if (env.get_instrs() == gpu_cuda) {\n      " + call + "\n      return;\n    }\n  }\n")
    (inc / "Influence.h").write_text(text)
    (tmp_path / "prog.cpp").write_text(REF_PROGRAM)
    te = tmp_path / "tinyexpr.o"
    r = subprocess.run(["gcc", "-O1", "-fPIC", "-c", os.path.join(build_ref.REF_ROOT, "lib", "tinyexpr", "tinyexpr.c"),
                        "-o", str(te)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    exe = tmp_path / "prog"
    cmd = ["g++", "-std=c++17", "-O1", "-fopenmp", "-DVERBOSE=false", "-w", "-I", str(inc),
           "-I", os.path.join(build_ref.REF_ROOT, "lib"), "-I", os.path.join(ROOT, "include"),
           str(tmp_path / "prog.cpp"), os.path.join(ref_src, "Body.cpp"), str(te), lib,
           "-Wl,-rpath," + os.path.dirname(lib), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    # without a GPU the first engine call reports the missing device; with one all four run
    last = out.stdout.strip().splitlines()[-1]
    assert last.startswith("ran ") or "obs_create" in last, out.stdout[-2000:]
