// omega2d_gb300_influence.hpp -- header-only C++ adapters with the reference's driver shapes.
//
// Drop these calls into the reference's drivers (src/Influence.h) behind
// `env.get_instrs() == gpu_cuda` (the unused enum value at src/ExecEnv.h:38).  They take any
// element container with the reference's accessors -- get_n(), is_inert(), get_pos(),
// get_rad(), get_str(), get_vel(), get_vort(), get_shear() (src/ElementBase.h:50-115,
// src/Points.h:116-117) -- so the reference's Points<float> work unchanged.
#pragma once

#include <cstdio>
#include <stdexcept>
#include <string>

#include "omega2d_gb300.h"

namespace omega2d_gb300 {

// The core the reference was compiled with (src/CoreFunc.h:35-39), as an engine enum.
inline int compiled_core() {
#if defined(USE_RM_KERNEL)
  return OBS_CORE_RM;
#elif defined(USE_EXPONENTIAL_KERNEL)
  return OBS_CORE_GAUSSIAN;
#elif defined(USE_WL_KERNEL)
  return OBS_CORE_WL;
#elif defined(USE_V3_KERNEL)
  return OBS_CORE_V3;
#else
  return OBS_CORE_V2;
#endif
}

// The engine takes straight panels: two node indices per panel.  The reference also allows
// more nodes per element (src/Reflect.h:512 reads idx[nper*j]); such surfaces are rejected
// here rather than read with the wrong stride.
template <class Surf>
inline void require_two_nodes_per_panel(const Surf& s, const char* who) {
  if (s.get_idx().size() != 2 * (size_t)s.get_npanels())
    throw std::runtime_error(std::string(who) + ": the engine takes two node indices per panel");
}

// One context per process and device, created on first use.
inline obs_context* context(int device = 0) {
  static obs_context* ctx = nullptr;
  if (!ctx) {
    const int s = obs_create(&ctx, device);
    if (s != OBS_OK) throw std::runtime_error(std::string("obs_create: ") + obs_status_string(s));
  }
  return ctx;
}

// Mirror of points_affect_points<float,A>(src, targ, restype, env) (src/Influence.h:56-416):
// accumulates the unscaled influence of src on targ.  result is a results_t value.
// Returns the reference's flop count for the call.
template <class SrcPoints, class TargPoints>
float points_affect_points(const SrcPoints& src, TargPoints& targ, int result,
                           int core = compiled_core(), int accum = OBS_COMPENSATED) {
  const auto& sx = src.get_pos();
  const auto& sr = src.get_rad();
  const auto& ss = src.get_str();
  const auto& tx = targ.get_pos();
  auto& tu = targ.get_vel();
  const float* tr = targ.is_inert() ? nullptr : targ.get_rad().data();
  float* e0 = nullptr;
  if (result == OBS_VELANDVORT) e0 = targ.get_vort().data();
  if (result == OBS_VELANDSHEAR) e0 = targ.get_shear().data();
  double flops = 0.0;
  const int s = obs_points_affect_points(context(), core, result, accum, 0, 0.0, 0.0,
                                         (int)src.get_n(), sx[0].data(), sx[1].data(), sr.data(), ss.data(),
                                         (int)targ.get_n(), tx[0].data(), tx[1].data(), tr,
                                         tu[0].data(), tu[1].data(), e0, nullptr, nullptr, nullptr, &flops);
  if (s != OBS_OK) throw std::runtime_error(std::string("obs_points_affect_points: ") + obs_status_string(s));
  return (float)flops;
}

// Mirror of panels_affect_points<float,A>(src, targ, restype, env) (src/Influence.h:422-614):
// accumulates the unscaled velocity of the panels' vortex sheets (and source sheets, when the
// surface has source strengths) at the points.  Surfaces accessors: get_pos() (nodes),
// get_idx() (two 32-bit node indices per panel), get_npanels(), get_str(), have_src_str(),
// get_src_str() (src/Surfaces.h:231-252).
template <class SrcSurfaces, class TargPoints>
void panels_affect_points(const SrcSurfaces& src, TargPoints& targ, int accum = OBS_COMPENSATED) {
  require_two_nodes_per_panel(src, "panels_affect_points");
  const auto& nx = src.get_pos();
  const auto& idx = src.get_idx();
  static_assert(sizeof(idx[0]) == sizeof(unsigned), "panel node indices must be 32-bit");
  const float* ss = src.have_src_str() ? src.get_src_str().data() : nullptr;
  const auto& tx = targ.get_pos();
  auto& tu = targ.get_vel();
  const int s = obs_panels_affect_points(context(), accum, 0, 0.0, 0.0, (int)nx[0].size(), nx[0].data(), nx[1].data(),
                                         (int)src.get_npanels(), reinterpret_cast<const unsigned*>(idx.data()),
                                         src.get_str().data(), ss, (int)targ.get_n(), tx[0].data(), tx[1].data(),
                                         tu[0].data(), tu[1].data());
  if (s != OBS_OK) throw std::runtime_error(std::string("obs_panels_affect_points: ") + obs_status_string(s));
}

// Mirror of points_affect_panels<float,A>(src, targ, restype, env) (src/Influence.h:633-771):
// accumulates into each panel's velocity the mean velocity of the point vortices over the
// panel (the BEM right-hand-side input; the points' core radii are ignored, as there).
template <class SrcPoints, class TargSurfaces>
void points_affect_panels(const SrcPoints& src, TargSurfaces& targ, int accum = OBS_COMPENSATED) {
  require_two_nodes_per_panel(targ, "points_affect_panels");
  const auto& sx = src.get_pos();
  const auto& nx = targ.get_pos();
  const auto& idx = targ.get_idx();
  static_assert(sizeof(idx[0]) == sizeof(unsigned), "panel node indices must be 32-bit");
  auto& pu = targ.get_vel();
  const int s = obs_points_affect_panels(context(), accum, 0, 0.0, 0.0, (int)src.get_n(), sx[0].data(), sx[1].data(),
                                         src.get_str().data(), (int)nx[0].size(), nx[0].data(), nx[1].data(),
                                         (int)targ.get_npanels(), reinterpret_cast<const unsigned*>(idx.data()),
                                         pu[0].data(), pu[1].data());
  if (s != OBS_OK) throw std::runtime_error(std::string("obs_points_affect_panels: ") + obs_status_string(s));
}

// Mirror of clear_inner_panp2<float>(method, src, targ, cutoff_mult, ips) (src/Reflect.h:491-729):
// crops (method 0) or pushes (method 1) the points inside the body's cutoff layer, in place, and
// returns the circulation removed, which clear_inner_layer hands to the body's
// add_to_reabsorbed (:733-760).  Points without radii (field points) take ips as radius.
// When a point still lies inside the layer after the engine's sweep limit, the points are
// updated as far as they went and the circulation removed is returned with a warning on
// stderr, so the caller's circulation bookkeeping stays whole.
template <class SrcSurfaces, class TargPoints>
float clear_inner_panp2(int method, const SrcSurfaces& src, TargPoints& targ, float cutoff_mult, float ips) {
  require_two_nodes_per_panel(src, "clear_inner_panp2");
  const auto& nx = src.get_pos();
  const auto& idx = src.get_idx();
  static_assert(sizeof(idx[0]) == sizeof(unsigned), "panel node indices must be 32-bit");
  auto& tx = targ.get_pos();
  auto& ts = targ.get_str();
  const auto& tr = targ.get_rad();
  double lost = 0.0;
  long long ncropped = 0;
  const int s = obs_clear_inner_layer(context(), method, cutoff_mult, ips, (int)nx[0].size(), nx[0].data(),
                                      nx[1].data(), (int)src.get_npanels(),
                                      reinterpret_cast<const unsigned*>(idx.data()), (int)tx[0].size(),
                                      tx[0].data(), tx[1].data(), ts.empty() ? nullptr : ts.data(),
                                      tr.empty() ? nullptr : tr.data(), &lost, &ncropped);
  if (s == OBS_ERR_NO_CONVERGENCE) {
    // the sweep limit ran out for some points: positions, strengths and the circulation
    // removed are written all the same, so hand the circulation back for add_to_reabsorbed
    std::fprintf(stderr, "omega2d_gb300::clear_inner_panp2: %s; the circulation removed is returned\n",
                 obs_status_string(s));
    return (float)lost;
  }
  if (s != OBS_OK) throw std::runtime_error(std::string("obs_clear_inner_layer: ") + obs_status_string(s));
  return (float)lost;
}

}  // namespace omega2d_gb300
