// frontend.hpp — WGSL-subset front end: field-function source -> CUDA C.
//
// Replaces the naga path of the reference (src/main_view.rs:649-690, which
// splices the user body into the shader with with_field_function,
// src/main_view.rs:852-861, and lets naga parse and validate it).  The input
// is the body of
//   fn field_function(p_prev: vec3<f32>, p: vec3<f32>, v0: vec3<f32>,
//                     v: vec3<f32>, t: f32) -> vec3<f32>
// plus optional module-scope helper functions and constants.  The output is
// CUDA C written against device/wgsl_rt.cuh.
#pragma once

#include <string>

namespace linon {
namespace wgslfe {

struct Translation {
  bool ok = false;
  std::string code;      // CUDA C: namespace <ns> { ... field_function ... }
  std::string log;       // diagnostics (errors) when !ok
  int flops_arith = 0;   // counted FP32 add/mul/div/sqrt of one evaluation
  int flops_transc = 0;  // transcendental calls of one evaluation
  bool has_private = false;  // the module declares var<private> state
};

// ns: C++ namespace that receives the generated functions; the field is
// ns::field_function(ns::Private& pv, vec3f p_prev, vec3f p, vec3f v0,
// vec3f v, float t), where ns::Private holds the module's var<private>
// variables (an empty struct when there are none): one Private per
// invocation, i.e. per ray.  pair = true emits the same functions with every
// f32 value a ::wgsl::f2 (two rays' values, evaluated with packed FP32
// pairs; see device/wgsl_rt.cuh): field_function(Private&, vec<f2,3> p_prev,
// vec<f2,3> p, vec<f2,3> v0, vec<f2,3> v, f2 t).  Integer and boolean values
// stay scalar in pair form, which is right for values that cannot depend on
// the ray (no f2 converts to them) but not for var<private> state, so the
// engine gives fields with private state no pair form.
Translation translate(const std::string& field_body, const std::string& helpers_src,
                      const std::string& ns, bool pair = false);

}  // namespace wgslfe
}  // namespace linon
