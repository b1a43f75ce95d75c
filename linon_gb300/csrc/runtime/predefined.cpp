// predefined.cpp — the predefined field-function bodies offered to users.
//
// Ids 1-9 are the set of src/functions.rs:1-128 (PredefinedFunction::to_code,
// display names from :15-30); the WGSL text is the same because it is the
// user-visible API of that set.  Id 10 is the stub body of
// src/main_view.wgsl:148, ids 11-14 are the field functions of the benchmark
// workloads (linear, twist, point lens, scaled Lorenz).
#include "../../../include/linon.h"

namespace {

struct Predef {
  const char* name;
  const char* body;
};

const Predef kPredef[LINON_FIELD_COUNT] = {
    {"Custom", ""},
    {"Mirage (spherical)",
     "let t_env = 15.0; // °C\n"
     "let t_src = 200.0; // °C\n"
     "let max_dist = 0.25;\n"
     "let center = vec3<f32>(-0.5, 0.5, -0.5);\n"
     "\n"
     "let center_dest = p - center;\n"
     "let normal = normalize(center_dest);\n"
     "let dist_in = length(p_prev - center);\n"
     "let dist_out = length(center_dest);\n"
     "let part_in = clamp(0.0, 1.0, dist_in / max_dist);\n"
     "let part_out = clamp(0.0, 1.0, dist_out / max_dist);\n"
     "let t_in = part_in * t_env + (1.0 - part_in) * t_src;\n"
     "let t_out = part_out * t_env + (1.0 - part_out) * t_src;\n"
     "\n"
     "return refraction(t_in, t_out, v, normal);"},
    {"Mirage (plane)",
     "let t_env = 15.0; // °C\n"
     "let t_src = 30.0; // °C\n"
     "let max_dist = 0.01;\n"
     "let plane_p0 = vec3<f32>(0.0, 0.1, 0.0);\n"
     "let plane_n = vec3<f32>(0.0, 1.0, 0.0);\n"
     "\n"
     "let dist_in = point_plane_distance(p_prev, plane_n, plane_p0);\n"
     "let dist_out = point_plane_distance(p, plane_n, plane_p0);\n"
     "let part_in = clamp(0.0, 1.0, dist_in / max_dist);\n"
     "let part_out = clamp(0.0, 1.0, dist_out / max_dist);\n"
     "let t_in = part_in * t_env + (1.0 - part_in) * t_src;\n"
     "let t_out = part_out * t_env + (1.0 - part_out) * t_src;\n"
     "\n"
     "return refraction(t_in, t_out, v, plane_n);"},
    {"Mirage (spherical sigmoid)",
     "let t_env = 15.0; // °C\n"
     "let t_src = 200.0; // °C\n"
     "let max_dist = 0.25;\n"
     "let center = vec3<f32>(-0.5, 0.5, -0.5);\n"
     "\n"
     "let center_dest = p - center;\n"
     "let normal = normalize(center_dest);\n"
     "let dist_in = length(p_prev - center);\n"
     "let dist_out = length(center_dest);\n"
     "let part_in = clamp(0.0, 1.0, sigmoid(dist_in / max_dist * 12.0 - 6.0));\n"
     "let part_out = clamp(0.0, 1.0, sigmoid(dist_out / max_dist * 12.0 - 6.0));\n"
     "let t_in = part_in * t_env + (1.0 - part_in) * t_src;\n"
     "let t_out = part_out * t_env + (1.0 - part_out) * t_src;\n"
     "\n"
     "return refraction(t_in, t_out, v, normal);"},
    {"Mirage (plane sigmoid)",
     "let t_env = 15.0; // °C\n"
     "let t_src = 30.0; // °C\n"
     "let max_dist = 0.01;\n"
     "let plane_p0 = vec3<f32>(0.0, 0.1, 0.0);\n"
     "let plane_n = vec3<f32>(0.0, 1.0, 0.0);\n"
     "\n"
     "let dist_in = point_plane_distance(p_prev, plane_n, plane_p0);\n"
     "let dist_out = point_plane_distance(p, plane_n, plane_p0);\n"
     "let part_in = clamp(0.0, 1.0, sigmoid(dist_in / max_dist * 12.0 - 6.0));\n"
     "let part_out = clamp(0.0, 1.0, sigmoid(dist_out / max_dist * 12.0 - 6.0));\n"
     "let t_in = part_in * t_env + (1.0 - part_in) * t_src;\n"
     "let t_out = part_out * t_env + (1.0 - part_out) * t_src;\n"
     "\n"
     "return refraction(t_in, t_out, v, plane_n);"},
    {"Translation (x-axis)",
     "let dx = 0.5 * t;\n"
     "let dy = 0.0;\n"
     "let dz = 0.0;\n"
     "return translate(v0, dx, dy, dz);"},
    {"Translation (z-axis)",
     "let dx = 0.0;\n"
     "let dy = 0.0;\n"
     "let dz = 0.5 * t;\n"
     "return translate(v0, dx, dy, dz);"},
    {"Rotation", "return normalize(v0 + rotateZ(v0, PI * t));"},
    {"Lorenz attractor",
     "let rho = 28.0;\n"
     "let sigma = 10.0;\n"
     "let beta = 8.0 / 3.0;\n"
     "return vec3<f32>(\n"
     "    sigma * (p.y - p.x),\n"
     "    p.x * (rho - p.z) - p.y,\n"
     "    p.x * p.y - beta * p.z,\n"
     ");"},
    {"Roessler attractor",
     "let a = 0.1;\n"
     "let b = 0.1;\n"
     "let c = 14.0;\n"
     "return vec3<f32>(\n"
     "    -p.y - p.z,\n"
     "    p.x + a * p.y,\n"
     "    b + p.z * (p.x - c),\n"
     ");"},
    {"Identity (shader stub)", "return v;"},
    {"Linear", "return v0;"},
    {"Twist", "return rotateY(v0, 0.5 * p.y);"},
    {"Point lens", "return normalize(v - 0.05 * p / pow(dot(p, p) + 0.01, 1.5));"},
    {"Lorenz (scaled) + v0",
     "let sigma = 10.0;\n"
     "let rho = 28.0;\n"
     "let beta = 8.0 / 3.0;\n"
     "return 0.05 * vec3<f32>(\n"
     "    sigma * (p.y - p.x),\n"
     "    p.x * (rho - p.z) - p.y,\n"
     "    p.x * p.y - beta * p.z,\n"
     ") + v0;"},
};

}  // namespace

extern "C" const char* linon_predefined_source(int id) {
  if (id < 0 || id >= LINON_FIELD_COUNT) return nullptr;
  return kPredef[id].body;
}

extern "C" const char* linon_predefined_name(int id) {
  if (id < 0 || id >= LINON_FIELD_COUNT) return nullptr;
  return kPredef[id].name;
}
