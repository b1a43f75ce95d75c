// obj.cpp — Wavefront OBJ ingestion and the reference's vertex normalisation.
//
// The reference loads a dropped .obj file with
// `tobj::load_obj(path, &LoadOptions { triangulate: true, ..Default })`,
// keeps `models[0].mesh` and passes its positions and indices to
// Application::load_model (src/main.rs:139-156,
// src/application.rs:199-226), which normalises the coordinates in place
// (src/vertices.rs:3-17) and takes the bounding-box centre for the arcball
// camera (src/vertices.rs:19-57, src/main_view.rs:460-488).
//
// tobj 4.0.2 (Cargo.lock:2898-2900) is not part of the reference's sources.
// This file restates its published behaviour for those options:
//  * the text is read line by line; each line is split on whitespace and the
//    first word selects the record; "#" and unknown records are skipped;
//  * "v x y z [r g b]" needs three floats (decimal, correctly rounded to
//    f32); a following colour is optional and ignored here;
//    "vt u v" needs two floats, "vn x y z" three;
//  * "f" and "l" take one vertex reference per word: "v", "v/vt", "v//vn" or
//    "v/vt/vn"; an index n > 0 is n - 1, n < 0 is relative to the records
//    read so far (count + n); a result of -1 (n = 0, or a relative index one
//    past the start) means "absent", which is an error for the position;
//  * "o" and "g" close the current model when it has faces;
//  * "usemtl name" closes the current model when it has faces and the named
//    material (looked up by its "newmtl" name in the "mtllib" files) differs
//    from the current one; unknown names are "no material";
//  * a model is exported (the default multi-index mesh): positions in the
//    order of their first reference, keyed by the position index, and
//    triangles from the faces: point a -> (a,a,a), line a b -> (a,b,b),
//    triangle as is, quad a b c d -> (a,b,c)(a,c,d), polygon -> a fan around
//    its first vertex; every reference is checked against the records read
//    when the model closes (texture / normal references only when that list
//    is not empty);
//  * after the last line the current model is exported even when it has no
//    faces, so a file always yields at least one model.
#include <cerrno>
#include <cfloat>
#include <cstdlib>
#include <memory>
#include <charconv>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "internal.hpp"

struct linon_mesh {
  std::vector<float> positions;  // n_vertices * 3
  std::vector<uint32_t> faces;   // n_faces * 3
  uint32_t n_models = 0;
  float center[3] = {0.0f, 0.0f, 0.0f};
};

namespace linon {
namespace {

constexpr int64_t kAbsent = -1;

struct VRef {
  int64_t v, vt, vn;
};

bool is_space(char c) { return c == ' ' || c == '\t' || c == '\r' || c == '\n' || c == '\v' || c == '\f'; }

// Rust's f32::from_str grammar: [+-]? (inf | infinity | nan | digits with an
// optional '.' and exponent), correctly rounded; nothing else.
bool parse_f32(const char* b, const char* e, float& out) {
  if (b == e) return false;
  const char* p = b;
  bool neg = false;
  if (*p == '+' || *p == '-') {
    neg = *p == '-';
    ++p;
  }
  if (p == e || *p == '+' || *p == '-') return false;
  for (const char* q = p; q != e; ++q)
    if (*q == '(' || *q == 'x' || *q == 'X' || *q == 'p' || *q == 'P') return false;
  float v = 0.0f;
  auto r = std::from_chars(p, e, v, std::chars_format::general);
  if (r.ec != std::errc() || r.ptr != e) {
    // from_chars reports out-of-range values as an error; Rust rounds them
    // to infinity or zero like any other decimal
    if (r.ec == std::errc::result_out_of_range && r.ptr == e) {
      std::string s(p, e);
      v = std::strtof(s.c_str(), nullptr);
    } else {
      return false;
    }
  }
  out = neg ? -v : v;
  return true;
}

// Rust's isize::from_str: [+-]? digits, no overflow.
bool parse_i64(const char* b, const char* e, int64_t& out) {
  if (b == e) return false;
  const char* p = b;
  if (*p == '+') {
    ++p;
    if (p == e || *p == '-' || *p == '+') return false;
  }
  auto r = std::from_chars(p, e, out, 10);
  return r.ec == std::errc() && r.ptr == e;
}

struct Token {
  const char* b;
  const char* e;
  bool is(const char* s) const {
    const size_t n = std::strlen(s);
    return size_t(e - b) == n && std::memcmp(b, s, n) == 0;
  }
};

class Parser {
 public:
  Parser(std::map<std::string, int>* materials, uint32_t want) : mats_(materials), want_(want) {}

  int run(const char* text, size_t len, linon_mesh& out) {
    const char* p = text;
    const char* end = text + len;
    line_no_ = 0;
    while (p < end) {
      const char* nl = static_cast<const char*>(std::memchr(p, '\n', size_t(end - p)));
      const char* le = nl ? nl : end;
      ++line_no_;
      if (int st = line(p, le, out)) return st;
      p = nl ? nl + 1 : end;
    }
    if (int st = close_model(out)) return st;
    out.n_models = n_models_;
    if (!found_) return set_error(LINON_EINVAL, "obj: model " + std::to_string(want_) + " requested, file has " +
                                                    std::to_string(n_models_));
    return LINON_OK;
  }

 private:
  std::map<std::string, int>* mats_;
  uint32_t want_;
  size_t line_no_ = 0;
  std::vector<float> pos_;
  size_t n_tex_ = 0, n_norm_ = 0;
  std::vector<VRef> refs_;         // vertex references of the current model's faces
  std::vector<uint32_t> arity_;    // references per face
  int material_ = -1;              // -1: none
  uint32_t n_models_ = 0;
  bool found_ = false;
  std::vector<uint32_t> local_, stamp_;

  int fail(const std::string& what) {
    return set_error(LINON_EINVAL, "obj line " + std::to_string(line_no_) + ": " + what);
  }

  static std::vector<Token> split(const char* b, const char* e) {
    std::vector<Token> w;
    const char* p = b;
    while (p < e) {
      while (p < e && is_space(*p)) ++p;
      if (p == e) break;
      const char* s = p;
      while (p < e && !is_space(*p)) ++p;
      w.push_back({s, p});
    }
    return w;
  }

  static std::string rest_trimmed(const char* b, const char* e, size_t skip) {
    const char* p = b;
    while (p < e && is_space(*p)) ++p;
    p += skip;
    if (p > e) p = e;
    while (p < e && is_space(*p)) ++p;
    const char* q = e;
    while (q > p && is_space(q[-1])) --q;
    return std::string(p, q);
  }

  int floats(const std::vector<Token>& w, size_t n, std::vector<float>* dst, const char* what) {
    if (w.size() < n + 1) return fail(std::string("expected ") + std::to_string(n) + " numbers in '" + what + "'");
    for (size_t i = 1; i <= n; ++i) {
      float v;
      if (!parse_f32(w[i].b, w[i].e, v))
        return fail(std::string("bad number '") + std::string(w[i].b, w[i].e) + "' in '" + what + "'");
      if (dst) dst->push_back(v);
    }
    return LINON_OK;
  }

  int face(const std::vector<Token>& w) {
    const int64_t n_pos = int64_t(pos_.size() / 3);
    uint32_t k = 0;
    for (size_t i = 1; i < w.size(); ++i) {
      VRef r{kAbsent, kAbsent, kAbsent};
      int64_t* slot[3] = {&r.v, &r.vt, &r.vn};
      const int64_t sizes[3] = {n_pos, int64_t(n_tex_), int64_t(n_norm_)};
      int part = 0;
      const char* s = w[i].b;
      while (true) {
        const char* slash = s;
        while (slash < w[i].e && *slash != '/') ++slash;
        if (part > 2) return fail("more than three indices in '" + std::string(w[i].b, w[i].e) + "'");
        if (slash > s) {
          int64_t x;
          if (!parse_i64(s, slash, x)) return fail("bad index '" + std::string(w[i].b, w[i].e) + "'");
          *slot[part] = x < 0 ? sizes[part] + x : x - 1;
        }
        if (slash == w[i].e) break;
        s = slash + 1;
        ++part;
      }
      refs_.push_back(r);
      ++k;
    }
    if (k == 0) return fail("face without vertices");
    arity_.push_back(k);
    return LINON_OK;
  }

  void emit(linon_mesh& out, const VRef& r) {
    const size_t v = size_t(r.v);
    if (stamp_[v] != n_models_ + 1) {
      stamp_[v] = n_models_ + 1;
      local_[v] = uint32_t(out.positions.size() / 3);
      out.positions.push_back(pos_[3 * v]);
      out.positions.push_back(pos_[3 * v + 1]);
      out.positions.push_back(pos_[3 * v + 2]);
    }
    out.faces.push_back(local_[v]);
  }

  // Exports the current model (checks it; builds it when it is the one asked for).
  int close_model(linon_mesh& out) {
    const int64_t n_pos = int64_t(pos_.size() / 3);
    for (const VRef& r : refs_) {
      if (r.v < 0 || r.v >= n_pos) return fail("face references a position that does not exist (model " +
                                               std::to_string(n_models_) + ")");
      if (n_tex_ && r.vt != kAbsent && (r.vt < 0 || r.vt >= int64_t(n_tex_)))
        return fail("face references a texture coordinate that does not exist");
      if (n_norm_ && r.vn != kAbsent && (r.vn < 0 || r.vn >= int64_t(n_norm_)))
        return fail("face references a normal that does not exist");
    }
    if (n_models_ == want_) {
      found_ = true;
      out.positions.clear();
      out.faces.clear();
      if (stamp_.size() < size_t(n_pos)) {
        stamp_.resize(size_t(n_pos), 0);
        local_.resize(size_t(n_pos), 0);
      }
      size_t at = 0;
      for (uint32_t a : arity_) {
        const VRef* f = refs_.data() + at;
        at += a;
        if (a == 1) {
          emit(out, f[0]), emit(out, f[0]), emit(out, f[0]);
        } else if (a == 2) {
          emit(out, f[0]), emit(out, f[1]), emit(out, f[1]);
        } else {
          for (uint32_t j = 1; j + 1 < a; ++j) emit(out, f[0]), emit(out, f[j]), emit(out, f[j + 1]);
        }
      }
    }
    ++n_models_;
    refs_.clear();
    arity_.clear();
    return LINON_OK;
  }

  int line(const char* b, const char* e, linon_mesh& out) {
    const char* p = b;
    while (p < e && is_space(*p)) ++p;
    if (p == e) return LINON_OK;
    const std::vector<Token> w = split(p, e);
    const Token& k = w[0];
    if (k.is("#")) return LINON_OK;
    if (k.is("v")) return floats(w, 3, &pos_, "v");
    if (k.is("vt")) {
      if (int st = floats(w, 2, nullptr, "vt")) return st;
      ++n_tex_;
      return LINON_OK;
    }
    if (k.is("vn")) {
      if (int st = floats(w, 3, nullptr, "vn")) return st;
      ++n_norm_;
      return LINON_OK;
    }
    if (k.is("f") || k.is("l")) return face(w);
    if (k.is("o") || k.is("g")) return refs_.empty() ? LINON_OK : close_model(out);
    if (k.is("usemtl")) {
      const std::string name = rest_trimmed(p, e, 6);
      if (name.empty()) return fail("usemtl without a name");
      int id = -1;
      if (mats_) {
        auto it = mats_->find(name);
        if (it != mats_->end()) id = it->second;
      }
      if (id != material_ && !refs_.empty())
        if (int st = close_model(out)) return st;
      material_ = id;
      return LINON_OK;
    }
    return LINON_OK;  // mtllib is read before parsing; everything else is ignored
  }
};

bool read_all(const std::string& path, std::string& out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::ostringstream s;
  s << f.rdbuf();
  out = s.str();
  return !f.bad();
}

// "newmtl name" records of every "mtllib" file, in file order; a material's
// id is its position in the concatenated list (a repeated name takes the
// later id), as tobj's material map does.
void load_materials(const char* text, size_t len, const std::string& dir, std::map<std::string, int>& mats) {
  int next = 0;
  const char* p = text;
  const char* end = text + len;
  while (p < end) {
    const char* nl = static_cast<const char*>(std::memchr(p, '\n', size_t(end - p)));
    const char* le = nl ? nl : end;
    const char* q = p;
    while (q < le && is_space(*q)) ++q;
    if (le - q > 6 && std::memcmp(q, "mtllib", 6) == 0 && is_space(q[6])) {
      const char* s = q + 6;
      while (s < le && is_space(*s)) ++s;
      const char* t = le;
      while (t > s && is_space(t[-1])) --t;
      std::string name(s, t), body;
      const std::string path = (!name.empty() && name[0] == '/') || dir.empty() ? name : dir + "/" + name;
      if (!name.empty() && read_all(path, body)) {
        std::istringstream is(body);
        std::string ln;
        while (std::getline(is, ln)) {
          size_t a = ln.find_first_not_of(" \t\r\v\f");
          if (a == std::string::npos || ln.compare(a, 6, "newmtl") != 0) continue;
          if (a + 6 < ln.size() && !is_space(ln[a + 6])) continue;
          size_t b = ln.find_first_not_of(" \t\r\v\f", a + 6);
          size_t c = ln.find_last_not_of(" \t\r\v\f");
          if (b == std::string::npos || c < b) continue;
          mats[ln.substr(b, c - b + 1)] = next++;
        }
      }
    }
    p = nl ? nl + 1 : end;
  }
}

void center_of(const float* v, size_t n_floats, float c[3]) {
  float lo[3] = {v[0], v[1], v[2]}, hi[3] = {v[0], v[1], v[2]};
  for (size_t i = 1; i < n_floats / 3; ++i)
    for (int k = 0; k < 3; ++k) {
      const float x = v[3 * i + k];
      if (x < lo[k]) lo[k] = x;
      if (x > hi[k]) hi[k] = x;
    }
  for (int k = 0; k < 3; ++k) c[k] = (lo[k] + hi[k]) / 2.0f;
}

void normalize(float* v, size_t n) {
  float mx = -FLT_MAX, mn = FLT_MAX;
  for (size_t i = 0; i < n; ++i) {
    if (v[i] > mx) mx = v[i];
    if (v[i] < mn) mn = v[i];
  }
  for (size_t i = 0; i < n; ++i) v[i] = (v[i] - mn) / (mx - mn) * 2.0f - 1.0f;
}

int parse_into(const char* text, size_t len, const std::string& mtl_dir, bool read_mtl, uint32_t model,
               uint32_t flags, linon_mesh** out) {
  if (!out) return set_error(LINON_EINVAL, "null output");
  *out = nullptr;
  if (!text && len) return set_error(LINON_EINVAL, "null text");
  if (flags & ~uint32_t(LINON_OBJ_NORMALIZE)) return set_error(LINON_EINVAL, "unknown obj flags");
  std::map<std::string, int> mats;
  if (read_mtl) load_materials(text, len, mtl_dir, mats);
  auto m = std::make_unique<linon_mesh>();
  Parser P(read_mtl ? &mats : nullptr, model);
  if (int st = P.run(text ? text : "", len, *m)) return st;
  if (flags & LINON_OBJ_NORMALIZE) normalize(m->positions.data(), m->positions.size());
  if (!m->positions.empty()) center_of(m->positions.data(), m->positions.size(), m->center);
  *out = m.release();
  return LINON_OK;
}

}  // namespace
}  // namespace linon

using namespace linon;

int linon_obj_load(const char* path, uint32_t model, uint32_t flags, linon_mesh** out) {
  LINON_TRY_BEGIN
  if (out) *out = nullptr;
  if (!path) return set_error(LINON_EINVAL, "null path");
  std::string text;
  if (!read_all(path, text)) return set_error(LINON_EIO, std::string("cannot read ") + path);
  std::string dir(path);
  const size_t slash = dir.find_last_of('/');
  dir = slash == std::string::npos ? std::string() : dir.substr(0, slash);
  return parse_into(text.data(), text.size(), dir, true, model, flags, out);
  LINON_TRY_END
}

int linon_obj_parse(const char* text, size_t len, const char* mtl_dir, uint32_t model, uint32_t flags,
                    linon_mesh** out) {
  LINON_TRY_BEGIN
  return parse_into(text, len, mtl_dir ? mtl_dir : "", mtl_dir != nullptr, model, flags, out);
  LINON_TRY_END
}

int linon_mesh_info(const linon_mesh* m, uint32_t* n_vertices, uint32_t* n_faces, uint32_t* n_models,
                    float center[3]) {
  if (!m) return set_error(LINON_EINVAL, "null mesh");
  if (n_vertices) *n_vertices = uint32_t(m->positions.size() / 3);
  if (n_faces) *n_faces = uint32_t(m->faces.size() / 3);
  if (n_models) *n_models = m->n_models;
  if (center) std::memcpy(center, m->center, sizeof m->center);
  return LINON_OK;
}

const float* linon_mesh_positions(const linon_mesh* m) { return m ? m->positions.data() : nullptr; }

const uint32_t* linon_mesh_faces(const linon_mesh* m) { return m ? m->faces.data() : nullptr; }

void linon_mesh_free(linon_mesh* m) { delete m; }

int linon_normalize_vertices(float* xyz, size_t n_floats, float center[3]) {
  if (n_floats && !xyz) return set_error(LINON_EINVAL, "null vertices");
  if (center && n_floats < 3) return set_error(LINON_EINVAL, "get_center needs at least one vertex");
  normalize(xyz, n_floats);
  if (center) center_of(xyz, n_floats, center);
  return LINON_OK;
}
