// frontend.cpp — WGSL-subset front end for linon field functions.
//
// Pipeline: lexer -> recursive-descent parser (AST) -> checker that resolves
// names and types (with WGSL's AbstractInt / AbstractFloat constants folded in
// double precision, as WGSL const-evaluates them) while counting FP32
// operations -> CUDA C emitter against device/wgsl_rt.cuh.
//
// Coverage: everything in src/functions.rs:33-128 and in the helper section of
// src/main_view.wgsl:76-146: let/var/const, f32/i32/u32/bool scalars,
// vecN<T> and matCxR<f32> constructors and arithmetic, swizzles, indexing,
// if/else, for/while/loop, break/continue/return, compound assignment,
// the WGSL numeric builtins and the linon helpers.  User helper functions and
// module-scope constants may precede the field body (README.md:46).
#include "frontend.hpp"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <cstdint>
#include <set>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace linon {
namespace wgslfe {
namespace {

// ===========================================================================
// types
// ===========================================================================
enum class SK { Bool, I32, U32, F32, AInt, AFloat };

struct Ty {
  enum Cat { Void, Scalar, Vec, Mat, Arr, Struct, Ptr } cat = Void;  // Ptr: ptr<function, T>
  SK s = SK::F32;
  int n = 0;  // vector size / matrix columns (of the element, for arrays)
  int r = 0;  // matrix rows (of the element, for arrays)
  // arrays: fixed-size array<E, alen> of scalar, vector, matrix or struct
  // elements
  Cat ecat = Void;
  int alen = 0;
  int sid = -1;  // struct (or array-of-struct element) index
  int eid = -1;  // arrays of arrays: the element type; pointers: the pointee (g_arr_elems)
};

// Struct declarations of the module being translated (one translation per
// thread at a time).
struct StructDef {
  std::string name;
  int line = 0, col = 0;
  std::vector<std::pair<std::string, Ty>> members;
  std::string cpp;  // built-in result structs (frexp, modf): the runtime's type
};
thread_local std::vector<StructDef>* g_structs = nullptr;
// Element types of arrays whose elements are arrays (one entry per distinct
// type, so equal types share an index).
thread_local std::vector<Ty>* g_arr_elems = nullptr;
int struct_id(const std::string& n) {
  if (!g_structs) return -1;
  for (size_t i = 0; i < g_structs->size(); ++i)
    if ((*g_structs)[i].name == n) return int(i);
  return -1;
}

Ty scalar(SK s) { Ty t; t.cat = Ty::Scalar; t.s = s; return t; }
Ty vecT(SK s, int n) { Ty t; t.cat = Ty::Vec; t.s = s; t.n = n; return t; }
Ty matT(int c, int r) { Ty t; t.cat = Ty::Mat; t.s = SK::F32; t.n = c; t.r = r; return t; }
Ty voidT() { return Ty(); }
bool operator==(const Ty& a, const Ty& b) {
  return a.cat == b.cat && (a.cat == Ty::Void || (a.s == b.s && a.n == b.n && a.r == b.r && a.ecat == b.ecat &&
                                                  a.alen == b.alen && a.sid == b.sid && a.eid == b.eid));
}
int intern_elem(const Ty& el) {
  for (size_t i = 0; i < g_arr_elems->size(); ++i)
    if ((*g_arr_elems)[i] == el) return int(i);
  g_arr_elems->push_back(el);
  return int(g_arr_elems->size()) - 1;
}
Ty arrT(const Ty& el, int len) {
  if (el.cat == Ty::Arr) {  // array of arrays: the element type by reference
    Ty t;
    t.cat = Ty::Arr;
    t.ecat = Ty::Arr;
    t.alen = len;
    t.eid = intern_elem(el);
    return t;
  }
  Ty t = el;
  t.ecat = el.cat;
  t.cat = Ty::Arr;
  t.alen = len;
  t.eid = -1;
  return t;
}
Ty elemT(const Ty& a) {
  if (a.ecat == Ty::Arr) return (*g_arr_elems)[size_t(a.eid)];
  Ty t = a;
  t.cat = a.ecat;
  t.ecat = Ty::Void;
  t.alen = 0;
  return t;
}
Ty ptrT(const Ty& pointee) {
  Ty t;
  t.cat = Ty::Ptr;
  t.eid = intern_elem(pointee);
  return t;
}
Ty pointeeT(const Ty& p) { return (*g_arr_elems)[size_t(p.eid)]; }
// the struct at the bottom of nested arrays (or the struct itself), or -1
int inner_struct(Ty t) {
  while (t.cat == Ty::Arr) t = elemT(t);
  return t.cat == Ty::Struct ? t.sid : -1;
}
bool operator!=(const Ty& a, const Ty& b) { return !(a == b); }

bool is_abstract(SK s) { return s == SK::AInt || s == SK::AFloat; }
bool is_float(SK s) { return s == SK::F32 || s == SK::AFloat; }
bool is_int(SK s) { return s == SK::I32 || s == SK::U32 || s == SK::AInt; }
bool is_numeric(SK s) { return s != SK::Bool; }

const char* sk_name(SK s) {
  switch (s) {
    case SK::Bool: return "bool";
    case SK::I32: return "i32";
    case SK::U32: return "u32";
    case SK::F32: return "f32";
    case SK::AInt: return "AbstractInt";
    case SK::AFloat: return "AbstractFloat";
  }
  return "?";
}
std::string wgsl_name(const Ty& t) {
  switch (t.cat) {
    case Ty::Void: return "void";
    case Ty::Scalar: return sk_name(t.s);
    case Ty::Vec: return "vec" + std::to_string(t.n) + "<" + sk_name(t.s) + ">";
    case Ty::Mat: return "mat" + std::to_string(t.n) + "x" + std::to_string(t.r) + "<f32>";
    case Ty::Arr: return "array<" + wgsl_name(elemT(t)) + ", " + std::to_string(t.alen) + ">";
    case Ty::Ptr: return "ptr<function, " + wgsl_name(pointeeT(t)) + ">";
    case Ty::Struct: return g_structs && t.sid >= 0 ? (*g_structs)[size_t(t.sid)].name : "struct";
  }
  return "?";
}
// Pair emission (translate(..., pair = true)): every f32 value becomes a
// ::wgsl::f2, the same value of two rays, so that one thread evaluates the
// field for two rays with packed FP32 pair instructions.  Literals stay
// float (they broadcast); anything that is not lane-wise in an f2 (a
// comparison, a branch on a value, a conversion to an integer) has no f2
// overload and fails to compile, and the engine then uses the one-ray
// kernels.
thread_local bool g_pair = false;
const char* sk_cpp(SK s) {
  switch (s) {
    case SK::Bool: return "bool";
    case SK::I32: case SK::AInt: return "int";
    case SK::U32: return "unsigned";
    case SK::F32: case SK::AFloat: return g_pair ? "::wgsl::f2" : "float";
  }
  return "?";
}
std::string cpp_name(const Ty& t) {
  switch (t.cat) {
    case Ty::Void: return "void";
    case Ty::Scalar: return sk_cpp(t.s);
    case Ty::Vec: return std::string("::wgsl::vec<") + sk_cpp(t.s) + "," + std::to_string(t.n) + ">";
    case Ty::Mat: return "::wgsl::mat<" + std::to_string(t.n) + "," + std::to_string(t.r) + ">";
    case Ty::Arr: return "::wgsl::arr<" + cpp_name(elemT(t)) + "," + std::to_string(t.alen) + ">";
    case Ty::Ptr: return cpp_name(pointeeT(t)) + "&";
    case Ty::Struct:
      if (g_structs && t.sid >= 0 && !(*g_structs)[size_t(t.sid)].cpp.empty()) return (*g_structs)[size_t(t.sid)].cpp;
      return "s_" + (g_structs && t.sid >= 0 ? (*g_structs)[size_t(t.sid)].name : std::string("?"));
  }
  return "?";
}

bool convertible(SK from, SK to) {
  if (from == to) return true;
  if (from == SK::AInt) return to == SK::I32 || to == SK::U32 || to == SK::F32 || to == SK::AFloat;
  if (from == SK::AFloat) return to == SK::F32;
  return false;
}
bool unify_sk(SK a, SK b, SK& out) {
  if (a == b) { out = a; return true; }
  if (convertible(a, b)) { out = b; return true; }
  if (convertible(b, a)) { out = a; return true; }
  return false;
}
SK concrete_sk(SK s) {
  if (s == SK::AInt) return SK::I32;
  if (s == SK::AFloat) return SK::F32;
  return s;
}
Ty concretize(Ty t) {
  if (t.cat == Ty::Arr && t.ecat == Ty::Arr) return arrT(concretize(elemT(t)), t.alen);
  if (t.cat == Ty::Scalar || t.cat == Ty::Vec || t.cat == Ty::Arr) t.s = concrete_sk(t.s);
  return t;
}
bool ty_convertible(const Ty& from, const Ty& to) {
  if (from.cat != to.cat) return false;
  if (from.cat == Ty::Struct) return from.sid == to.sid;
  if (from.cat == Ty::Ptr) return from.eid == to.eid;
  if (from.cat == Ty::Arr && (from.ecat == Ty::Arr || to.ecat == Ty::Arr))
    return from.alen == to.alen && from.ecat == to.ecat && ty_convertible(elemT(from), elemT(to));
  if (from.cat == Ty::Arr)
    return from.alen == to.alen && from.ecat == to.ecat && from.n == to.n && from.r == to.r &&
           from.sid == to.sid && convertible(from.s, to.s);
  if (from.cat == Ty::Vec && from.n != to.n) return false;
  if (from.cat == Ty::Mat) return from.n == to.n && from.r == to.r;
  if (from.cat == Ty::Void) return true;
  return convertible(from.s, to.s);
}

// ===========================================================================
// diagnostics
// ===========================================================================
struct CompileError : std::runtime_error {
  int line, col;
  CompileError(int l, int c, const std::string& m) : std::runtime_error(m), line(l), col(c) {}
};
[[noreturn]] void fail(int line, int col, const std::string& msg) { throw CompileError(line, col, msg); }

// ===========================================================================
// lexer
// ===========================================================================
enum class TT { Ident, Int, Float, Punct, End };
struct Tok {
  TT t = TT::End;
  std::string s;
  int line = 1, col = 1;
  double fv = 0;
  long long iv = 0;
  char suffix = 0;
};

std::vector<Tok> lex(const std::string& src) {
  std::vector<Tok> out;
  size_t i = 0;
  int line = 1, col = 1;
  auto adv = [&](size_t k) {
    for (size_t j = 0; j < k && i < src.size(); ++j, ++i) {
      if (src[i] == '\n') { line++; col = 1; } else if ((unsigned char)src[i] < 0x80 || (unsigned char)src[i] >= 0xC0) { col++; }
    }
  };
  static const char* puncts[] = {"->", "&&", "||", "==", "!=", "<=", ">=", "<<", ">>", "+=", "-=",
                                 "*=", "/=", "%=", "&=", "|=", "^=", "++", "--", "(", ")", "{",
                                 "}", "[", "]", "<", ">", ",", ";", ":", ".", "=", "+", "-", "*",
                                 "/", "%", "!", "&", "|", "^", "~", "@", nullptr};
  while (i < src.size()) {
    char c = src[i];
    if (c == ' ' || c == '\t' || c == '\r' || c == '\n') { adv(1); continue; }
    if (c == '/' && i + 1 < src.size() && src[i + 1] == '/') {
      while (i < src.size() && src[i] != '\n') adv(1);
      continue;
    }
    if (c == '/' && i + 1 < src.size() && src[i + 1] == '*') {
      int sl = line, sc = col;
      int depth = 0;
      do {
        if (i + 1 < src.size() && src[i] == '/' && src[i + 1] == '*') { depth++; adv(2); }
        else if (i + 1 < src.size() && src[i] == '*' && src[i + 1] == '/') { depth--; adv(2); }
        else if (i < src.size()) adv(1);
        if (i >= src.size() && depth > 0) fail(sl, sc, "unterminated block comment");
      } while (depth > 0);
      continue;
    }
    Tok t;
    t.line = line;
    t.col = col;
    if (std::isalpha((unsigned char)c) || c == '_') {
      size_t j = i;
      while (j < src.size() && (std::isalnum((unsigned char)src[j]) || src[j] == '_')) ++j;
      t.t = TT::Ident;
      t.s = src.substr(i, j - i);
      adv(j - i);
      out.push_back(t);
      continue;
    }
    if (std::isdigit((unsigned char)c) || (c == '.' && i + 1 < src.size() && std::isdigit((unsigned char)src[i + 1]))) {
      size_t j = i;
      bool is_float = false;
      if (c == '0' && j + 1 < src.size() && (src[j + 1] == 'x' || src[j + 1] == 'X')) {
        j += 2;
        while (j < src.size() && (std::isxdigit((unsigned char)src[j]) || src[j] == '.')) {
          if (src[j] == '.') is_float = true;
          ++j;
        }
        if (j < src.size() && (src[j] == 'p' || src[j] == 'P')) {
          is_float = true;
          ++j;
          if (j < src.size() && (src[j] == '+' || src[j] == '-')) ++j;
          while (j < src.size() && std::isdigit((unsigned char)src[j])) ++j;
        }
      } else {
        while (j < src.size() && std::isdigit((unsigned char)src[j])) ++j;
        if (j < src.size() && src[j] == '.') {
          is_float = true;
          ++j;
          while (j < src.size() && std::isdigit((unsigned char)src[j])) ++j;
        }
        if (j < src.size() && (src[j] == 'e' || src[j] == 'E')) {
          size_t k = j + 1;
          if (k < src.size() && (src[k] == '+' || src[k] == '-')) ++k;
          if (k < src.size() && std::isdigit((unsigned char)src[k])) {
            is_float = true;
            j = k;
            while (j < src.size() && std::isdigit((unsigned char)src[j])) ++j;
          }
        }
      }
      std::string text = src.substr(i, j - i);
      char suffix = 0;
      if (j < src.size() && (src[j] == 'f' || src[j] == 'h' || src[j] == 'i' || src[j] == 'u')) {
        suffix = src[j];
        ++j;
      }
      if (suffix == 'h') fail(line, col, "f16 literals are not supported");
      if (suffix == 'f') is_float = true;
      if (is_float && (suffix == 'i' || suffix == 'u')) fail(line, col, "invalid numeric literal suffix");
      t.suffix = suffix;
      if (is_float) {
        t.t = TT::Float;
        t.fv = std::strtod(text.c_str(), nullptr);
      } else {
        t.t = TT::Int;
        errno = 0;
        t.iv = std::strtoll(text.c_str(), nullptr, 0);
        if (errno == ERANGE) fail(line, col, "integer literal out of range");
      }
      t.s = src.substr(i, j - i);
      adv(j - i);
      out.push_back(t);
      continue;
    }
    bool matched = false;
    for (int k = 0; puncts[k]; ++k) {
      size_t L = std::strlen(puncts[k]);
      if (src.compare(i, L, puncts[k]) == 0) {
        t.t = TT::Punct;
        t.s = puncts[k];
        adv(L);
        out.push_back(t);
        matched = true;
        break;
      }
    }
    if (!matched) {
      std::string ch(1, c);
      fail(line, col, "unexpected character '" + ch + "'");
    }
  }
  Tok e;
  e.t = TT::End;
  e.line = line;
  e.col = col;
  out.push_back(e);
  return out;
}

// ===========================================================================
// AST
// ===========================================================================
struct Expr;
using EP = std::unique_ptr<Expr>;
struct Expr {
  enum Kind { Lit, Name, Unary, Binary, Call, Member, Index } kind = Lit;
  int line = 0, col = 0;
  std::string op;  // operator / identifier / member / callee
  std::vector<EP> args;
  // literal
  int lit = 0;  // 1 int, 2 float, 3 bool
  double lf = 0;
  long long li = 0;
  char suffix = 0;
  bool bval = false;
  // explicit template type of a constructor call (vec3<f32>(...))
  bool has_targ = false;
  Ty targ;
  // checked
  Ty ty;
  bool cst = false;  // abstract constant (value in cv)
  double cv = 0;
  int fl = 0, tr = 0;
  bool lv = false, mut = false;
};

struct Stmt;
using SP = std::unique_ptr<Stmt>;
struct Stmt {
  enum Kind { Let, Var, Const, Assign, Compound, Incr, Decr, Phony, ExprS, If, For, While, Loop,
              Break, Continue, Return, Block, BreakIf, Switch, ConstAssert } kind = ExprS;
  int line = 0, col = 0;
  std::string name, op;
  bool has_ty = false;
  Ty ty;
  EP e, lhs;
  std::vector<SP> body, els, continuing;
  SP init, update;
  // switch: one clause per `case ...` / `default` with its selectors
  struct Clause {
    std::vector<EP> sel;
    bool def = false;
    std::vector<SP> body;
    int line = 0, col = 0;
  };
  std::vector<Clause> clauses;
};

struct Param {
  std::string name;
  Ty ty;
  int line, col;
};
struct Func {
  std::string name;
  int line = 0, col = 0;
  std::vector<Param> params;
  bool has_ret = false;
  Ty ret;
  std::vector<SP> body;
  int state = 0;  // 0 unchecked, 1 checking, 2 done
  int fl = 0, tr = 0;
  std::string code;
};
struct GConst {
  std::string name;
  int line = 0, col = 0;
  bool is_override = false;  // `override`: the default value, a concrete scalar
  bool is_assert = false;    // module-scope const_assert (no name, no value)
  bool is_private = false;   // var<private>: per-invocation state (a member of Private)
  bool has_ty = false;
  Ty ty;
  EP e;
  int state = 0;
};

// ===========================================================================
// parser
// ===========================================================================
class Parser {
 public:
  explicit Parser(std::vector<Tok> toks) : t_(std::move(toks)) {}

  void module(std::vector<std::unique_ptr<Func>>& fns, std::vector<std::unique_ptr<GConst>>& consts) {
    // struct names first: module-scope declarations may be used before
    // they appear
    for (size_t i = 0; i + 1 < t_.size(); ++i) {
      if (t_[i].t == TT::Ident && t_[i].s == "struct" && t_[i + 1].t == TT::Ident) {
        if (struct_id(t_[i + 1].s) >= 0) fail(t_[i + 1].line, t_[i + 1].col, "redefinition of struct '" + t_[i + 1].s + "'");
        StructDef d;
        d.name = t_[i + 1].s;
        d.line = t_[i + 1].line;
        d.col = t_[i + 1].col;
        g_structs->push_back(d);
      }
    }
    // type aliases too (alias Name = Type;), resolved where they are used
    for (size_t i = 0; i + 3 < t_.size(); ++i) {
      if (t_[i].t == TT::Ident && t_[i].s == "alias" && t_[i + 1].t == TT::Ident && t_[i + 2].t == TT::Punct &&
          t_[i + 2].s == "=") {
        const Tok& nt = t_[i + 1];
        Ty dummy;
        if (aliases_.count(nt.s) || struct_id(nt.s) >= 0 || alias_type(nt.s, dummy) || builtin_type_name(nt.s))
          fail(nt.line, nt.col, "redefinition of type '" + nt.s + "'");
        aliases_[nt.s] = i + 3;
      }
    }
    while (!at_end()) {
      skip_attributes();
      if (is_kw("struct")) {
        struct_decl();
      } else if (is_kw("fn")) {
        fns.push_back(function());
      } else if (is_kw("const") || is_kw("let") || is_kw("override")) {
        const bool ovr = is_kw("override");
        Tok k = next();
        auto g = std::make_unique<GConst>();
        g->line = k.line;
        g->col = k.col;
        g->is_override = ovr;
        g->name = ident("constant name");
        if (accept(":")) { g->has_ty = true; g->ty = type(); }
        if (ovr && !is_p("="))
          fail(k.line, k.col, "override '" + g->name + "' needs a default value: the engine sets no pipeline constants");
        expect("=");
        g->e = expr();
        expect(";");
        consts.push_back(std::move(g));
      } else if (is_kw("const_assert")) {
        Tok k = next();
        auto g = std::make_unique<GConst>();
        g->line = k.line;
        g->col = k.col;
        g->is_assert = true;
        g->e = expr();
        expect(";");
        consts.push_back(std::move(g));
      } else if (is_kw("diagnostic")) {
        // diagnostic(severity, rule); — the front end reports no
        // uniformity diagnostics, so the filter has nothing to change
        next();
        expect("(");
        Tok sv = cur();
        const std::string sev = ident("diagnostic severity");
        if (sev != "error" && sev != "warning" && sev != "info" && sev != "off")
          fail(sv.line, sv.col, "unknown diagnostic severity '" + sev + "'");
        expect(",");
        ident("diagnostic rule");
        while (accept(".")) ident("diagnostic rule");
        accept(",");
        expect(")");
        expect(";");
      } else if (is_kw("requires")) {
        // language extensions: the ones WGSL defines are all satisfied here
        // (or concern resources a field function cannot use)
        next();
        static const std::set<std::string> known = {"readonly_and_readwrite_storage_textures",
                                                    "packed_4x8_integer_dot_product",
                                                    "unrestricted_pointer_parameters", "pointer_composite_access"};
        for (;;) {
          Tok xt = cur();
          const std::string x = ident("language extension");
          if (!known.count(x)) fail(xt.line, xt.col, "unknown language extension '" + x + "'");
          if (!accept(",")) break;
          if (is_p(";")) break;
        }
        expect(";");
      } else if (is_kw("alias")) {
        next();
        ident("alias name");
        expect("=");
        type();  // checked here; uses re-read it from aliases_
        expect(";");
      } else if (is_kw("enable")) {
        fail(cur().line, cur().col,
             "'enable' extensions are not available: the reference's device requests no optional WGSL "
             "feature (f16 needs SHADER_F16)");
      } else if (is_kw("var") && peek().t == TT::Punct && peek().s == "<") {
        // var<private> name[: T][ = init];  state of one invocation (one ray)
        Tok k = next();
        expect("<");
        Tok sp = cur();
        const std::string space = ident("address space");
        if (space != "private")
          fail(sp.line, sp.col, "only var<private> is allowed at module scope in a field function module, found '" +
                                    space + "'");
        close_template();
        auto g = std::make_unique<GConst>();
        g->line = k.line;
        g->col = k.col;
        g->is_private = true;
        g->name = ident("variable name");
        if (accept(":")) { g->has_ty = true; g->ty = type(); }
        if (accept("=")) g->e = expr();
        else if (!g->has_ty) fail(k.line, k.col, "'var<private>' needs a type or an initializer");
        expect(";");
        consts.push_back(std::move(g));
      } else if (is_kw("var")) {
        fail(cur().line, cur().col, "'" + cur().s + "' declarations are not supported in field function modules");
      } else if (cur().t == TT::Punct && cur().s == ";") {
        next();
      } else {
        fail(cur().line, cur().col, "expected a function or constant declaration, found '" + cur().s + "'");
      }
    }
  }

 private:
  std::vector<Tok> t_;
  size_t p_ = 0;
  std::map<std::string, size_t> aliases_;  // alias name -> first token of its type
  std::set<std::string> resolving_;         // aliases being resolved (cycle check)

  static bool builtin_type_name(const std::string& n) {
    return n == "f32" || n == "i32" || n == "u32" || n == "bool" || n == "f16" || n == "f64" || type_generator(n);
  }

  const Tok& cur() const { return t_[p_]; }
  // Closes a template list: '>' or the first '>' of '>>' / '>=' / '>>='
  // (vec3<vec3<f32>> style nesting), as WGSL's template disambiguation does.
  void close_template() {
    Tok& t = t_[p_];
    if (t.t == TT::Punct && t.s == ">") { p_++; return; }
    if (t.t == TT::Punct && (t.s == ">>" || t.s == ">=" || t.s == ">>=")) {
      t.s = t.s.substr(1);
      t.col++;
      return;
    }
    fail(t.line, t.col, "expected '>', found '" + t.s + "'");
  }
  const Tok& peek(int k = 1) const { return t_[std::min(p_ + k, t_.size() - 1)]; }
  bool at_end() const { return cur().t == TT::End; }
  Tok next() { Tok t = t_[p_]; if (p_ + 1 < t_.size()) ++p_; return t; }
  bool is_p(const char* s) const { return cur().t == TT::Punct && cur().s == s; }
  bool is_kw(const char* s) const { return cur().t == TT::Ident && cur().s == s; }
  bool accept(const char* s) { if (is_p(s)) { next(); return true; } return false; }
  void expect(const char* s) {
    if (!is_p(s)) fail(cur().line, cur().col, std::string("expected '") + s + "', found '" + (at_end() ? std::string("end of input") : cur().s) + "'");
    next();
  }
  std::string ident(const char* what) {
    if (cur().t != TT::Ident) fail(cur().line, cur().col, std::string("expected ") + what + ", found '" + cur().s + "'");
    static const std::set<std::string> kw = {"fn", "let", "var", "const", "if", "else", "for", "while", "loop",
                                             "return", "break", "continue", "true", "false", "struct", "continuing"};
    if (kw.count(cur().s)) fail(cur().line, cur().col, "'" + cur().s + "' is a reserved keyword");
    if (cur().s.size() >= 2 && cur().s[0] == '_' && cur().s[1] == '_')
      fail(cur().line, cur().col, "identifiers starting with '__' are reserved");
    return next().s;
  }
  void skip_attributes() {
    while (is_p("@")) {
      next();
      ident("attribute name");
      if (accept("(")) {
        int depth = 1;
        while (depth > 0 && !at_end()) {
          if (is_p("(")) depth++;
          if (is_p(")")) depth--;
          next();
        }
      }
    }
  }

  // struct Name { member: type, ... }  (attributes on members are ignored)
  void struct_decl() {
    next();  // struct
    Tok nt = cur();
    const std::string name = ident("struct name");
    StructDef& d = (*g_structs)[size_t(struct_id(name))];
    expect("{");
    while (!is_p("}")) {
      if (at_end()) fail(cur().line, cur().col, "expected '}' before end of input");
      skip_attributes();
      Tok mt = cur();
      const std::string m = ident("member name");
      for (auto& x : d.members)
        if (x.first == m) fail(mt.line, mt.col, "duplicate member '" + m + "' in struct '" + name + "'");
      expect(":");
      Ty t = type();
      if (t.cat == Ty::Struct && t.sid == struct_id(name))
        fail(mt.line, mt.col, "struct '" + name + "' cannot contain itself");
      if (t.cat == Ty::Ptr) fail(mt.line, mt.col, "a struct member cannot be a pointer");
      d.members.push_back({m, t});
      if (!accept(",")) break;
    }
    expect("}");
    accept(";");
    if (d.members.empty()) fail(nt.line, nt.col, "struct '" + name + "' must have at least one member");
  }

  static bool type_generator(const std::string& s) {
    return s == "vec2" || s == "vec3" || s == "vec4" || (s.size() == 6 && s.compare(0, 3, "mat") == 0 && s[4] == 'x') || s == "array";
  }

  // Parses a type (after which the cursor is on the next token).
  Ty type() {
    Tok k = cur();
    std::string n = ident("type");
    if (n == "f32") return scalar(SK::F32);
    if (n == "i32") return scalar(SK::I32);
    if (n == "u32") return scalar(SK::U32);
    if (n == "bool") return scalar(SK::Bool);
    if (n == "f16" || n == "f64") fail(k.line, k.col, "type '" + n + "' is not supported");
    if (n == "ptr") {
      // ptr<function, T[, read_write]>: function-space pointers only
      expect("<");
      Tok sp = cur();
      const std::string space = ident("address space");
      if (space != "function")
        fail(sp.line, sp.col, "only ptr<function, T> is supported in field functions, found address space '" + space + "'");
      expect(",");
      Ty pt = type();
      if (pt.cat == Ty::Ptr) fail(k.line, k.col, "pointers to pointers are not allowed");
      if (accept(",")) {
        Tok am = cur();
        if (ident("access mode") != "read_write") fail(am.line, am.col, "function-space pointers are read_write");
      }
      close_template();
      return ptrT(pt);
    }
    Ty t;
    if (alias_type(n, t)) return t;
    auto ua = aliases_.find(n);
    if (ua != aliases_.end()) {
      if (resolving_.count(n)) fail(k.line, k.col, "cyclic type alias '" + n + "'");
      resolving_.insert(n);
      const size_t saved = p_;
      p_ = ua->second;
      t = type();
      p_ = saved;
      resolving_.erase(n);
      return t;
    }
    if (struct_id(n) >= 0) {
      t.cat = Ty::Struct;
      t.sid = struct_id(n);
      return t;
    }
    if (n == "vec2" || n == "vec3" || n == "vec4") {
      expect("<");
      Ty e = type();
      if (e.cat != Ty::Scalar) fail(k.line, k.col, "vector element must be a scalar type");
      close_template();
      return vecT(e.s, n[3] - '0');
    }
    if (n.size() == 6 && n.compare(0, 3, "mat") == 0 && n[4] == 'x') {
      int c = n[3] - '0', r = n[5] - '0';
      if (c < 2 || c > 4 || r < 2 || r > 4) fail(k.line, k.col, "unknown type '" + n + "'");
      expect("<");
      Ty e = type();
      if (!(e.cat == Ty::Scalar && e.s == SK::F32)) fail(k.line, k.col, "matrix element type must be f32");
      close_template();
      return matT(c, r);
    }
    if (n == "array") {
      // array<E, N>: E a scalar, vector or matrix type, N an integer literal
      expect("<");
      Ty e = type();
      if (e.cat == Ty::Void) fail(k.line, k.col, "invalid array element type");
      if (e.cat == Ty::Ptr) fail(k.line, k.col, "an array element cannot be a pointer");
      if (is_p(">") || is_p(">>") || is_p(">="))
        fail(cur().line, cur().col, "runtime-sized arrays are not allowed in a function; give the element count");
      expect(",");
      Tok nt = cur();
      if (nt.t != TT::Int) fail(nt.line, nt.col, "array element count must be an integer literal");
      next();
      if (nt.iv <= 0 || nt.iv > 65536) fail(nt.line, nt.col, "array element count must be between 1 and 65536");
      accept(",");
      close_template();
      return arrT(e, int(nt.iv));
    }
    fail(k.line, k.col, "unknown type '" + n + "'");
  }

 public:
  static bool alias_type(const std::string& n, Ty& t) {
    if (n.size() == 5 && n.compare(0, 3, "vec") == 0 && n[3] >= '2' && n[3] <= '4') {
      int k = n[3] - '0';
      switch (n[4]) {
        case 'f': t = vecT(SK::F32, k); return true;
        case 'i': t = vecT(SK::I32, k); return true;
        case 'u': t = vecT(SK::U32, k); return true;
        default: return false;
      }
    }
    if (n.size() == 7 && n.compare(0, 3, "mat") == 0 && n[4] == 'x' && n[6] == 'f') {
      int c = n[3] - '0', r = n[5] - '0';
      if (c >= 2 && c <= 4 && r >= 2 && r <= 4) { t = matT(c, r); return true; }
    }
    return false;
  }

 private:
  std::unique_ptr<Func> function() {
    Tok k = next();  // fn
    auto f = std::make_unique<Func>();
    f->line = k.line;
    f->col = k.col;
    f->name = ident("function name");
    expect("(");
    while (!is_p(")")) {
      skip_attributes();
      Param pr;
      pr.line = cur().line;
      pr.col = cur().col;
      pr.name = ident("parameter name");
      expect(":");
      pr.ty = type();
      f->params.push_back(pr);
      if (!accept(",")) break;
    }
    expect(")");
    if (accept("->")) {
      skip_attributes();
      f->has_ret = true;
      Tok rt = cur();
      f->ret = type();
      if (f->ret.cat == Ty::Ptr) fail(rt.line, rt.col, "a function cannot return a pointer");
    }
    f->body = block();
    return f;
  }

  std::vector<SP> block() {
    expect("{");
    std::vector<SP> out;
    while (!is_p("}")) {
      if (at_end()) fail(cur().line, cur().col, "expected '}' before end of input");
      SP s = statement();
      if (s) out.push_back(std::move(s));
    }
    expect("}");
    return out;
  }

  SP mk(Stmt::Kind k, const Tok& at) {
    SP s = std::make_unique<Stmt>();
    s->kind = k;
    s->line = at.line;
    s->col = at.col;
    return s;
  }

  SP statement() {
    skip_attributes();
    Tok at = cur();
    if (accept(";")) return nullptr;
    if (is_p("{")) {
      SP s = mk(Stmt::Block, at);
      s->body = block();
      return s;
    }
    if (is_kw("let") || is_kw("var") || is_kw("const")) {
      SP s = decl();
      expect(";");
      return s;
    }
    if (is_kw("const_assert")) {
      next();
      SP s = mk(Stmt::ConstAssert, at);
      s->e = expr();
      expect(";");
      return s;
    }
    if (is_kw("return")) {
      next();
      SP s = mk(Stmt::Return, at);
      if (!is_p(";")) s->e = expr();
      expect(";");
      return s;
    }
    if (is_kw("if")) return if_stmt();
    if (is_kw("for")) {
      next();
      SP s = mk(Stmt::For, at);
      expect("(");
      if (!is_p(";")) s->init = simple_or_decl();
      expect(";");
      if (!is_p(";")) s->e = expr();
      expect(";");
      if (!is_p(")")) s->update = simple_stmt();
      expect(")");
      s->body = block();
      return s;
    }
    if (is_kw("while")) {
      next();
      SP s = mk(Stmt::While, at);
      s->e = expr();
      s->body = block();
      return s;
    }
    if (is_kw("loop")) {
      next();
      SP s = mk(Stmt::Loop, at);
      expect("{");
      while (!is_p("}")) {
        if (at_end()) fail(cur().line, cur().col, "expected '}' before end of input");
        if (is_kw("continuing")) {
          next();
          expect("{");
          while (!is_p("}")) {
            if (at_end()) fail(cur().line, cur().col, "expected '}'");
            if (is_kw("break") && peek().t == TT::Ident && peek().s == "if") {
              Tok b = next();
              next();
              SP bi = mk(Stmt::BreakIf, b);
              bi->e = expr();
              expect(";");
              s->continuing.push_back(std::move(bi));
            } else {
              SP c = statement();
              if (c) s->continuing.push_back(std::move(c));
            }
          }
          expect("}");
          continue;
        }
        SP c = statement();
        if (c) s->body.push_back(std::move(c));
      }
      expect("}");
      return s;
    }
    if (is_kw("break")) { next(); expect(";"); return mk(Stmt::Break, at); }
    if (is_kw("continue")) { next(); expect(";"); return mk(Stmt::Continue, at); }
    if (is_kw("discard")) fail(at.line, at.col, "'discard' is only valid in fragment shaders");
    if (is_kw("switch")) return switch_stmt();
    SP s = simple_stmt();
    expect(";");
    return s;
  }

  // switch_statement: 'switch' expression '{' clause+ '}'; a clause is
  // 'case' selector (',' selector)* ','? ':'? compound, or 'default' ':'?
  // compound; a selector is an expression or 'default'.
  SP switch_stmt() {
    Tok at = next();  // switch
    SP s = mk(Stmt::Switch, at);
    s->e = expr();
    expect("{");
    while (!is_p("}")) {
      if (at_end()) fail(cur().line, cur().col, "expected '}' before end of input");
      Stmt::Clause cl;
      cl.line = cur().line;
      cl.col = cur().col;
      if (is_kw("default")) {
        next();
        cl.def = true;
      } else if (is_kw("case")) {
        next();
        for (;;) {
          if (is_kw("default")) {
            next();
            cl.def = true;
          } else {
            cl.sel.push_back(expr());
          }
          if (!accept(",")) break;
          if (is_p(":") || is_p("{")) break;
        }
      } else {
        fail(cur().line, cur().col, "expected 'case' or 'default' in switch");
      }
      accept(":");
      cl.body = block();
      s->clauses.push_back(std::move(cl));
    }
    expect("}");
    return s;
  }

  SP if_stmt() {
    Tok at = next();  // if
    SP s = mk(Stmt::If, at);
    s->e = expr();
    s->body = block();
    if (is_kw("else")) {
      next();
      if (is_kw("if")) {
        s->els.push_back(if_stmt());
      } else {
        s->els = block();
      }
    }
    return s;
  }

  SP decl() {
    Tok at = next();
    SP s = mk(at.s == "let" ? Stmt::Let : (at.s == "var" ? Stmt::Var : Stmt::Const), at);
    if (s->kind == Stmt::Var && is_p("<")) fail(at.line, at.col, "address-space qualified var is not allowed in a function");
    s->name = ident("variable name");
    if (accept(":")) { s->has_ty = true; s->ty = type(); }
    if (accept("=")) s->e = expr();
    else if (s->kind != Stmt::Var) fail(cur().line, cur().col, "'" + at.s + "' declaration needs an initializer");
    else if (!s->has_ty) fail(cur().line, cur().col, "'var' declaration needs a type or an initializer");
    return s;
  }

  SP simple_or_decl() {
    if (is_kw("let") || is_kw("var") || is_kw("const")) return decl();
    return simple_stmt();
  }

  // assignment, increment, phony assignment or call statement
  SP simple_stmt() {
    Tok at = cur();
    if (cur().t == TT::Ident && cur().s == "_" && peek().t == TT::Punct && peek().s == "=") {
      next();
      next();
      SP s = mk(Stmt::Phony, at);
      s->e = expr();
      return s;
    }
    EP lhs = unary();
    static const char* compound[] = {"+=", "-=", "*=", "/=", "%=", "&=", "|=", "^=", nullptr};
    if (is_p("=")) {
      next();
      SP s = mk(Stmt::Assign, at);
      s->lhs = std::move(lhs);
      s->e = expr();
      return s;
    }
    for (int k = 0; compound[k]; ++k) {
      if (is_p(compound[k])) {
        std::string op = next().s;
        SP s = mk(Stmt::Compound, at);
        s->op = op.substr(0, 1);
        s->lhs = std::move(lhs);
        s->e = expr();
        return s;
      }
    }
    if (is_p("++") || is_p("--")) {
      SP s = mk(next().s == "++" ? Stmt::Incr : Stmt::Decr, at);
      s->lhs = std::move(lhs);
      return s;
    }
    if (lhs->kind != Expr::Call) fail(at.line, at.col, "expression statement must be a function call or an assignment");
    SP s = mk(Stmt::ExprS, at);
    s->e = std::move(lhs);
    return s;
  }

  // ---- expressions (C-like precedence; WGSL forbids some mixes, which a
  //      conforming program therefore never contains) ----
  EP mkE(Expr::Kind k, const Tok& at) {
    EP e = std::make_unique<Expr>();
    e->kind = k;
    e->line = at.line;
    e->col = at.col;
    return e;
  }
  EP bin(const std::string& op, EP a, EP b, const Tok& at) {
    EP e = mkE(Expr::Binary, at);
    e->op = op;
    e->args.push_back(std::move(a));
    e->args.push_back(std::move(b));
    return e;
  }

 public:
  EP expr() { return logic_or(); }

 private:
  EP logic_or() {
    EP a = logic_and();
    while (is_p("||")) { Tok at = next(); a = bin("||", std::move(a), logic_and(), at); }
    return a;
  }
  EP logic_and() {
    EP a = bit_or();
    while (is_p("&&")) { Tok at = next(); a = bin("&&", std::move(a), bit_or(), at); }
    return a;
  }
  EP bit_or() {
    EP a = bit_xor();
    while (is_p("|")) { Tok at = next(); a = bin("|", std::move(a), bit_xor(), at); }
    return a;
  }
  EP bit_xor() {
    EP a = bit_and();
    while (is_p("^")) { Tok at = next(); a = bin("^", std::move(a), bit_and(), at); }
    return a;
  }
  EP bit_and() {
    EP a = equality();
    while (is_p("&")) { Tok at = next(); a = bin("&", std::move(a), equality(), at); }
    return a;
  }
  EP equality() {
    EP a = relational();
    while (is_p("==") || is_p("!=")) { Tok at = next(); a = bin(at.s, std::move(a), relational(), at); }
    return a;
  }
  EP relational() {
    EP a = shift();
    while (is_p("<") || is_p(">") || is_p("<=") || is_p(">=")) {
      Tok at = next();
      a = bin(at.s, std::move(a), shift(), at);
    }
    return a;
  }
  EP shift() {
    EP a = additive();
    while (is_p("<<") || is_p(">>")) { Tok at = next(); a = bin(at.s, std::move(a), additive(), at); }
    return a;
  }
  EP additive() {
    EP a = multiplicative();
    while (is_p("+") || is_p("-")) { Tok at = next(); a = bin(at.s, std::move(a), multiplicative(), at); }
    return a;
  }
  EP multiplicative() {
    EP a = unary();
    while (is_p("*") || is_p("/") || is_p("%")) { Tok at = next(); a = bin(at.s, std::move(a), unary(), at); }
    return a;
  }
  EP unary() {
    if (is_p("-") || is_p("!") || is_p("~")) {
      Tok at = next();
      EP e = mkE(Expr::Unary, at);
      e->op = at.s;
      e->args.push_back(unary());
      return e;
    }
    if (is_p("&") || is_p("*")) {  // address-of / indirection (function-space pointers)
      Tok at = next();
      EP e = mkE(Expr::Unary, at);
      e->op = at.s;
      e->args.push_back(unary());
      return e;
    }
    return postfix(primary());
  }
  EP postfix(EP e) {
    for (;;) {
      if (is_p(".")) {
        Tok at = next();
        EP m = mkE(Expr::Member, at);
        m->op = ident("member name");
        m->args.push_back(std::move(e));
        e = std::move(m);
      } else if (is_p("[")) {
        Tok at = next();
        EP ix = mkE(Expr::Index, at);
        ix->args.push_back(std::move(e));
        ix->args.push_back(expr());
        expect("]");
        e = std::move(ix);
      } else {
        return e;
      }
    }
  }
  EP primary() {
    Tok at = cur();
    if (at.t == TT::Int || at.t == TT::Float) {
      next();
      EP e = mkE(Expr::Lit, at);
      if (at.t == TT::Float) { e->lit = 2; e->lf = at.fv; }
      else { e->lit = 1; e->li = at.iv; }
      e->suffix = at.suffix;
      return e;
    }
    if (accept("(")) {
      EP e = expr();
      expect(")");
      return e;
    }
    if (at.t == TT::Ident) {
      if (at.s == "true" || at.s == "false") {
        next();
        EP e = mkE(Expr::Lit, at);
        e->lit = 3;
        e->bval = at.s == "true";
        return e;
      }
      std::string name = ident("expression");
      EP e;
      if (name == "bitcast" && is_p("<")) {
        // bitcast<T>(e): reinterpret the bits of e as T
        next();
        Ty t = type();
        close_template();
        e = mkE(Expr::Call, at);
        e->op = name;
        e->has_targ = true;
        e->targ = t;
        if (!is_p("(")) fail(cur().line, cur().col, "expected '(' after bitcast<T>");
      } else if (type_generator(name) && is_p("<")) {
        // templated constructor vec3<f32>(...) / mat3x3<f32>(...)
        p_--;  // re-read the generator as a type
        Ty t = type();
        e = mkE(Expr::Call, at);
        e->op = name;
        e->has_targ = true;
        e->targ = t;
        if (!is_p("(")) fail(cur().line, cur().col, "expected '(' after type in constructor");
      } else if (aliases_.count(name) && is_p("(")) {
        // a type alias used as a constructor: the aliased type's constructor
        p_--;
        Ty t = type();
        e = mkE(Expr::Call, at);
        if (t.cat == Ty::Struct) {
          e->op = (*g_structs)[size_t(t.sid)].name;
        } else if (t.cat == Ty::Scalar) {
          e->op = wgsl_name(t);
        } else {
          e->op = t.cat == Ty::Vec   ? "vec" + std::to_string(t.n)
                  : t.cat == Ty::Mat ? "mat" + std::to_string(t.n) + "x" + std::to_string(t.r)
                                     : std::string("array");
          e->has_targ = true;
          e->targ = t;
        }
      } else if (is_p("(")) {
        e = mkE(Expr::Call, at);
        e->op = name;
      } else {
        e = mkE(Expr::Name, at);
        e->op = name;
        return e;
      }
      expect("(");
      while (!is_p(")")) {
        e->args.push_back(expr());
        if (!accept(",")) break;
      }
      expect(")");
      return e;
    }
    fail(at.line, at.col, "expected an expression, found '" + (at.t == TT::End ? std::string("end of input") : at.s) + "'");
  }
};

// ===========================================================================
// checker + emitter
// ===========================================================================
std::string f32_literal(double v) {
  float f = float(v);
  if (std::isnan(f)) return "::wgsl::f32_from_bits(0x7fc00000u)";
  if (std::isinf(f)) return f > 0 ? "::wgsl::f32_from_bits(0x7f800000u)" : "::wgsl::f32_from_bits(0xff800000u)";
  char buf[64];
  std::snprintf(buf, sizeof buf, "%a", double(f));
  std::string s = std::string(buf) + "f";
  if (s[0] == '-') s = "(" + s + ")";
  return s;
}

struct Sym {
  Ty ty;
  bool is_var = false;
  std::string cpp;
  bool cst = false;  // abstract constant value known (const decls)
  double cv = 0;
};

class Compiler {
 public:
  std::vector<std::unique_ptr<Func>> fns;
  std::vector<std::unique_ptr<GConst>> consts;
  std::map<std::string, Func*> fmap;
  std::map<std::string, GConst*> cmap;
  std::map<std::string, Sym> gsyms;  // checked module constants
  std::vector<std::map<std::string, Sym>> scopes;
  Func* cur_fn = nullptr;
  std::vector<std::string> const_code;
  std::vector<std::string> private_code;  // members of struct Private (var<private>)
  bool in_module_init = false;  // checking a module constant or a private initializer
  int loop_depth = 0;

  static bool is_helper(const std::string& n) {
    return n == "rotateX" || n == "rotateY" || n == "rotateZ" || n == "translate" ||
           n == "refraction_index" || n == "refraction" || n == "point_plane_distance" ||
           n == "sigmoid";
  }

  void declare_module(int line_offset_unused) {
    (void)line_offset_unused;
    for (auto& f : fns) {
      if (fmap.count(f->name) || cmap.count(f->name) || is_helper(f->name) || f->name == "PI")
        fail(f->line, f->col, "redefinition of '" + f->name + "'");
      fmap[f->name] = f.get();
    }
    for (auto& c : consts) {
      if (c->is_assert) continue;
      if (fmap.count(c->name) || cmap.count(c->name) || is_helper(c->name) || c->name == "PI")
        fail(c->line, c->col, "redefinition of '" + c->name + "'");
      cmap[c->name] = c.get();
    }
  }

  // ---- literal / conversion emission ----
  std::string lit_as(double v, const Ty& t, int line, int col) {
    if (t.cat == Ty::Scalar) {
      switch (t.s) {
        case SK::F32: case SK::AFloat: return f32_literal(v);
        case SK::I32: case SK::AInt: {
          if (v < -2147483648.0 || v > 2147483647.0) fail(line, col, "value does not fit in i32");
          long long iv = (long long)v;
          if (iv == -2147483648LL) return "(-2147483647-1)";
          return iv < 0 ? "(" + std::to_string(iv) + ")" : std::to_string(iv);
        }
        case SK::U32: {
          if (v < 0 || v > 4294967295.0) fail(line, col, "value does not fit in u32");
          return std::to_string((unsigned long long)v) + "u";
        }
        case SK::Bool: return v != 0 ? "true" : "false";
      }
    }
    if (t.cat == Ty::Vec) {  // splat of an abstract scalar (only from conversions we emit)
      return cpp_name(t) + "(" + lit_as(v, scalar(t.s), line, col) + ")";
    }
    fail(line, col, "cannot convert constant to " + wgsl_name(t));
  }

  std::string ex_as(Expr& e, const Ty& t) {
    if (e.cst) return lit_as(e.cv, t, e.line, e.col);
    if (e.ty == t) return ex(e);
    if (ty_convertible(e.ty, t)) return ex(e);  // same C++ representation
    fail(e.line, e.col, "cannot convert " + wgsl_name(e.ty) + " to " + wgsl_name(t));
  }

  // ---- scopes ----
  Sym* lookup(const std::string& n) {
    for (int i = int(scopes.size()) - 1; i >= 0; --i) {
      auto it = scopes[i].find(n);
      if (it != scopes[i].end()) return &it->second;
    }
    auto g = gsyms.find(n);
    if (g != gsyms.end()) return &g->second;
    return nullptr;
  }
  void declare(const std::string& n, const Sym& s, int line, int col) {
    if (scopes.back().count(n)) fail(line, col, "redefinition of '" + n + "' in the same scope");
    scopes.back()[n] = s;
  }

  // The value of a constant boolean expression: bool literals, '!', '&&',
  // '||', '==' / '!=' of booleans, and comparisons of folded numbers.
  bool const_bool(Expr& e, bool& val) {
    if (e.kind == Expr::Lit && e.lit == 3) {
      val = e.bval;
      return true;
    }
    if (e.kind == Expr::Unary && e.op == "!") {
      bool v;
      if (!const_bool(*e.args[0], v)) return false;
      val = !v;
      return true;
    }
    if (e.kind != Expr::Binary) return false;
    const std::string& op = e.op;
    Expr& L = *e.args[0];
    Expr& R = *e.args[1];
    if (L.ty.cat == Ty::Scalar && L.ty.s == SK::Bool) {
      bool a, b;
      if (!const_bool(L, a) || !const_bool(R, b)) return false;
      if (op == "&&" || op == "&") val = a && b;
      else if (op == "||" || op == "|") val = a || b;
      else if (op == "==") val = a == b;
      else if (op == "!=") val = a != b;
      else return false;
      return true;
    }
    if (!(L.cst && R.cst && L.ty.cat == Ty::Scalar && R.ty.cat == Ty::Scalar)) return false;
    const double a = L.cv, b = R.cv;
    if (op == "<") val = a < b;
    else if (op == "<=") val = a <= b;
    else if (op == ">") val = a > b;
    else if (op == ">=") val = a >= b;
    else if (op == "==") val = a == b;
    else if (op == "!=") val = a != b;
    else return false;
    return true;
  }

  void check_const_assert(Expr& e, int line, int col) {
    check(e);
    if (!(e.ty.cat == Ty::Scalar && e.ty.s == SK::Bool))
      fail(line, col, "const_assert needs a bool expression, found " + wgsl_name(e.ty));
    bool v = false;
    if (!const_bool(e, v))
      fail(line, col, "const_assert needs a constant expression (literals, abstract constants, comparisons, ! && ||)");
    if (!v) fail(line, col, "const_assert failed");
  }

  void check_gconst(GConst& g) {
    if (g.state == 2) return;
    if (g.state == 1) fail(g.line, g.col, "cyclic constant definition '" + g.name + "'");
    g.state = 1;
    if (g.is_private) {
      auto saved = scopes;
      scopes.clear();
      scopes.emplace_back();
      Ty t;
      std::string init;
      if (g.e) {
        const bool saved_init = in_module_init;
        in_module_init = true;
        check(*g.e);
        in_module_init = saved_init;
        if (g.e->ty.cat == Ty::Void) fail(g.line, g.col, "initializer has no value");
        t = g.has_ty ? g.ty : concretize(g.e->ty);
        if (g.has_ty && !(g.e->ty == t || ty_convertible(g.e->ty, t)))
          fail(g.line, g.col, "cannot initialize '" + g.name + "' of type " + wgsl_name(t) + " with " + wgsl_name(g.e->ty));
        init = ex_as(*g.e, t);
      } else {
        t = g.ty;
        init = cpp_name(t) + "()";
      }
      if (t.cat == Ty::Ptr) fail(g.line, g.col, "a private variable cannot be a pointer");
      scopes = saved;
      private_code.push_back("  " + cpp_name(t) + " u_" + g.name + " = " + init + ";");
      Sym sym;
      sym.ty = t;
      sym.is_var = true;
      sym.cpp = "pv.u_" + g.name;
      gsyms[g.name] = sym;
      g.state = 2;
      return;
    }
    if (g.is_assert) {
      auto saved = scopes;
      scopes.clear();
      scopes.emplace_back();
      check_const_assert(*g.e, g.line, g.col);
      scopes = saved;
      g.state = 2;
      return;
    }
    auto saved = scopes;
    scopes.clear();
    scopes.emplace_back();
    const bool saved_init = in_module_init;
    in_module_init = true;
    check(*g.e);
    in_module_init = saved_init;
    if (g.is_override) {
      // an override is a concrete scalar: its declared type, or its default
      // value's type made concrete
      if (!g.has_ty) {
        g.has_ty = true;
        g.ty = concretize(g.e->ty);
      }
      if (g.ty.cat != Ty::Scalar)
        fail(g.line, g.col, "override '" + g.name + "' must have a scalar type, found " + wgsl_name(g.ty));
    }
    if (g.has_ty && !(ty_convertible(g.e->ty, g.ty) || g.e->ty == g.ty))
      fail(g.line, g.col, "cannot initialize '" + g.name + "' of type " + wgsl_name(g.ty) + " with " + wgsl_name(g.e->ty));
    Sym s;
    if (!g.has_ty && g.e->cst && g.e->ty.cat == Ty::Scalar) {
      // an abstract constant keeps its full-precision value
      s.ty = g.e->ty;
      s.cst = true;
      s.cv = g.e->cv;
    } else {
      // module constants become functions: no device-global initialisers
      Ty ct = g.has_ty ? g.ty : concretize(g.e->ty);
      s.ty = ct;
      s.cpp = "u_" + g.name + "()";
      const_code.push_back("WG_HD " + cpp_name(ct) + " u_" + g.name + "() { return " + ex_as(*g.e, ct) + "; }");
    }
    scopes = saved;
    gsyms[g.name] = s;
    g.state = 2;
  }

  std::map<std::string, int> name_uses;  // per function: unique C++ names
  std::string fresh(const std::string& n) {
    int k = name_uses[n]++;
    return k == 0 ? "u_" + n : "u_" + n + "_" + std::to_string(k);
  }

  // ---- expressions ----
  void check(Expr& e) {
    switch (e.kind) {
      case Expr::Lit: return check_lit(e);
      case Expr::Name: return check_name(e);
      case Expr::Unary: return check_unary(e);
      case Expr::Binary: return check_binary(e);
      case Expr::Call: return check_call(e);
      case Expr::Member: return check_member(e);
      case Expr::Index: return check_index(e);
    }
  }

  void check_lit(Expr& e) {
    if (e.lit == 3) { e.ty = scalar(SK::Bool); return; }
    if (e.lit == 2) {
      if (e.suffix == 'f') { e.ty = scalar(SK::F32); return; }
      e.ty = scalar(SK::AFloat);
      e.cst = true;
      e.cv = e.lf;
      return;
    }
    if (e.suffix == 'i') {
      if (e.li > 2147483647LL) fail(e.line, e.col, "value does not fit in i32");
      e.ty = scalar(SK::I32);
      return;
    }
    if (e.suffix == 'u') {
      if (e.li > 4294967295LL) fail(e.line, e.col, "value does not fit in u32");
      e.ty = scalar(SK::U32);
      return;
    }
    e.ty = scalar(SK::AInt);
    e.cst = true;
    e.cv = double(e.li);
  }

  void check_name(Expr& e) {
    if (e.op == "PI" && !lookup("PI")) {
      // const PI: f32 = 3.141592653589793; (main_view.wgsl:76)
      e.ty = scalar(SK::F32);
      return;
    }
    Sym* s = lookup(e.op);
    if (!s) {
      auto c = cmap.find(e.op);
      if (c != cmap.end()) {
        check_gconst(*c->second);
        s = lookup(e.op);
      }
    }
    if (!s) {
      if (fmap.count(e.op) || is_helper(e.op)) fail(e.line, e.col, "function '" + e.op + "' used as a value");
      fail(e.line, e.col, "no definition in scope for identifier: '" + e.op + "'");
    }
    if (in_module_init && s->cpp.compare(0, 3, "pv.") == 0)
      fail(e.line, e.col, "'" + e.op + "' is a private variable: module initializers must be constant");
    e.ty = s->ty;
    e.cst = s->cst;
    e.cv = s->cv;
    e.lv = true;
    e.mut = s->is_var;
  }

  void check_unary(Expr& e) {
    Expr& a = *e.args[0];
    check(a);
    e.fl = a.fl;
    e.tr = a.tr;
    if (e.op == "&") {
      // the address of a variable (or of a part of one other than a vector
      // component): a ptr<function, T>
      if (!(a.lv && a.mut)) fail(e.line, e.col, "'&' needs a variable (a 'var' or a part of one)");
      if ((a.kind == Expr::Member || a.kind == Expr::Index) && a.args[0]->ty.cat == Ty::Vec)
        fail(e.line, e.col, "cannot take the address of a vector component");
      if (a.ty.cat == Ty::Ptr) fail(e.line, e.col, "pointers to pointers are not allowed");
      e.ty = ptrT(a.ty);
      return;
    }
    if (e.op == "*") {
      if (a.ty.cat != Ty::Ptr) fail(e.line, e.col, "'*' needs a pointer, found " + wgsl_name(a.ty));
      e.ty = pointeeT(a.ty);
      e.lv = true;
      e.mut = true;  // function-space pointers are read_write
      return;
    }
    if (a.ty.cat == Ty::Ptr) fail(e.line, e.col, "operator '" + e.op + "' cannot be applied to a pointer");
    if (a.ty.cat == Ty::Arr) fail(e.line, e.col, "operator '" + e.op + "' cannot be applied to an array");
    if (a.ty.cat == Ty::Struct) fail(e.line, e.col, "operator '" + e.op + "' cannot be applied to a struct");
    if (e.op == "-") {
      if (!((a.ty.cat == Ty::Scalar || a.ty.cat == Ty::Vec) && is_numeric(a.ty.s)) && a.ty.cat != Ty::Mat)
        fail(e.line, e.col, "unary '-' needs a numeric operand, found " + wgsl_name(a.ty));
      if (a.ty.s == SK::U32 && a.ty.cat != Ty::Mat) fail(e.line, e.col, "unary '-' is not defined for u32");
      e.ty = a.ty;
      if (a.cst) { e.cst = true; e.cv = -a.cv; }
    } else if (e.op == "!") {
      if (!(a.ty.s == SK::Bool && (a.ty.cat == Ty::Scalar || a.ty.cat == Ty::Vec)))
        fail(e.line, e.col, "'!' needs a bool operand, found " + wgsl_name(a.ty));
      e.ty = a.ty;
    } else {  // ~
      if (!((a.ty.cat == Ty::Scalar || a.ty.cat == Ty::Vec) && is_int(a.ty.s)))
        fail(e.line, e.col, "'~' needs an integer operand, found " + wgsl_name(a.ty));
      e.ty = a.ty;
      if (a.cst) { e.cst = true; e.cv = double(~(long long)a.cv); }
    }
  }

  static int vcount(const Ty& t) { return t.cat == Ty::Vec ? t.n : (t.cat == Ty::Mat ? t.n * t.r : 1); }
  static bool is_f32(const Ty& t) { return t.s == SK::F32 || t.cat == Ty::Mat; }

  // operand target types for emission
  struct BinInfo { Ty tl, tr; };
  std::map<Expr*, BinInfo> bininfo;

  void check_binary(Expr& e) {
    Expr& L = *e.args[0];
    Expr& R = *e.args[1];
    check(L);
    check(R);
    e.fl = L.fl + R.fl;
    e.tr = L.tr + R.tr;
    if (L.ty.cat == Ty::Arr || R.ty.cat == Ty::Arr)
      fail(e.line, e.col, "operator '" + e.op + "' cannot be applied to arrays");
    if (L.ty.cat == Ty::Struct || R.ty.cat == Ty::Struct)
      fail(e.line, e.col, "operator '" + e.op + "' cannot be applied to structs");
    const std::string& op = e.op;
    auto mismatch = [&]() -> void {
      fail(e.line, e.col, "no matching operator '" + op + "' for " + wgsl_name(L.ty) + " and " + wgsl_name(R.ty));
    };
    BinInfo bi;
    if (op == "&&" || op == "||") {
      if (!(L.ty.cat == Ty::Scalar && L.ty.s == SK::Bool && R.ty.cat == Ty::Scalar && R.ty.s == SK::Bool)) mismatch();
      e.ty = scalar(SK::Bool);
      bi.tl = bi.tr = e.ty;
      bininfo[&e] = bi;
      return;
    }
    bool arith = op == "+" || op == "-" || op == "*" || op == "/" || op == "%";
    bool cmp = op == "<" || op == ">" || op == "<=" || op == ">=" || op == "==" || op == "!=";
    bool bits = op == "&" || op == "|" || op == "^";
    bool shift = op == "<<" || op == ">>";
    const Ty& a = L.ty;
    const Ty& b = R.ty;
    if (a.cat == Ty::Void || b.cat == Ty::Void) mismatch();
    if (arith && (a.cat == Ty::Mat || b.cat == Ty::Mat)) {
      // matrix arithmetic
      if (op == "*" && a.cat == Ty::Mat && b.cat == Ty::Vec) {
        if (b.n != a.n || !is_float(b.s)) mismatch();
        e.ty = vecT(SK::F32, a.r);
        bi.tl = a; bi.tr = vecT(SK::F32, b.n);
        e.fl += a.n * a.r + (a.n - 1) * a.r;
      } else if (op == "*" && a.cat == Ty::Vec && b.cat == Ty::Mat) {
        if (a.n != b.r || !is_float(a.s)) mismatch();
        e.ty = vecT(SK::F32, b.n);
        bi.tl = vecT(SK::F32, a.n); bi.tr = b;
        e.fl += b.n * (b.r + b.r - 1);
      } else if (op == "*" && a.cat == Ty::Mat && b.cat == Ty::Mat) {
        if (b.r != a.n) mismatch();
        e.ty = matT(b.n, a.r);
        bi.tl = a; bi.tr = b;
        e.fl += b.n * (a.n * a.r + (a.n - 1) * a.r);
      } else if (op == "*" && (a.cat == Ty::Scalar || b.cat == Ty::Scalar)) {
        const Ty& s = a.cat == Ty::Scalar ? a : b;
        const Ty& m = a.cat == Ty::Mat ? a : b;
        if (!is_float(s.s)) mismatch();
        e.ty = m;
        bi.tl = a.cat == Ty::Mat ? a : scalar(SK::F32);
        bi.tr = b.cat == Ty::Mat ? b : scalar(SK::F32);
        e.fl += m.n * m.r;
      } else if ((op == "+" || op == "-") && a.cat == Ty::Mat && b.cat == Ty::Mat) {
        if (a.n != b.n || a.r != b.r) mismatch();
        e.ty = a;
        bi.tl = a; bi.tr = b;
        e.fl += a.n * a.r;
      } else {
        mismatch();
      }
      bininfo[&e] = bi;
      return;
    }
    if (a.cat == Ty::Mat || b.cat == Ty::Mat) mismatch();
    if (shift) {
      // e1 << e2, e1 >> e2: e1 an i32 / u32 scalar or vector, e2 u32 of the
      // same shape; the low 5 bits of e2 are the amount (wgsl_rt.cuh shl)
      if (!(is_int(a.s) && (b.s == SK::U32 || b.s == SK::AInt)) || a.cat != b.cat ||
          (a.cat == Ty::Vec && a.n != b.n))
        mismatch();
      const bool folded = a.s == SK::AInt && L.cst && R.cst && a.cat == Ty::Scalar;
      e.ty = a.cat == Ty::Vec ? vecT(concrete_sk(a.s), a.n) : scalar(folded ? SK::AInt : concrete_sk(a.s));
      bi.tl = e.ty;
      bi.tr = a.cat == Ty::Vec ? vecT(SK::U32, a.n) : scalar(SK::U32);
      if (folded) {
        e.cst = true;
        long long x = (long long)L.cv, y = (long long)R.cv;
        if (y < 0 || y >= 32) fail(e.line, e.col, "shift amount out of range in a constant expression");
        e.cv = double(op == "<<" ? (x << y) : (x >> y));
      }
      bininfo[&e] = bi;
      return;
    }
    SK u;
    if (!unify_sk(a.s, b.s, u)) mismatch();
    int n = 1;
    Ty::Cat cat = Ty::Scalar;
    if (a.cat == Ty::Vec && b.cat == Ty::Vec) {
      if (a.n != b.n) mismatch();
      n = a.n;
      cat = Ty::Vec;
    } else if (a.cat == Ty::Vec || b.cat == Ty::Vec) {
      n = a.cat == Ty::Vec ? a.n : b.n;
      cat = Ty::Vec;
      if (cmp || bits || shift) mismatch();  // WGSL has no mixed scalar/vector comparison
    }
    auto typed = [&](const Ty& orig) { Ty t = orig; t.s = u; return t; };
    bi.tl = typed(a);
    bi.tr = typed(b);
    if (arith) {
      if (u == SK::Bool) mismatch();
      e.ty = cat == Ty::Vec ? vecT(u, n) : scalar(u);
      if (u == SK::F32) e.fl += n;
      if (L.cst && R.cst && cat == Ty::Scalar) {
        e.cst = true;
        double x = L.cv, y = R.cv;
        bool integer = u == SK::AInt;
        if (op == "+") e.cv = x + y;
        else if (op == "-") e.cv = x - y;
        else if (op == "*") e.cv = x * y;
        else if (op == "/") {
          if (integer) {
            if (y == 0) fail(e.line, e.col, "integer division by zero in a constant expression");
            e.cv = double((long long)x / (long long)y);
          } else {
            e.cv = x / y;
          }
        } else {
          if (integer) {
            if (y == 0) fail(e.line, e.col, "integer remainder by zero in a constant expression");
            e.cv = double((long long)x % (long long)y);
          } else {
            e.cv = std::fmod(x, y);
          }
        }
      }
    } else if (cmp) {
      if (u == SK::Bool && !(op == "==" || op == "!=")) mismatch();
      e.ty = cat == Ty::Vec ? vecT(SK::Bool, n) : scalar(SK::Bool);
      if (L.cst && R.cst && cat == Ty::Scalar) {
        // fold only to keep abstract operands out of C++; result stays a bool expression
      }
    } else if (bits) {
      // & | ^ on integers; & | also on bools (WGSL has no bool ^)
      if (!(is_int(u) || (u == SK::Bool && op != "^"))) mismatch();
      e.ty = cat == Ty::Vec ? vecT(u, n) : scalar(u);
      if (L.cst && R.cst && cat == Ty::Scalar && u == SK::AInt) {
        e.cst = true;
        long long x = (long long)L.cv, y = (long long)R.cv;
        e.cv = double(op == "&" ? (x & y) : op == "|" ? (x | y) : (x ^ y));
      }
    } else {
      mismatch();
    }
    bininfo[&e] = bi;
  }

  static int swz_index(char c) {
    switch (c) {
      case 'x': case 'r': return 0;
      case 'y': case 'g': return 1;
      case 'z': case 'b': return 2;
      case 'w': case 'a': return 3;
    }
    return -1;
  }

  // p.m and p[i] on a pointer p access its pointee (WGSL's pointer
  // composite access); the pointer is a C++ reference, so nothing changes in
  // the emitted code
  static void deref_in_place(Expr& a) {
    if (a.ty.cat != Ty::Ptr) return;
    a.ty = pointeeT(a.ty);
    a.lv = true;
    a.mut = true;
  }

  void check_member(Expr& e) {
    Expr& a = *e.args[0];
    check(a);
    deref_in_place(a);
    e.fl = a.fl;
    e.tr = a.tr;
    if (a.ty.cat == Ty::Struct) {
      for (auto& m : (*g_structs)[size_t(a.ty.sid)].members) {
        if (m.first == e.op) {
          e.ty = m.second;
          e.lv = a.lv;
          e.mut = a.mut;
          return;
        }
      }
      fail(e.line, e.col, "struct " + wgsl_name(a.ty) + " has no member '" + e.op + "'");
    }
    if (a.ty.cat != Ty::Vec) fail(e.line, e.col, "type " + wgsl_name(a.ty) + " has no member '" + e.op + "'");
    const std::string& m = e.op;
    if (m.empty() || m.size() > 4) fail(e.line, e.col, "invalid swizzle '" + m + "'");
    bool rgba = std::strchr("rgba", m[0]) != nullptr;
    for (char c : m) {
      int k = swz_index(c);
      bool c_rgba = std::strchr("rgba", c) != nullptr;
      if (k < 0 || c_rgba != rgba) fail(e.line, e.col, "invalid swizzle '" + m + "'");
      if (k >= a.ty.n) fail(e.line, e.col, "swizzle '" + m + "' out of range for " + wgsl_name(a.ty));
    }
    if (m.size() == 1) {
      e.ty = scalar(a.ty.s);
      e.lv = a.lv;
      e.mut = a.mut;
    } else {
      e.ty = vecT(a.ty.s, int(m.size()));
    }
  }

  void check_index(Expr& e) {
    Expr& a = *e.args[0];
    Expr& i = *e.args[1];
    check(a);
    deref_in_place(a);
    check(i);
    e.fl = a.fl + i.fl;
    e.tr = a.tr + i.tr;
    if (!(i.ty.cat == Ty::Scalar && is_int(i.ty.s))) fail(i.line, i.col, "index must be an integer, found " + wgsl_name(i.ty));
    if (a.ty.cat == Ty::Vec) {
      if (i.cst && (i.cv < 0 || i.cv >= a.ty.n)) fail(i.line, i.col, "index out of bounds");
      e.ty = scalar(a.ty.s);
    } else if (a.ty.cat == Ty::Mat) {
      if (i.cst && (i.cv < 0 || i.cv >= a.ty.n)) fail(i.line, i.col, "index out of bounds");
      e.ty = vecT(SK::F32, a.ty.r);
    } else if (a.ty.cat == Ty::Arr) {
      // a constant index is checked here; a runtime index is clamped to the
      // array (wgpu's default bounds-check policy)
      if (i.cst && (i.cv < 0 || i.cv >= a.ty.alen)) fail(i.line, i.col, "index out of bounds");
      e.ty = elemT(a.ty);
    } else {
      fail(e.line, e.col, "cannot index a value of type " + wgsl_name(a.ty));
    }
    e.lv = a.lv;
    e.mut = a.mut;
  }

  // ---- calls ----
  struct CallInfo {
    std::vector<Ty> targets;
    std::string fn;  // C++ callee
    int kind = 0;    // 0 plain call, 1 vector ctor, 2 matrix ctor (columns), 3 matrix ctor (scalars), 4 scalar conv, 5 zero value
  };
  std::map<Expr*, CallInfo> callinfo;

  void check_args(Expr& e) {
    for (auto& a : e.args) {
      check(*a);
      e.fl += a->fl;
      e.tr += a->tr;
      if (a->ty.cat == Ty::Void) fail(a->line, a->col, "function returning nothing used as a value");
    }
  }

  bool ctor_type(Expr& e, Ty& out, bool& inferred) {
    inferred = false;
    if (e.has_targ) { out = e.targ; return true; }
    const std::string& n = e.op;
    if (n == "f32") { out = scalar(SK::F32); return true; }
    if (n == "i32") { out = scalar(SK::I32); return true; }
    if (n == "u32") { out = scalar(SK::U32); return true; }
    if (n == "bool") { out = scalar(SK::Bool); return true; }
    if (Parser::alias_type(n, out)) return true;
    if (n == "vec2" || n == "vec3" || n == "vec4") { out = vecT(SK::AFloat, n[3] - '0'); inferred = true; return true; }
    if (n == "array") { out = Ty(); out.cat = Ty::Arr; inferred = true; return true; }
    if (n.size() == 6 && n.compare(0, 3, "mat") == 0 && n[4] == 'x') {
      int c = n[3] - '0', r = n[5] - '0';
      if (c >= 2 && c <= 4 && r >= 2 && r <= 4) { out = matT(c, r); return true; }
    }
    return false;
  }

  // bitcast<T>(e): T and e's type are i32 / u32 / f32 scalars, or vectors
  // of them with the same component count.
  void check_bitcast(Expr& e) {
    if (!e.has_targ) fail(e.line, e.col, "bitcast needs a target type: bitcast<T>(e)");
    need_args(e, 1);
    const Ty t = e.targ;
    const Ty a = concretize(e.args[0]->ty);
    auto ok = [](const Ty& x) {
      return (x.cat == Ty::Scalar || x.cat == Ty::Vec) && (x.s == SK::I32 || x.s == SK::U32 || x.s == SK::F32);
    };
    if (!ok(t)) fail(e.line, e.col, "bitcast target must be i32, u32, f32 or a vector of them, found " + wgsl_name(t));
    if (!ok(a)) fail(e.line, e.col, "bitcast argument must be i32, u32, f32 or a vector of them, found " + wgsl_name(a));
    if (t.cat != a.cat || (t.cat == Ty::Vec && t.n != a.n))
      fail(e.line, e.col, "bitcast between types of different sizes: " + wgsl_name(a) + " to " + wgsl_name(t));
    CallInfo ci;
    ci.fn = "::wgsl::bitcast_<" + cpp_name(t) + ">";
    ci.targets.push_back(a);
    e.ty = t;
    callinfo[&e] = ci;
  }

  // Name(m1, ..., mN): every member in declaration order; Name(): zero value.
  void check_struct_ctor(Expr& e, int sid) {
    const StructDef& d = (*g_structs)[size_t(sid)];
    Ty t;
    t.cat = Ty::Struct;
    t.sid = sid;
    e.ty = t;
    CallInfo ci;
    if (e.args.empty()) {
      ci.kind = 5;
      callinfo[&e] = ci;
      return;
    }
    if (e.args.size() != d.members.size())
      fail(e.line, e.col, "constructor of struct " + d.name + " needs " + std::to_string(d.members.size()) +
                              " arguments, found " + std::to_string(e.args.size()));
    for (size_t i = 0; i < e.args.size(); ++i) {
      const Ty& mt = d.members[i].second;
      const Ty& at = e.args[i]->ty;
      if (!(at == mt || ty_convertible(at, mt)))
        fail(e.args[i]->line, e.args[i]->col, "cannot convert " + wgsl_name(at) + " to " + wgsl_name(mt) +
                                                  " (member '" + d.members[i].first + "')");
      ci.targets.push_back(mt);
    }
    ci.kind = 1;
    callinfo[&e] = ci;
  }

  void check_call(Expr& e) {
    check_args(e);
    if (e.op == "bitcast" && !fmap.count(e.op)) return check_bitcast(e);
    if (!fmap.count(e.op) && struct_id(e.op) >= 0) return check_struct_ctor(e, struct_id(e.op));
    Ty ct;
    bool inferred;
    if (!fmap.count(e.op) && ctor_type(e, ct, inferred)) return check_ctor(e, ct, inferred);
    if (fmap.count(e.op)) return check_user_call(e, *fmap[e.op]);
    if (is_helper(e.op)) return check_helper(e);
    return check_builtin(e);
  }

  void check_ctor(Expr& e, Ty t, bool inferred) {
    CallInfo ci;
    ci.fn.clear();
    const size_t na = e.args.size();
    if (t.cat == Ty::Arr) {
      if (inferred) {
        // array(e1, ..., eN): the element type is the common type of the
        // arguments (abstract scalars made concrete)
        if (na == 0) fail(e.line, e.col, "cannot infer the type of an empty array constructor");
        Ty el = e.args[0]->ty;
        for (auto& a : e.args) {
          const Ty& at = a->ty;
          if (at.cat == Ty::Arr || at.cat == Ty::Struct) {  // arrays of arrays / of structs
            if (!(concretize(at) == concretize(el)))
              fail(a->line, a->col, "array elements of different types: " + wgsl_name(el) + " and " + wgsl_name(at));
            continue;
          }
          if (at.cat != Ty::Scalar && at.cat != Ty::Vec && at.cat != Ty::Mat)
            fail(a->line, a->col, "invalid array element " + wgsl_name(at));
          if (at.cat != el.cat || at.n != el.n || at.r != el.r)
            fail(a->line, a->col, "array elements of different types: " + wgsl_name(el) + " and " + wgsl_name(at));
          SK u;
          if (!unify_sk(el.s, at.s, u)) fail(a->line, a->col, "array elements of different types");
          el.s = u;
        }
        t = arrT(concretize(el), int(na));
      }
      e.ty = t;
      if (na == 0) { ci.kind = 5; callinfo[&e] = ci; return; }
      if (int(na) != t.alen)
        fail(e.line, e.col, wgsl_name(t) + " constructor needs " + std::to_string(t.alen) + " elements, found " +
                                std::to_string(na));
      const Ty el = elemT(t);
      for (auto& a : e.args) {
        if (!(a->ty == el || ty_convertible(a->ty, el)))
          fail(a->line, a->col, "cannot convert " + wgsl_name(a->ty) + " to " + wgsl_name(el));
        ci.targets.push_back(el);
      }
      ci.kind = 1;  // element-wise constructor
      callinfo[&e] = ci;
      return;
    }
    if (t.cat == Ty::Scalar) {
      if (na == 0) { e.ty = t; ci.kind = 5; callinfo[&e] = ci; return; }
      if (na != 1 || e.args[0]->ty.cat != Ty::Scalar)
        fail(e.line, e.col, "scalar constructor " + wgsl_name(t) + " takes one scalar");
      Expr& a = *e.args[0];
      e.ty = t;
      ci.kind = 4;
      ci.targets.push_back(concretize(a.ty));
      if (t.s == SK::I32 && is_float(a.ty.s)) ci.fn = "::wgsl::to_i32";
      if (t.s == SK::U32 && is_float(a.ty.s)) ci.fn = "::wgsl::to_u32";
      callinfo[&e] = ci;
      return;
    }
    if (t.cat == Ty::Vec) {
      if (inferred) {
        // infer the element type from the arguments
        SK u = SK::AInt;
        bool first = true;
        for (auto& a : e.args) {
          if (a->ty.cat != Ty::Scalar && a->ty.cat != Ty::Vec) fail(a->line, a->col, "invalid vector component " + wgsl_name(a->ty));
          if (first) { u = a->ty.s; first = false; }
          else if (!unify_sk(u, a->ty.s, u)) fail(a->line, a->col, "mismatched vector component types");
        }
        if (first) fail(e.line, e.col, "cannot infer the type of an empty vector constructor");
        t.s = concrete_sk(u);
      }
      e.ty = t;
      if (na == 0) { ci.kind = 5; callinfo[&e] = ci; return; }
      if (na == 1 && e.args[0]->ty.cat == Ty::Vec) {
        Expr& a = *e.args[0];
        if (a.ty.n != t.n) fail(e.line, e.col, "cannot construct " + wgsl_name(t) + " from " + wgsl_name(a.ty));
        ci.kind = 4;  // conversion
        ci.targets.push_back(a.ty);
        callinfo[&e] = ci;
        return;
      }
      int total = 0;
      for (auto& a : e.args) {
        Ty at = a->ty;
        if (at.cat == Ty::Scalar) {
          if (!convertible(at.s, t.s)) fail(a->line, a->col, "cannot convert " + wgsl_name(at) + " to " + sk_name(t.s));
          total += 1;
          ci.targets.push_back(scalar(t.s));
        } else if (at.cat == Ty::Vec) {
          if (!convertible(at.s, t.s)) fail(a->line, a->col, "cannot convert " + wgsl_name(at) + " to " + wgsl_name(vecT(t.s, at.n)));
          total += at.n;
          ci.targets.push_back(vecT(t.s, at.n));
        } else {
          fail(a->line, a->col, "invalid vector component " + wgsl_name(at));
        }
      }
      if (na == 1 && total == 1) {
        ci.kind = 1;  // splat
        callinfo[&e] = ci;
        return;
      }
      if (total != t.n) fail(e.line, e.col, "wrong number of components for " + wgsl_name(t) + ": " + std::to_string(total));
      ci.kind = 1;
      callinfo[&e] = ci;
      return;
    }
    // matrices
    e.ty = t;
    if (na == 0) { ci.kind = 5; callinfo[&e] = ci; return; }
    if (na == 1 && e.args[0]->ty.cat == Ty::Mat) {
      if (!(e.args[0]->ty == t)) fail(e.line, e.col, "cannot construct " + wgsl_name(t) + " from " + wgsl_name(e.args[0]->ty));
      ci.kind = 4;
      ci.targets.push_back(t);
      callinfo[&e] = ci;
      return;
    }
    if (int(na) == t.n) {
      for (auto& a : e.args) {
        if (!(a->ty.cat == Ty::Vec && a->ty.n == t.r && is_float(a->ty.s)))
          fail(a->line, a->col, "matrix column must be " + wgsl_name(vecT(SK::F32, t.r)) + ", found " + wgsl_name(a->ty));
        ci.targets.push_back(vecT(SK::F32, t.r));
      }
      ci.kind = 2;
      callinfo[&e] = ci;
      return;
    }
    if (int(na) == t.n * t.r) {
      for (auto& a : e.args) {
        if (!(a->ty.cat == Ty::Scalar && convertible(a->ty.s, SK::F32)))
          fail(a->line, a->col, "matrix element must be f32, found " + wgsl_name(a->ty));
        ci.targets.push_back(scalar(SK::F32));
      }
      ci.kind = 3;
      callinfo[&e] = ci;
      return;
    }
    fail(e.line, e.col, "wrong number of arguments for " + wgsl_name(t));
  }

  void check_user_call(Expr& e, Func& f) {
    check_function(f);
    if (e.args.size() != f.params.size())
      fail(e.line, e.col, "function '" + f.name + "' expects " + std::to_string(f.params.size()) + " arguments, got " + std::to_string(e.args.size()));
    CallInfo ci;
    for (size_t i = 0; i < f.params.size(); ++i) {
      Expr& a = *e.args[i];
      if (!(a.ty == f.params[i].ty || ty_convertible(a.ty, f.params[i].ty)))
        fail(a.line, a.col, "argument " + std::to_string(i + 1) + " of '" + f.name + "': expected " + wgsl_name(f.params[i].ty) + ", found " + wgsl_name(a.ty));
      ci.targets.push_back(f.params[i].ty);
    }
    // two pointer arguments into the same variable would alias (WGSL rejects
    // such a call): compare the roots of the '&' arguments
    std::set<std::string> roots;
    for (auto& a : e.args) {
      if (a->ty.cat != Ty::Ptr || a->kind != Expr::Unary) continue;
      const Expr* r = a->args[0].get();
      while (r->kind == Expr::Member || r->kind == Expr::Index || (r->kind == Expr::Unary && r->op == "*"))
        r = r->args[0].get();
      if (r->kind == Expr::Name && !roots.insert(r->op).second)
        fail(a->line, a->col, "two pointer arguments of '" + f.name + "' refer to '" + r->op + "' (aliasing)");
    }
    ci.fn = f.name == "field_function" ? f.name : "u_" + f.name;
    e.ty = f.has_ret ? f.ret : voidT();
    e.fl += f.fl;
    e.tr += f.tr;
    callinfo[&e] = ci;
  }

  void check_helper(Expr& e) {
    const std::string& n = e.op;
    const Ty f = scalar(SK::F32), v3 = vecT(SK::F32, 3);
    std::vector<Ty> sig;
    Ty ret = v3;
    int fl = 0, tr = 0;
    if (n == "rotateX" || n == "rotateY" || n == "rotateZ") { sig = {v3, f}; fl = 15; tr = 2; }
    else if (n == "translate") { sig = {v3, f, f, f}; fl = 3; }
    else if (n == "refraction_index") { sig = {f}; ret = f; fl = 10; }
    else if (n == "refraction") { sig = {f, f, v3, v3}; fl = 2 * 10 + 5 + 1 + 5 + 12; }
    else if (n == "point_plane_distance") { sig = {v3, v3, v3}; ret = f; fl = 11; }
    else if (n == "sigmoid") { sig = {f}; ret = f; fl = 2; tr = 1; }
    if (e.args.size() != sig.size())
      fail(e.line, e.col, "function '" + n + "' expects " + std::to_string(sig.size()) + " arguments, got " + std::to_string(e.args.size()));
    CallInfo ci;
    for (size_t i = 0; i < sig.size(); ++i) {
      Expr& a = *e.args[i];
      if (!(a.ty == sig[i] || ty_convertible(a.ty, sig[i])))
        fail(a.line, a.col, "argument " + std::to_string(i + 1) + " of '" + n + "': expected " + wgsl_name(sig[i]) + ", found " + wgsl_name(a.ty));
      ci.targets.push_back(sig[i]);
    }
    ci.fn = "::wgsl::" + n;
    e.ty = ret;
    e.fl += fl;
    e.tr += tr;
    callinfo[&e] = ci;
  }

  // Common argument type of a builtin (all args unified), float-only or not.
  Ty unify_args(Expr& e, size_t first, size_t count, bool float_only, bool allow_int) {
    Ty t;
    bool init = false;
    for (size_t i = first; i < first + count; ++i) {
      Expr& a = *e.args[i];
      if (!(a.ty.cat == Ty::Scalar || a.ty.cat == Ty::Vec) || a.ty.s == SK::Bool)
        fail(a.line, a.col, "invalid argument " + wgsl_name(a.ty) + " to '" + e.op + "'");
      if (!init) { t = a.ty; init = true; continue; }
      if (a.ty.cat != t.cat || (t.cat == Ty::Vec && a.ty.n != t.n))
        fail(a.line, a.col, "mismatched arguments to '" + e.op + "': " + wgsl_name(t) + " and " + wgsl_name(a.ty));
      SK u;
      if (!unify_sk(t.s, a.ty.s, u)) fail(a.line, a.col, "mismatched arguments to '" + e.op + "'");
      t.s = u;
    }
    if (float_only) {
      if (t.s == SK::AInt) t.s = SK::AFloat;
      if (!is_float(t.s)) fail(e.line, e.col, "'" + e.op + "' needs floating-point arguments, found " + wgsl_name(t));
    } else if (!allow_int && !is_float(t.s)) {
      fail(e.line, e.col, "'" + e.op + "' needs floating-point arguments");
    }
    return t;
  }

  void need_args(Expr& e, size_t n) {
    if (e.args.size() != n)
      fail(e.line, e.col, "builtin '" + e.op + "' expects " + std::to_string(n) + " arguments, got " + std::to_string(e.args.size()));
  }

  static bool all_cst(Expr& e) {
    for (auto& a : e.args)
      if (!a->cst) return false;
    return !e.args.empty();
  }

  // Folds a builtin over abstract constants (WGSL const-evaluation in
  // AbstractFloat precision); returns false when not foldable.
  static bool fold_builtin(const std::string& n, const std::vector<double>& x, double& r) {
    if (x.size() == 1) {
      double v = x[0];
      if (n == "sin") r = std::sin(v); else if (n == "cos") r = std::cos(v); else if (n == "tan") r = std::tan(v);
      else if (n == "asin") r = std::asin(v); else if (n == "acos") r = std::acos(v); else if (n == "atan") r = std::atan(v);
      else if (n == "sinh") r = std::sinh(v); else if (n == "cosh") r = std::cosh(v); else if (n == "tanh") r = std::tanh(v);
      else if (n == "asinh") r = std::asinh(v); else if (n == "acosh") r = std::acosh(v); else if (n == "atanh") r = std::atanh(v);
      else if (n == "exp") r = std::exp(v); else if (n == "exp2") r = std::exp2(v); else if (n == "log") r = std::log(v);
      else if (n == "log2") r = std::log2(v); else if (n == "floor") r = std::floor(v); else if (n == "ceil") r = std::ceil(v);
      else if (n == "trunc") r = std::trunc(v); else if (n == "round") r = std::nearbyint(v); else if (n == "fract") r = v - std::floor(v);
      else if (n == "sign") r = v > 0 ? 1 : (v < 0 ? -1 : 0); else if (n == "saturate") r = std::fmin(std::fmax(v, 0.0), 1.0);
      else if (n == "degrees") r = v * 57.295779513082320876798; else if (n == "radians") r = v * 0.017453292519943295769;
      else if (n == "sqrt") r = std::sqrt(v); else if (n == "inverseSqrt") r = 1.0 / std::sqrt(v);
      else if (n == "abs") r = std::fabs(v);
      else return false;
      return true;
    }
    if (x.size() == 2) {
      if (n == "pow") r = std::pow(x[0], x[1]); else if (n == "atan2") r = std::atan2(x[0], x[1]);
      else if (n == "step") r = x[1] >= x[0] ? 1.0 : 0.0; else if (n == "min") r = std::fmin(x[0], x[1]);
      else if (n == "max") r = std::fmax(x[0], x[1]);
      else return false;
      return true;
    }
    if (x.size() == 3 && n == "clamp") { r = std::fmin(std::fmax(x[0], x[1]), x[2]); return true; }
    return false;
  }

  void check_builtin(Expr& e) {
    const std::string& n = e.op;
    for (auto& a : e.args) {
      if (a->ty.cat == Ty::Arr) fail(a->line, a->col, "built-in '" + n + "' does not take an array argument");
      if (a->ty.cat == Ty::Struct) fail(a->line, a->col, "built-in '" + n + "' does not take a struct argument");
    }
    CallInfo ci;
    ci.fn = "::wgsl::" + n;
    static const std::set<std::string> transc1 = {"sin", "cos", "tan", "asin", "acos", "atan", "sinh", "cosh",
                                                  "tanh", "asinh", "acosh", "atanh", "exp", "exp2", "log", "log2"};
    static const std::set<std::string> cheap1 = {"floor", "ceil", "trunc", "round", "fract", "sign", "saturate",
                                                 "degrees", "radians", "sqrt", "inverseSqrt"};
    // component-wise builtins: common argument type t; folded when every
    // argument is an abstract scalar constant, otherwise concrete.
    auto componentwise = [&](Ty t, int per_fl, int per_tr) {
      if (all_cst(e) && t.cat == Ty::Scalar && is_abstract(t.s)) {
        std::vector<double> xs;
        for (auto& a : e.args) xs.push_back(a->cv);
        double r;
        if (fold_builtin(n, xs, r)) {
          e.ty = t;
          e.cst = true;
          e.cv = r;
          return;
        }
      }
      t = concretize(t);
      e.ty = t;
      int k = vcount(t);
      if (t.s == SK::F32) {
        e.fl += per_fl * k;
        e.tr += per_tr * k;
      }
      for (size_t i = 0; i < e.args.size(); ++i) ci.targets.push_back(t);
      callinfo[&e] = ci;
    };
    if (transc1.count(n) || cheap1.count(n)) {
      need_args(e, 1);
      Ty t = unify_args(e, 0, 1, true, false);
      int fl = 0, trc = 0;
      if (transc1.count(n)) trc = 1;
      else if (n == "sqrt") fl = 1;
      else if (n == "inverseSqrt") fl = 2;
      else if (n == "fract" || n == "degrees" || n == "radians") fl = 1;
      return componentwise(t, fl, trc);
    }
    if (n == "abs") {
      need_args(e, 1);
      return componentwise(unify_args(e, 0, 1, false, true), 0, 0);
    }
    if (n == "pow" || n == "atan2" || n == "step") {
      need_args(e, 2);
      componentwise(unify_args(e, 0, 2, true, false), 0, n == "step" ? 0 : 1);
      // a constant scalar exponent lets fast modules use sqrt / products
      if (n == "pow" && !e.cst && e.ty.cat == Ty::Scalar && e.args[1]->cst) callinfo[&e].fn = "::wgsl::pow_k";
      return;
    }
    if (n == "min" || n == "max") {
      need_args(e, 2);
      return componentwise(unify_args(e, 0, 2, false, true), 0, 0);
    }
    if (n == "clamp") {
      need_args(e, 3);
      return componentwise(unify_args(e, 0, 3, false, true), 0, 0);
    }
    if (n == "fma" || n == "smoothstep") {
      need_args(e, 3);
      return componentwise(unify_args(e, 0, 3, true, false), n == "fma" ? 2 : 8, 0);
    }
    if (n == "mix") {
      need_args(e, 3);
      Ty t = concretize(unify_args(e, 0, 2, true, false));
      Expr& c = *e.args[2];
      Ty tc;
      if (c.ty.cat == Ty::Scalar && convertible(c.ty.s, SK::F32)) {
        tc = scalar(SK::F32);
      } else if (c.ty.cat == Ty::Vec && t.cat == Ty::Vec && c.ty.n == t.n && convertible(c.ty.s, SK::F32)) {
        tc = t;
      } else {
        fail(c.line, c.col, "invalid mix factor " + wgsl_name(c.ty));
      }
      e.ty = t;
      e.fl += 4 * vcount(t);
      ci.targets = {t, t, tc};
      callinfo[&e] = ci;
      return;
    }
    // ---- integer bit builtins: i32 / u32 scalars and vectors ----
    auto int_arg = [&](size_t i) {
      Expr& a = *e.args[i];
      if (!((a.ty.cat == Ty::Scalar || a.ty.cat == Ty::Vec) &&
            (a.ty.s == SK::I32 || a.ty.s == SK::U32 || a.ty.s == SK::AInt)))
        fail(a.line, a.col, "'" + n + "' needs an i32 or u32 scalar or vector, found " + wgsl_name(a.ty));
      return concretize(a.ty);
    };
    auto fixed_arg = [&](size_t i, const Ty& want) {
      Expr& a = *e.args[i];
      if (!(a.ty == want || ty_convertible(a.ty, want)))
        fail(a.line, a.col, "argument " + std::to_string(i + 1) + " of '" + n + "' must be " + wgsl_name(want) +
                                ", found " + wgsl_name(a.ty));
      return want;
    };
    auto float_arg = [&](size_t i) {
      Expr& a = *e.args[i];
      if (!((a.ty.cat == Ty::Scalar || a.ty.cat == Ty::Vec) &&
            (a.ty.s == SK::F32 || a.ty.s == SK::AFloat || a.ty.s == SK::AInt)))
        fail(a.line, a.col, "'" + n + "' needs an f32 scalar or vector, found " + wgsl_name(a.ty));
      Ty t = a.ty;
      t.s = SK::F32;
      return t;
    };
    auto finish = [&](const Ty& result, std::vector<Ty> targets, int fl) {
      e.ty = result;
      e.fl += fl;
      ci.targets = std::move(targets);
      callinfo[&e] = ci;
    };
    static const std::set<std::string> bits1 = {"countLeadingZeros", "countOneBits", "countTrailingZeros",
                                                "reverseBits", "firstLeadingBit", "firstTrailingBit"};
    if (bits1.count(n)) {
      need_args(e, 1);
      const Ty t = int_arg(0);
      return finish(t, {t}, 0);
    }
    if (n == "extractBits") {
      need_args(e, 3);
      const Ty t = int_arg(0), u = scalar(SK::U32);
      return finish(t, {t, fixed_arg(1, u), fixed_arg(2, u)}, 0);
    }
    if (n == "insertBits") {
      need_args(e, 4);
      const Ty t = int_arg(0), u = scalar(SK::U32);
      return finish(t, {t, fixed_arg(1, t), fixed_arg(2, u), fixed_arg(3, u)}, 0);
    }
    // ---- float decomposition ----
    if (n == "ldexp") {
      need_args(e, 2);
      const Ty t = float_arg(0);
      Ty ti = t;
      ti.s = SK::I32;
      return finish(t, {t, fixed_arg(1, ti)}, vcount(t));
    }
    if (n == "quantizeToF16") {
      need_args(e, 1);
      const Ty t = float_arg(0);
      return finish(t, {t}, 0);
    }
    if (n == "frexp" || n == "modf") {
      need_args(e, 1);
      const Ty t = float_arg(0);
      Ty ti = t;
      ti.s = SK::I32;
      // WGSL's built-in result structure (__frexp_result_f32,
      // __modf_result_vec3_f32, ...): fract and exp, or fract and whole
      const std::string shape = t.cat == Ty::Vec ? "vec" + std::to_string(t.n) + "_f32" : std::string("f32");
      const std::string sname = "__" + n + "_result_" + shape;
      int sid = struct_id(sname);
      if (sid < 0) {
        StructDef d;
        d.name = sname;
        if (n == "frexp") {
          d.members = {{"fract", t}, {"exp", ti}};
          d.cpp = "::wgsl::frexp_result<" + cpp_name(t) + "," + cpp_name(ti) + ">";
        } else {
          d.members = {{"fract", t}, {"whole", t}};
          d.cpp = "::wgsl::modf_result<" + cpp_name(t) + ">";
        }
        g_structs->push_back(d);
        sid = int(g_structs->size()) - 1;
      }
      Ty st;
      st.cat = Ty::Struct;
      st.sid = sid;
      return finish(st, {t}, n == "modf" ? vcount(t) : 0);
    }
    // ---- data packing ----
    const Ty u32t = scalar(SK::U32), v4f = vecT(SK::F32, 4), v2f = vecT(SK::F32, 2);
    if (n == "pack4x8snorm" || n == "pack4x8unorm") {
      need_args(e, 1);
      return finish(u32t, {fixed_arg(0, v4f)}, 12);
    }
    if (n == "pack2x16snorm" || n == "pack2x16unorm" || n == "pack2x16float") {
      need_args(e, 1);
      return finish(u32t, {fixed_arg(0, v2f)}, n == "pack2x16float" ? 0 : 6);
    }
    if (n == "unpack4x8snorm" || n == "unpack4x8unorm") {
      need_args(e, 1);
      return finish(v4f, {fixed_arg(0, u32t)}, 4);
    }
    if (n == "unpack2x16snorm" || n == "unpack2x16unorm" || n == "unpack2x16float") {
      need_args(e, 1);
      return finish(v2f, {fixed_arg(0, u32t)}, n == "unpack2x16float" ? 0 : 2);
    }
    if (n == "pack4xI8" || n == "pack4xI8Clamp") {
      need_args(e, 1);
      return finish(u32t, {fixed_arg(0, vecT(SK::I32, 4))}, 0);
    }
    if (n == "pack4xU8" || n == "pack4xU8Clamp") {
      need_args(e, 1);
      return finish(u32t, {fixed_arg(0, vecT(SK::U32, 4))}, 0);
    }
    if (n == "unpack4xI8") {
      need_args(e, 1);
      return finish(vecT(SK::I32, 4), {fixed_arg(0, u32t)}, 0);
    }
    if (n == "unpack4xU8") {
      need_args(e, 1);
      return finish(vecT(SK::U32, 4), {fixed_arg(0, u32t)}, 0);
    }
    if (n == "dot4U8Packed" || n == "dot4I8Packed") {
      need_args(e, 2);
      return finish(scalar(n == "dot4U8Packed" ? SK::U32 : SK::I32), {fixed_arg(0, u32t), fixed_arg(1, u32t)}, 0);
    }
    if (n == "dot") {
      need_args(e, 2);
      Ty t = concretize(unify_args(e, 0, 2, false, true));
      if (t.cat != Ty::Vec) fail(e.line, e.col, "'dot' needs vector arguments");
      e.ty = scalar(t.s);
      if (t.s == SK::F32) e.fl += 2 * t.n - 1;
      ci.targets = {t, t};
      callinfo[&e] = ci;
      return;
    }
    if (n == "cross") {
      need_args(e, 2);
      Ty t = concretize(unify_args(e, 0, 2, true, false));
      if (!(t.cat == Ty::Vec && t.n == 3)) fail(e.line, e.col, "'cross' needs vec3<f32> arguments");
      e.ty = t;
      e.fl += 9;
      ci.targets = {t, t};
      callinfo[&e] = ci;
      return;
    }
    if (n == "length" || n == "normalize") {
      need_args(e, 1);
      Ty t = concretize(unify_args(e, 0, 1, true, false));
      int k = vcount(t);
      if (n == "length") {
        e.ty = scalar(SK::F32);
        e.fl += t.cat == Ty::Vec ? (2 * k - 1) + 1 : 0;
      } else {
        if (t.cat != Ty::Vec) fail(e.line, e.col, "'normalize' needs a vector argument");
        e.ty = t;
        e.fl += (2 * k - 1) + 1 + k;
      }
      ci.targets = {t};
      callinfo[&e] = ci;
      return;
    }
    if (n == "distance") {
      need_args(e, 2);
      Ty t = concretize(unify_args(e, 0, 2, true, false));
      int k = vcount(t);
      e.ty = scalar(SK::F32);
      e.fl += t.cat == Ty::Vec ? k + (2 * k - 1) + 1 : 1;
      ci.targets = {t, t};
      callinfo[&e] = ci;
      return;
    }
    if (n == "reflect" || n == "faceForward") {
      need_args(e, n == "reflect" ? 2 : 3);
      Ty t = concretize(unify_args(e, 0, e.args.size(), true, false));
      if (t.cat != Ty::Vec) fail(e.line, e.col, "'" + n + "' needs vector arguments");
      e.ty = t;
      e.fl += n == "reflect" ? (2 * t.n - 1) + 1 + 2 * t.n : (2 * t.n - 1);
      for (size_t i = 0; i < e.args.size(); ++i) ci.targets.push_back(t);
      callinfo[&e] = ci;
      return;
    }
    if (n == "refract") {
      need_args(e, 3);
      Ty t = concretize(unify_args(e, 0, 2, true, false));
      if (t.cat != Ty::Vec) fail(e.line, e.col, "'refract' needs vector arguments");
      Expr& c = *e.args[2];
      if (!(c.ty.cat == Ty::Scalar && convertible(c.ty.s, SK::F32))) fail(c.line, c.col, "'refract' eta must be f32");
      e.ty = t;
      e.fl += (2 * t.n - 1) + 6 + 1 + 4 * t.n;
      ci.targets = {t, t, scalar(SK::F32)};
      callinfo[&e] = ci;
      return;
    }
    if (n == "select") {
      need_args(e, 3);
      Expr& f = *e.args[0];
      Expr& t = *e.args[1];
      Expr& c = *e.args[2];
      if (!(f.ty.cat == t.ty.cat && (f.ty.cat != Ty::Vec || f.ty.n == t.ty.n) && f.ty.cat != Ty::Mat && f.ty.cat != Ty::Void))
        fail(e.line, e.col, "'select' arguments must have the same type");
      SK u;
      if (!unify_sk(f.ty.s, t.ty.s, u)) fail(e.line, e.col, "'select' arguments must have the same type");
      Ty ty = f.ty;
      ty.s = concrete_sk(u);
      if (!(c.ty.s == SK::Bool && (c.ty.cat == Ty::Scalar || (c.ty.cat == Ty::Vec && ty.cat == Ty::Vec && c.ty.n == ty.n))))
        fail(c.line, c.col, "'select' condition must be bool or a bool vector of the same size");
      e.ty = ty;
      ci.targets = {ty, ty, c.ty};
      callinfo[&e] = ci;
      return;
    }
    if (n == "all" || n == "any") {
      need_args(e, 1);
      Expr& a = *e.args[0];
      if (a.ty.s != SK::Bool || a.ty.cat == Ty::Mat) fail(a.line, a.col, "'" + n + "' needs a bool vector");
      e.ty = scalar(SK::Bool);
      ci.targets = {a.ty};
      callinfo[&e] = ci;
      return;
    }
    if (n == "transpose" || n == "determinant") {
      need_args(e, 1);
      Expr& a = *e.args[0];
      if (a.ty.cat != Ty::Mat) fail(a.line, a.col, "'" + n + "' needs a matrix");
      if (n == "determinant") {
        if (a.ty.n != a.ty.r || a.ty.n > 3) fail(a.line, a.col, "'determinant' supports mat2x2 and mat3x3");
        e.ty = scalar(SK::F32);
        e.fl += a.ty.n == 2 ? 3 : 14;
      } else {
        e.ty = matT(a.ty.r, a.ty.n);
      }
      ci.targets = {a.ty};
      callinfo[&e] = ci;
      return;
    }
    if (n == "field_function") fail(e.line, e.col, "recursion is not allowed: 'field_function' calls itself");
    fail(e.line, e.col, "unknown function: '" + n + "'");
  }

  // ---- expression emission ----
  std::string ex(Expr& e) {
    switch (e.kind) {
      case Expr::Lit:
        if (e.lit == 3) return e.bval ? "true" : "false";
        if (e.cst) return lit_as(e.cv, concretize(e.ty), e.line, e.col);
        if (e.lit == 2) return f32_literal(double(float(e.lf)));
        if (e.ty.s == SK::U32) return std::to_string((unsigned long long)e.li) + "u";
        return std::to_string(e.li);
      case Expr::Name: {
        if (e.cst) return lit_as(e.cv, concretize(e.ty), e.line, e.col);
        if (e.op == "PI" && !lookup("PI")) return f32_literal(3.141592653589793);
        Sym* s = lookup(e.op);
        return s->cpp;
      }
      case Expr::Unary:
        if (e.cst) return lit_as(e.cv, concretize(e.ty), e.line, e.col);
        // a pointer is a C++ reference: &x and *p are the reference itself
        if (e.op == "&" || e.op == "*") return ex(*e.args[0]);
        if (e.op == "-" && e.ty.s == SK::I32) return "::wgsl::neg_i32(" + ex(*e.args[0]) + ")";  // -INT_MIN wraps
        return "(" + e.op + ex(*e.args[0]) + ")";
      case Expr::Binary: {
        if (e.cst) return lit_as(e.cv, concretize(e.ty), e.line, e.col);
        BinInfo& bi = bininfo[&e];
        std::string a = ex_as(*e.args[0], bi.tl), b = ex_as(*e.args[1], bi.tr);
        const std::string& op = e.op;
        bool vec = e.args[0]->ty.cat == Ty::Vec || e.args[1]->ty.cat == Ty::Vec;
        if (op == "%" && is_float(e.ty.s)) return "::wgsl::fmod_wgsl(" + a + ", " + b + ")";
        // integer '/' and '%' with WGSL's results for a zero divisor and for
        // the most negative i32 over -1; shifts use the amount's low 5 bits
        if ((op == "/" || op == "%") && (e.ty.s == SK::I32 || e.ty.s == SK::U32))
          return std::string("::wgsl::") + (op == "/" ? "div_int(" : "mod_int(") + a + ", " + b + ")";
        if (op == "<<" || op == ">>") return std::string("::wgsl::") + (op == "<<" ? "shl(" : "shr(") + a + ", " + b + ")";
        // i32 + - * wrap on overflow (WGSL); computed in u32, no undefined behaviour
        if ((op == "+" || op == "-" || op == "*") && e.ty.s == SK::I32)
          return std::string("::wgsl::") + (op == "+" ? "add_i32(" : op == "-" ? "sub_i32(" : "mul_i32(") + a + ", " +
                 b + ")";
        // dot(a, b) + s or s + dot(a, b) in f32: fast modules fold s into the
        // dot product's first FMA (wgsl_rt.cuh dot_add); precise modules and
        // the host add as written (IEEE addition commutes, so either order is
        // the shader's value)
        if (op == "+" && e.ty.cat == Ty::Scalar && e.ty.s == SK::F32) {
          for (int side = 0; side < 2; ++side) {
            Expr& D = *e.args[size_t(side)];
            auto ci = callinfo.find(&D);
            if (D.kind == Expr::Call && !D.cst && ci != callinfo.end() && ci->second.fn == "::wgsl::dot" &&
                ci->second.targets[0].s == SK::F32)
              return "::wgsl::dot_add(" + ex_as(*D.args[0], ci->second.targets[0]) + ", " +
                     ex_as(*D.args[1], ci->second.targets[1]) + ", " + (side == 0 ? b : a) + ")";
          }
        }
        // a / pow(x, k) with a constant exponent: fast modules multiply by
        // pow(x, -k) (see wgsl_rt.cuh div_pow_k); precise modules divide
        if (op == "/" && is_float(e.ty.s)) {
          Expr& R = *e.args[1];
          auto ci = callinfo.find(&R);
          if (R.kind == Expr::Call && !R.cst && ci != callinfo.end() && ci->second.fn == "::wgsl::pow_k") {
            const std::string xk = ex_as(*R.args[0], ci->second.targets[0]) + ", " +
                                   ex_as(*R.args[1], ci->second.targets[1]);
            // (s * V) / pow(x, k) with a scalar s and a vector V: fast
            // modules scale V once by s * pow(x, -k) (div_pow_k_sv)
            Expr& L = *e.args[0];
            if (L.kind == Expr::Binary && L.op == "*" && !L.cst && e.ty.cat == Ty::Vec) {
              BinInfo& li = bininfo[&L];
              const bool s0 = L.args[0]->ty.cat == Ty::Scalar && L.args[1]->ty.cat == Ty::Vec;
              const bool s1 = L.args[1]->ty.cat == Ty::Scalar && L.args[0]->ty.cat == Ty::Vec;
              if (s0)
                return "::wgsl::div_pow_k_sv(" + ex_as(*L.args[0], li.tl) + ", " + ex_as(*L.args[1], li.tr) + ", " +
                       xk + ")";
              if (s1)
                return "::wgsl::div_pow_k_vs(" + ex_as(*L.args[0], li.tl) + ", " + ex_as(*L.args[1], li.tr) + ", " +
                       xk + ")";
            }
            return "::wgsl::div_pow_k(" + a + ", " + xk + ")";
          }
        }
        if (vec) {
          if (op == "<") return "::wgsl::cmp_lt(" + a + ", " + b + ")";
          if (op == "<=") return "::wgsl::cmp_le(" + a + ", " + b + ")";
          if (op == ">") return "::wgsl::cmp_gt(" + a + ", " + b + ")";
          if (op == ">=") return "::wgsl::cmp_ge(" + a + ", " + b + ")";
          if (op == "==") return "::wgsl::cmp_eq(" + a + ", " + b + ")";
          if (op == "!=") return "::wgsl::cmp_ne(" + a + ", " + b + ")";
          if ((op == "&" || op == "|") && e.ty.s == SK::Bool) return std::string("::wgsl::") + (op == "&" ? "land(" : "lor(") + a + ", " + b + ")";
        }
        if ((op == "&" || op == "|" || op == "^") && e.ty.s == SK::Bool && e.ty.cat == Ty::Scalar)
          return "bool(" + a + " " + op + " " + b + ")";
        return "(" + a + " " + op + " " + b + ")";
      }
      case Expr::Member: {
        std::string a = ex(*e.args[0]);
        if (e.args[0]->ty.cat == Ty::Struct) return a + ".m_" + e.op;
        static const char* comp = "xyzw";
        if (e.op.size() == 1) return a + "." + comp[swz_index(e.op[0])];
        std::string s = "::wgsl::swz<";
        for (size_t i = 0; i < e.op.size(); ++i) s += (i ? "," : "") + std::to_string(swz_index(e.op[i]));
        return s + ">(" + a + ")";
      }
      case Expr::Index:
        return ex(*e.args[0]) + "[" + ex_as(*e.args[1], concretize(e.args[1]->ty)) + "]";
      case Expr::Call: {
        if (e.cst) return lit_as(e.cv, concretize(e.ty), e.line, e.col);
        CallInfo& ci = callinfo[&e];
        std::vector<std::string> as;
        for (size_t i = 0; i < e.args.size(); ++i) as.push_back(ex_as(*e.args[i], ci.targets[i]));
        auto join = [&](size_t from) {
          std::string s;
          for (size_t i = from; i < as.size(); ++i) s += (i > from ? ", " : "") + as[i];
          return s;
        };
        switch (ci.kind) {
          case 5: return cpp_name(e.ty) + "()";
          case 4: return (ci.fn.empty() ? cpp_name(e.ty) : ci.fn) + "(" + join(0) + ")";
          case 1: return cpp_name(e.ty) + "(" + join(0) + ")";
          case 2: return "::wgsl::make_mat(" + join(0) + ")";
          case 3: {
            std::string s = "::wgsl::make_mat(";
            for (int c = 0; c < e.ty.n; ++c) {
              s += (c ? ", " : "") + cpp_name(vecT(SK::F32, e.ty.r)) + "(";
              for (int r = 0; r < e.ty.r; ++r) s += (r ? ", " : "") + as[size_t(c * e.ty.r + r)];
              s += ")";
            }
            return s + ")";
          }
          default:
            // user functions also receive the invocation's private variables
            if (ci.fn.compare(0, 2, "u_") == 0 || ci.fn == "field_function") return ci.fn + "(pv" + (as.empty() ? "" : ", ") + join(0) + ")";
            return ci.fn + "(" + join(0) + ")";
        }
      }
    }
    return "";
  }

  // ---- statements ----
  std::string ind(int d) { return std::string(size_t(2 * d), ' '); }

  struct Cost { int fl = 0, tr = 0; };

  bool returns(const std::vector<SP>& b) {
    if (b.empty()) return false;
    const Stmt& s = *b.back();
    if (s.kind == Stmt::Return) return true;
    if (s.kind == Stmt::Block) return returns(s.body);
    if (s.kind == Stmt::If) return !s.els.empty() && returns(s.body) && returns(s.els);
    if (s.kind == Stmt::Switch) {
      for (auto& cl : s.clauses)
        if (!returns(cl.body)) return false;
      return true;  // the type check requires a default clause
    }
    if (s.kind == Stmt::Loop) {
      // a loop without break only leaves through return
      std::function<bool(const std::vector<SP>&)> has_break = [&](const std::vector<SP>& v) {
        for (auto& x : v) {
          if (x->kind == Stmt::Break || x->kind == Stmt::BreakIf) return true;
          if (x->kind == Stmt::If || x->kind == Stmt::Block)
            if (has_break(x->body) || has_break(x->els)) return true;
        }
        return false;
      };
      return !has_break(s.body) && !has_break(s.continuing);
    }
    return false;
  }

  void stmts(std::vector<SP>& b, std::string& out, int d, Cost& c) {
    scopes.emplace_back();
    for (auto& s : b) stmt(*s, out, d, c);
    scopes.pop_back();
  }

  void check_lvalue(Expr& l, const Stmt& s) {
    if (!l.lv) fail(s.line, s.col, "left side of assignment is not a reference");
    if (!l.mut) fail(s.line, s.col, "cannot assign to an immutable value (declared with 'let' or 'const', or a parameter)");
  }

  void stmt(Stmt& s, std::string& out, int d, Cost& c) {
    switch (s.kind) {
      case Stmt::Let:
      case Stmt::Const:
      case Stmt::Var: {
        Ty t;
        std::string init;
        bool cst = false;
        double cv = 0;
        if (s.e) {
          check(*s.e);
          c.fl += s.e->fl;
          c.tr += s.e->tr;
          if (s.e->ty.cat == Ty::Void) fail(s.line, s.col, "initializer has no value");
        }
        if (s.has_ty) {
          t = s.ty;
          if (s.e && !(s.e->ty == t || ty_convertible(s.e->ty, t)))
            fail(s.line, s.col, "cannot initialize '" + s.name + "' of type " + wgsl_name(t) + " with " + wgsl_name(s.e->ty));
        } else {
          t = concretize(s.e->ty);
        }
        if (s.kind == Stmt::Const && !s.e->cst && !s.has_ty) {
          // const of a non-abstract expression: treat like let (values are
          // still compile-time constants after C++ folding)
        }
        if (s.kind == Stmt::Const && s.e->cst && !s.has_ty && s.e->ty.cat == Ty::Scalar) {
          // abstract const keeps its abstract value (used at full precision)
          cst = true;
          cv = s.e->cv;
          t = s.e->ty;
        }
        if (t.cat == Ty::Ptr && s.kind != Stmt::Let)
          fail(s.line, s.col, "a pointer can only be declared with 'let'");
        init = s.e ? ex_as(*s.e, concretize(t)) : cpp_name(t) + "()";
        Sym sym;
        sym.ty = cst ? t : concretize(t);
        sym.is_var = s.kind == Stmt::Var;
        sym.cpp = cst ? std::string() : fresh(s.name);
        sym.cst = cst;
        sym.cv = cv;
        if (!cst) {
          // a pointer binds a (non-const) C++ reference to the variable
          const bool konst = !sym.is_var && sym.ty.cat != Ty::Ptr;
          out += ind(d) + (konst ? "const " : "") + cpp_name(sym.ty) + " " + sym.cpp + " = " + init + ";\n";
        }
        declare(s.name, sym, s.line, s.col);
        return;
      }
      case Stmt::Assign: {
        check(*s.lhs);
        check(*s.e);
        check_lvalue(*s.lhs, s);
        if (!(s.e->ty == s.lhs->ty || ty_convertible(s.e->ty, s.lhs->ty)))
          fail(s.line, s.col, "cannot assign " + wgsl_name(s.e->ty) + " to " + wgsl_name(s.lhs->ty));
        c.fl += s.e->fl + s.lhs->fl;
        c.tr += s.e->tr + s.lhs->tr;
        out += ind(d) + ex(*s.lhs) + " = " + ex_as(*s.e, s.lhs->ty) + ";\n";
        return;
      }
      case Stmt::Compound: {
        // lhs op= e  is  lhs = lhs op e
        check(*s.lhs);
        check_lvalue(*s.lhs, s);
        Expr tmp;
        tmp.kind = Expr::Binary;
        tmp.line = s.line;
        tmp.col = s.col;
        tmp.op = s.op;
        // the read side is a fresh copy of the lhs expression
        tmp.args.push_back(clone(*s.lhs));
        tmp.args.push_back(std::move(s.e));
        check(tmp);
        if (!(tmp.ty == s.lhs->ty || ty_convertible(tmp.ty, s.lhs->ty)))
          fail(s.line, s.col, "cannot assign " + wgsl_name(tmp.ty) + " to " + wgsl_name(s.lhs->ty));
        c.fl += tmp.fl;
        c.tr += tmp.tr;
        out += ind(d) + ex(*s.lhs) + " = " + ex_as(tmp, s.lhs->ty) + ";\n";
        s.e = std::move(tmp.args[1]);
        return;
      }
      case Stmt::Incr:
      case Stmt::Decr: {
        check(*s.lhs);
        check_lvalue(*s.lhs, s);
        if (!(s.lhs->ty.cat == Ty::Scalar && is_int(s.lhs->ty.s))) fail(s.line, s.col, "'++'/'--' need an integer variable");
        out += ind(d) + ex(*s.lhs) + (s.kind == Stmt::Incr ? "++" : "--") + ";\n";
        return;
      }
      case Stmt::Phony:
        check(*s.e);
        out += ind(d) + "(void)(" + ex_as(*s.e, concretize(s.e->ty)) + ");\n";
        return;
      case Stmt::ExprS:
        check(*s.e);
        c.fl += s.e->fl;
        c.tr += s.e->tr;
        out += ind(d) + ex(*s.e) + ";\n";
        return;
      case Stmt::Return: {
        if (!cur_fn->has_ret) {
          if (s.e) fail(s.line, s.col, "function '" + cur_fn->name + "' has no return type but returns a value");
          out += ind(d) + "return;\n";
          return;
        }
        if (!s.e) fail(s.line, s.col, "function '" + cur_fn->name + "' must return a value of type " + wgsl_name(cur_fn->ret));
        check(*s.e);
        c.fl += s.e->fl;
        c.tr += s.e->tr;
        if (!(s.e->ty == cur_fn->ret || ty_convertible(s.e->ty, cur_fn->ret)))
          fail(s.e->line, s.e->col, "return type mismatch: expected " + wgsl_name(cur_fn->ret) + ", found " + wgsl_name(s.e->ty));
        out += ind(d) + "return " + ex_as(*s.e, cur_fn->ret) + ";\n";
        return;
      }
      case Stmt::Block: {
        out += ind(d) + "{\n";
        stmts(s.body, out, d + 1, c);
        out += ind(d) + "}\n";
        return;
      }
      case Stmt::If: {
        check(*s.e);
        if (!(s.e->ty.cat == Ty::Scalar && s.e->ty.s == SK::Bool))
          fail(s.e->line, s.e->col, "'if' condition must be bool, found " + wgsl_name(s.e->ty));
        c.fl += s.e->fl;
        c.tr += s.e->tr;
        Cost a, b;
        out += ind(d) + "if (" + ex(*s.e) + ") {\n";
        stmts(s.body, out, d + 1, a);
        out += ind(d) + "}";
        if (!s.els.empty()) {
          out += " else {\n";
          stmts(s.els, out, d + 1, b);
          out += ind(d) + "}";
        }
        out += "\n";
        c.fl += std::max(a.fl, b.fl);
        c.tr += std::max(a.tr, b.tr);
        return;
      }
      case Stmt::For: {
        scopes.emplace_back();
        std::string init, cond = "true", upd;
        Cost body;
        if (s.init) {
          std::string tmp;
          stmt(*s.init, tmp, 0, c);
          init = tmp;
          while (!init.empty() && (init.back() == '\n' || init.back() == ';')) init.pop_back();
        }
        if (s.e) {
          check(*s.e);
          if (!(s.e->ty.cat == Ty::Scalar && s.e->ty.s == SK::Bool)) fail(s.e->line, s.e->col, "'for' condition must be bool");
          cond = ex(*s.e);
          body.fl += s.e->fl;
          body.tr += s.e->tr;
        }
        if (s.update) {
          std::string tmp;
          stmt(*s.update, tmp, 0, body);
          upd = tmp;
          while (!upd.empty() && (upd.back() == '\n' || upd.back() == ';')) upd.pop_back();
        }
        out += ind(d) + "{\n" + ind(d + 1) + init + ";\n";
        out += ind(d + 1) + "for (; " + cond + "; " + upd + ") {\n";
        loop_depth++;
        loop_labels.push_back(std::string());
        stmts(s.body, out, d + 2, body);
        loop_labels.pop_back();
        loop_depth--;
        out += ind(d + 1) + "}\n" + ind(d) + "}\n";
        scopes.pop_back();
        c.fl += body.fl;
        c.tr += body.tr;
        return;
      }
      case Stmt::While: {
        check(*s.e);
        if (!(s.e->ty.cat == Ty::Scalar && s.e->ty.s == SK::Bool)) fail(s.e->line, s.e->col, "'while' condition must be bool");
        out += ind(d) + "while (" + ex(*s.e) + ") {\n";
        loop_depth++;
        loop_labels.push_back(std::string());
        stmts(s.body, out, d + 1, c);
        loop_labels.pop_back();
        loop_depth--;
        out += ind(d) + "}\n";
        c.fl += s.e->fl;
        c.tr += s.e->tr;
        return;
      }
      case Stmt::Loop: {
        const bool has_cont = !s.continuing.empty();
        const std::string label = "linon_continuing_" + std::to_string(label_counter++);
        out += ind(d) + "for (;;) {\n";
        loop_labels.push_back(has_cont ? label : std::string());
        loop_depth++;
        out += ind(d + 1) + "{\n";
        stmts(s.body, out, d + 2, c);
        out += ind(d + 1) + "}\n";
        if (has_cont) {
          out += ind(d + 1) + label + ":;\n";
          scopes.emplace_back();
          for (auto& cs : s.continuing) stmt(*cs, out, d + 1, c);
          scopes.pop_back();
        }
        loop_depth--;
        loop_labels.pop_back();
        out += ind(d) + "}\n";
        return;
      }
      case Stmt::Switch: {
        check(*s.e);
        const Ty st = s.e->ty;
        if (!(st.cat == Ty::Scalar && is_int(st.s)))
          fail(s.e->line, s.e->col, "'switch' selector must be i32 or u32, found " + wgsl_name(st));
        c.fl += s.e->fl;
        c.tr += s.e->tr;
        SK want = st.s;
        int n_default = 0;
        for (auto& cl : s.clauses) {
          if (cl.def) n_default++;
          for (auto& e : cl.sel) {
            check(*e);
            if (!(e->ty.cat == Ty::Scalar && is_int(e->ty.s)))
              fail(e->line, e->col, "case selector must be an integer, found " + wgsl_name(e->ty));
            if (!e->cst && !(e->kind == Expr::Lit && e->lit == 1))
              fail(e->line, e->col, "case selector must be a constant expression");
            if (!is_abstract(e->ty.s)) {
              if (is_abstract(want)) want = e->ty.s;
              else if (e->ty.s != want)
                fail(e->line, e->col, "case selector type " + wgsl_name(e->ty) + " does not match the selector's " +
                                          std::string(sk_name(want)));
            }
          }
        }
        if (n_default != 1)
          fail(s.line, s.col, n_default == 0 ? "switch statement must have a default clause"
                                             : "switch statement has more than one default clause");
        if (is_abstract(want)) want = SK::I32;
        if (!is_abstract(st.s) && st.s != want)
          fail(s.e->line, s.e->col, "switch selector type " + wgsl_name(st) + " does not match its case selectors");
        std::set<long long> seen;
        out += ind(d) + "switch (" + ex_as(*s.e, scalar(want)) + ") {\n";
        Cost worst;
        for (auto& cl : s.clauses) {
          std::string labels;
          for (auto& e : cl.sel) {
            const long long v = e->cst ? (long long)e->cv : e->li;
            const bool ok = want == SK::U32 ? (v >= 0 && v <= 0xffffffffLL) : (v >= INT32_MIN && v <= INT32_MAX);
            if (!ok) fail(e->line, e->col, "case selector " + std::to_string(v) + " out of range for " + sk_name(want));
            if (!seen.insert(v).second) fail(e->line, e->col, "duplicate case selector " + std::to_string(v));
            labels += "case " + std::to_string(v) + (want == SK::U32 ? "u" : "") + ": ";
          }
          if (cl.def) labels += "default: ";
          out += ind(d + 1) + labels + "{\n";
          Cost cc;
          switch_depth++;
          stmts(cl.body, out, d + 2, cc);
          switch_depth--;
          out += ind(d + 1) + "} break;\n";
          worst.fl = std::max(worst.fl, cc.fl);
          worst.tr = std::max(worst.tr, cc.tr);
        }
        out += ind(d) + "}\n";
        c.fl += worst.fl;
        c.tr += worst.tr;
        return;
      }
      case Stmt::ConstAssert:
        check_const_assert(*s.e, s.line, s.col);
        return;
      case Stmt::BreakIf:
        check(*s.e);
        if (!(s.e->ty.cat == Ty::Scalar && s.e->ty.s == SK::Bool)) fail(s.e->line, s.e->col, "'break if' condition must be bool");
        out += ind(d) + "if (" + ex(*s.e) + ") break;\n";
        return;
      case Stmt::Break:
        if (loop_depth == 0 && switch_depth == 0) fail(s.line, s.col, "'break' outside of a loop or switch");
        out += ind(d) + "break;\n";
        return;
      case Stmt::Continue:
        if (loop_depth == 0) fail(s.line, s.col, "'continue' outside of a loop");
        if (!loop_labels.empty() && !loop_labels.back().empty())
          out += ind(d) + "goto " + loop_labels.back() + ";\n";
        else
          out += ind(d) + "continue;\n";
        return;
    }
  }
  std::vector<std::string> loop_labels;  // "" = C++ continue, else goto label
  int label_counter = 0;
  int switch_depth = 0;  // break inside a switch clause leaves the switch

  static EP clone(const Expr& e) {
    EP c = std::make_unique<Expr>();
    c->kind = e.kind;
    c->line = e.line;
    c->col = e.col;
    c->op = e.op;
    c->lit = e.lit;
    c->lf = e.lf;
    c->li = e.li;
    c->suffix = e.suffix;
    c->bval = e.bval;
    c->has_targ = e.has_targ;
    c->targ = e.targ;
    for (auto& a : e.args) c->args.push_back(clone(*a));
    return c;
  }

  void check_function(Func& f) {
    if (f.state == 2) return;
    if (f.state == 1) fail(f.line, f.col, "recursion is not allowed (function '" + f.name + "')");
    f.state = 1;
    Func* saved_fn = cur_fn;
    auto saved_scopes = scopes;
    int saved_loop = loop_depth;
    int saved_switch = switch_depth;
    auto saved_names = name_uses;
    name_uses.clear();
    scopes.clear();
    scopes.emplace_back();
    loop_depth = 0;
    switch_depth = 0;
    cur_fn = &f;
    // every function receives the invocation's private variables
    std::string params = "Private& pv";
    for (size_t i = 0; i < f.params.size(); ++i) {
      const Param& p = f.params[i];
      Sym s;
      s.ty = p.ty;
      s.cpp = fresh(p.name);
      declare(p.name, s, p.line, p.col);
      params += ", " + cpp_name(p.ty) + " " + s.cpp;
    }
    std::string body;
    Cost c;
    stmts(f.body, body, 1, c);
    if (f.has_ret && !returns(f.body))
      fail(f.line, f.col, "function '" + f.name + "' must return a value of type " + wgsl_name(f.ret) + " on every path");
    std::string name = f.name == "field_function" ? "field_function" : "u_" + f.name;
    f.code = "WG_HD " + cpp_name(f.has_ret ? f.ret : voidT()) + " " + name + "(" + params + ") {\n" + body + "}\n";
    f.fl = c.fl;
    f.tr = c.tr;
    cur_fn = saved_fn;
    scopes = saved_scopes;
    loop_depth = saved_loop;
    switch_depth = saved_switch;
    name_uses = saved_names;
    f.state = 2;
  }
};

int count_lines(const std::string& s) {
  int n = 0;
  for (char c : s)
    if (c == '\n') ++n;
  return n;
}

}  // namespace

Translation translate(const std::string& field_body, const std::string& helpers_src,
                      const std::string& ns, bool pair) {
  struct PairScope {
    bool old;
    explicit PairScope(bool on) : old(g_pair) { g_pair = on; }
    ~PairScope() { g_pair = old; }
  } pair_scope(pair);
  Translation tr;
  // The module the reference builds: the shader's helpers followed by the
  // spliced field function (main_view.rs:852-861).  User helpers take the
  // place of edits to main_view.wgsl.
  const std::string header =
      "fn field_function(p_prev: vec3<f32>, p: vec3<f32>, v0: vec3<f32>, v: vec3<f32>, t: f32) -> vec3<f32> {\n";
  const std::string module = helpers_src + "\n" + header + field_body + "\n}\n";
  const int body_first_line = count_lines(helpers_src) + 3;  // 1-based line of the body
  std::vector<StructDef> structs;
  std::vector<Ty> arr_elems;
  struct Reset {
    ~Reset() {
      g_structs = nullptr;
      g_arr_elems = nullptr;
    }
  } reset;
  g_structs = &structs;
  g_arr_elems = &arr_elems;
  try {
    Parser ps(lex(module));
    Compiler cc;
    ps.module(cc.fns, cc.consts);
    // structs may nest (by value) but not recursively; emit each after the
    // structs its members contain
    std::vector<int> state(structs.size(), 0), order;
    std::function<void(int)> visit = [&](int i) {
      if (state[size_t(i)] == 2) return;
      const StructDef& d = structs[size_t(i)];
      if (state[size_t(i)] == 1) throw CompileError(d.line, d.col, "struct '" + d.name + "' contains itself");
      state[size_t(i)] = 1;
      for (auto& m : d.members)
        if (inner_struct(m.second) >= 0) visit(inner_struct(m.second));
      state[size_t(i)] = 2;
      order.push_back(i);
    };
    for (size_t i = 0; i < structs.size(); ++i) visit(int(i));
    // room for the built-in result structs the checker adds (frexp and modf
    // of f32 and vec2..4), so references into the list stay valid
    structs.reserve(structs.size() + 8);
    cc.declare_module(0);
    Func* field = nullptr;
    for (auto& f : cc.fns)
      if (f->name == "field_function") field = f.get();
    if (!field) throw CompileError(1, 1, "missing field_function");
    for (auto& f : cc.fns) cc.check_function(*f);
    for (auto& g : cc.consts) cc.check_gconst(*g);
    std::ostringstream os;
    os << "// flops " << field->fl << " " << field->tr << " (FP32 arith, transcendental per evaluation)\n";
    os << "namespace " << ns << " {\n";
    for (int i : order) {
      const StructDef& d = structs[size_t(i)];
      const std::string cn = "s_" + d.name;
      os << "struct " << cn << " {\n";
      for (auto& m : d.members) os << "  " << cpp_name(m.second) << " m_" << m.first << ";\n";
      os << "  WG_HD " << cn << "() : ";
      for (size_t k = 0; k < d.members.size(); ++k) os << (k ? ", " : "") << "m_" << d.members[k].first << "()";
      os << " {}\n  WG_HD " << cn << "(";
      for (size_t k = 0; k < d.members.size(); ++k) os << (k ? ", " : "") << cpp_name(d.members[k].second) << " a" << k;
      os << ") : ";
      for (size_t k = 0; k < d.members.size(); ++k) os << (k ? ", " : "") << "m_" << d.members[k].first << "(a" << k << ")";
      os << " {}\n};\n";
    }
    for (auto& c : cc.const_code) os << c << "\n";
    // the state of one invocation (one ray): var<private> variables
    os << "struct Private {\n";
    for (auto& m : cc.private_code) os << m << "\n";
    os << "};\n";
    // prototypes (WGSL functions may be used before their declaration; a
    // helper may call the field function, as the shader's march loop does)
    for (auto& f : cc.fns) {
      std::string sig = f->code.substr(0, f->code.find('{'));
      os << sig << ";\n";
    }
    for (auto& f : cc.fns) os << f->code;
    os << "}  // namespace " << ns << "\n";
    tr.ok = true;
    tr.code = os.str();
    tr.flops_arith = field->fl;
    tr.flops_transc = field->tr;
    tr.has_private = !cc.private_code.empty();
  } catch (const CompileError& e) {
    std::ostringstream os;
    os << "error: " << e.what() << "\n";
    if (e.line >= body_first_line && e.line < body_first_line + count_lines(field_body) + 1) {
      os << "  --> field function body, line " << (e.line - body_first_line + 1) << ", column " << e.col << "\n";
    } else if (e.line <= count_lines(helpers_src) + 1) {
      os << "  --> helper source, line " << e.line << ", column " << e.col << "\n";
    } else {
      os << "  --> field function, line " << e.line << ", column " << e.col << "\n";
    }
    // echo the offending line
    std::istringstream ls(module);
    std::string l;
    for (int i = 1; std::getline(ls, l); ++i) {
      if (i == e.line) {
        os << "   | " << l << "\n   | " << std::string(size_t(std::max(0, e.col - 1)), ' ') << "^\n";
        break;
      }
    }
    tr.ok = false;
    tr.log = os.str();
  } catch (const std::exception& e) {
    tr.ok = false;
    tr.log = std::string("error: internal front-end failure: ") + e.what() + "\n";
  }
  return tr;
}

}  // namespace wgslfe
}  // namespace linon
