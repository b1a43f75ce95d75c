"""WGSL front end: lowering, diagnostics, FLOP counts, NVRTC compile (CPU only).

The generated CUDA C is also compiled for the host with g++ (device/wgsl_rt.cuh
is host/device code) and evaluated against the oracle's hand-written field
functions: without FMA contraction both are the same IEEE operations in the
same order, so every predefined field must agree bit for bit.
"""
import ctypes as C
import re
import subprocess
import tempfile
from pathlib import Path

import numpy as np
import pytest

from linon_gb300 import _abi, translate_wgsl, validate_field
from linon_gb300.engine import predefined_source

ROOT = Path(__file__).resolve().parents[1]
RT = ROOT / "linon_gb300" / "csrc" / "device" / "wgsl_rt.cuh"
EVAL_IDS = [i for i in range(1, _abi.FIELD_COUNT)]


def _inputs(n=512, seed=0):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1.5, 1.5, size=(n, 13)).astype(np.float32)
    # unit-ish velocities like the march passes
    for a in (6, 9):
        x[:, a:a + 3] /= np.linalg.norm(x[:, a:a + 3], axis=1, keepdims=True)
    x[:, 12] = rng.uniform(0, 5, size=n)
    return x


@pytest.fixture(scope="module")
def host_fields(lib):
    """All predefined fields lowered by the front end and compiled with g++."""
    parts = [f'#include "{RT}"', "#include <cstdint>"]
    for fid in EVAL_IDS:
        code = translate_wgsl(predefined_source(fid)).replace("namespace linon_user", f"namespace f{fid}")
        parts.append(code)
    parts.append('extern "C" int eval_field(int id, const float* in, long n, float* out) {')
    parts.append("  for (long i = 0; i < n; ++i) { const float* q = in + 13 * i; wgsl::vec3f r;")
    parts.append("    wgsl::vec3f pp(q[0],q[1],q[2]), p(q[3],q[4],q[5]), v0(q[6],q[7],q[8]), v(q[9],q[10],q[11]);")
    parts.append("    switch (id) {")
    for fid in EVAL_IDS:
        parts.append(f"      case {fid}: r = f{fid}::field_function(pp, p, v0, v, q[12]); break;")
    parts.append("      default: return 1; }")
    parts.append("    out[3*i] = r.x; out[3*i+1] = r.y; out[3*i+2] = r.z; }")
    parts.append("  return 0; }")
    d = Path(tempfile.mkdtemp(prefix="linon_fe_"))
    src = d / "fields.cpp"
    src.write_text("\n".join(parts))
    so = d / "fields.so"
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-shared", "-fPIC", "-o", str(so),
                        str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-4000:]
    h = C.CDLL(str(so))
    h.eval_field.argtypes = [C.c_int, C.c_void_p, C.c_long, C.c_void_p]
    return h


@pytest.mark.parametrize("fid", EVAL_IDS)
def test_lowered_field_matches_oracle_bit_exact(host_fields, oracle, fid):
    x = _inputs()
    out = np.zeros((len(x), 3), np.float32)
    assert host_fields.eval_field(fid, x.ctypes.data, len(x), out.ctypes.data) == 0
    ref = oracle.field_eval(fid, x)
    np.testing.assert_array_equal(out.view(np.uint32), ref.view(np.uint32))


def test_custom_empty_body_is_an_error():
    with pytest.raises(_abi.LinonCompileError) as e:
        translate_wgsl(predefined_source(0))
    assert "must return a value" in e.value.message


@pytest.mark.parametrize("body,needle", [
    ("return q;", "no definition in scope for identifier: 'q'"),
    ("return p + 1.0;", None),  # vec3 + scalar is fine in WGSL
    ("return p.w;", "out of range"),
    ("return p.xq;", "invalid swizzle"),
    ("let a = 1.0; a = 2.0; return p;", "cannot assign to an immutable"),
    ("return rotateY(p);", "expects 2 arguments"),
    ("return vec3<f32>(1.0, 2.0);", "wrong number of components"),
    ("return 1.0;", "return type mismatch"),
    ("if (p.x) { return p; } return v;", "condition must be bool"),
    ("return foo(p);", "unknown function"),
    ("let x: i32 = 1.5; return p;", "cannot initialize"),
    ("return p", "expected ';'"),
])
def test_diagnostics(body, needle):
    if needle is None:
        translate_wgsl(body)
        return
    with pytest.raises(_abi.LinonCompileError) as e:
        translate_wgsl(body)
    assert needle in e.value.message, e.value.message
    assert "--> field function" in e.value.message


def test_var_compound_int_float_rejected():
    # AbstractFloat 1.5 cannot convert to i32
    with pytest.raises(_abi.LinonCompileError):
        translate_wgsl("var x = 1; x += 1.5; return p;")


def test_helpers_and_control_flow():
    helpers = """
const K: f32 = 2.0;
const HALF = 0.5;
fn bend(v: vec3<f32>, a: f32) -> vec3<f32> {
    var r = v;
    for (var i: i32 = 0; i < 3; i++) {
        if (i == 1) { continue; }
        r = r + a * HALF * vec3<f32>(0.0, 1.0, 0.0);
    }
    var j = 0;
    loop {
        j += 1;
        if (j > 2) { break; }
    }
    while (j < 5) { j = j + 1; }
    return select(r, -r, j > 10) * K;
}
"""
    code = translate_wgsl("let m = mat3x3<f32>(1.0, 0.0, 0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 1.0);\n"
                          "let q = m * bend(v, t).zyx;\nreturn q;", helpers)
    assert "u_bend" in code and "field_function" in code


def test_dot_plus_scalar_lowering():
    """dot(a, b) + s in f32, in either order, is emitted as dot_add (fast
    modules fold s into the first FMA; precise modules add as written);
    integer dots, vector sums and user functions named like builtins are
    left alone."""
    code = translate_wgsl("let a = dot(p, p) + 0.01;\nlet b = 2.0 + dot(v, p);\n"
                          "let c = dot(vec2<i32>(1, 2), vec2<i32>(3, 4)) + 1;\n"
                          "return vec3<f32>(a, b, f32(c)) + dot(p, v);")
    assert code.count("::wgsl::dot_add(") == 2
    assert "dot_add(u_p, u_p, 0x1.47ae14p-7f)" in code
    assert "dot_add(u_v, u_p, 2.0f)" in code or "dot_add(u_v, u_p, 0x1p+1f)" in code
    code = translate_wgsl("return vec3<f32>(mydot(p, p) + 1.0);",
                          "fn mydot(a: vec3<f32>, b: vec3<f32>) -> f32 { return a.x * b.x; }")
    assert "dot_add" not in code


def test_shadowing_and_abstract_constants():
    code = translate_wgsl("let x = 8.0 / 3.0;\n{ let x = x * 2.0; }\nreturn vec3<f32>(x);")
    # 8/3 folded in double then rounded once to f32
    assert "0x1.555556p+1f" in code


def test_flop_counts_match_oracle(oracle, lib):
    """Front-end static FP32 op counts == the oracle's CountingFloat counts for
    the branch-free fields."""
    x = _inputs(1)[0]
    for name in ("linear", "twist", "lens", "lorenz", "lorenz_scaled", "roessler", "translation_x", "rotation"):
        fid = _abi.FIELD_IDS[name]
        counts = oracle.count_field(fid, x)  # add, mul, div, sqrt, cmp, transc
        arith = int(counts[0] + counts[1] + counts[2] + counts[3])
        got = _fe_counts(predefined_source(fid))
        assert got == (arith, int(counts[5])), (name, got, arith, counts)


def _fe_counts(body):
    """FLOP counts of the front end, read from the annotated translation."""
    lib = _abi.load()
    out = C.create_string_buffer(1 << 16)
    log = C.create_string_buffer(1 << 12)
    assert lib.linon_wgsl_translate(body.encode(), None, out, len(out), log, len(log)) == 0
    text = out.value.decode()
    line = [l for l in text.splitlines() if l.startswith("// flops")][0]
    a, t = line.split()[2:4]
    return int(a), int(t)


@pytest.mark.parametrize("fid", [_abi.FIELD_IDS[n] for n in ("twist", "mirage_spherical_sigmoid", "lens")])
@pytest.mark.parametrize("precise", [False, True])
def test_nvrtc_compiles_for_sm103a(fid, precise):
    report = validate_field(predefined_source(fid), precise=precise)
    assert "linon_march_v14" in report and "linon_march_v1" in report
    assert "sm_103a" in report


@pytest.mark.parametrize("name,precise", [("lens", False), ("twist", True)])
def test_nvrtc_compiles_batched_kernels(name, precise):
    """LINON_VALIDATE_BATCHED: the batched module (persistent queue and one
    CTA per tile, each with its three step modes) compiles with the field."""
    report = validate_field(predefined_source(_abi.FIELD_IDS[name]), precise=precise, batched=True)
    for k in ("linon_multi_fk", "linon_multi_f", "linon_multi", "linon_batch_fk", "linon_batch_f", "linon_batch"):
        assert re.search(rf"Function properties for {k}\b", report), k


def test_validate_rejects_front_end_errors():
    validate_field("return v;")
    with pytest.raises(_abi.LinonCompileError):
        validate_field("return undefined_thing;")


def _host_eval(body, x, helpers=None):
    """Lowers one field body, compiles it for the host with g++ and
    evaluates it on inputs [n, 13] (p_prev, p, v0, v, t)."""
    code = translate_wgsl(body, helpers)
    src = "\n".join([f'#include "{RT}"', code,
                     'extern "C" void eval(const float* in, long n, float* out) {',
                     "  for (long i = 0; i < n; ++i) { const float* q = in + 13 * i;",
                     "    wgsl::vec3f pp(q[0],q[1],q[2]), p(q[3],q[4],q[5]), v0(q[6],q[7],q[8]), v(q[9],q[10],q[11]);",
                     "    wgsl::vec3f r = linon_user::field_function(pp, p, v0, v, q[12]);",
                     "    out[3*i] = r.x; out[3*i+1] = r.y; out[3*i+2] = r.z; } }"])
    d = Path(tempfile.mkdtemp(prefix="linon_fe1_"))
    (d / "f.cpp").write_text(src)
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-shared", "-fPIC", "-o", str(d / "f.so"),
                        str(d / "f.cpp")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    h = C.CDLL(str(d / "f.so"))
    h.eval.argtypes = [C.c_void_p, C.c_long, C.c_void_p]
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros((len(x), 3), np.float32)
    h.eval(x.ctypes.data, len(x), out.ctypes.data)
    return out


SWITCH_BODY = """
var r = vec3<f32>(0.0);
switch (i32(t)) {
  case 0, 1: { r = p; }
  case 2 { r = -v; }
  case 3: {
    if (p.x > 0.0) { r = vec3<f32>(9.0); break; }
    r = vec3<f32>(8.0);
  }
  case -3, default: { r = v0; }
}
var acc = 0.0;
for (var i = 0; i < 4; i++) {
  switch (u32(i)) {
    case 1u: { continue; }
    case 3u: { break; }
    default: { acc += 1.0; }
  }
  acc += 10.0;
}
return r + vec3<f32>(acc);
"""


def test_switch_semantics():
    """case lists, default merged with a case, break leaving the switch,
    continue inside a switch inside a loop."""
    ts = np.array([0, 1, 2, 3, 3, -3, 7, -1], np.float32)
    x = np.zeros((len(ts), 13), np.float32)
    x[:, 3:6] = [1, 2, 3]
    x[4, 3] = -1.0  # p.x < 0 for the second t = 3 sample
    x[:, 6:9] = [4, 5, 6]
    x[:, 9:12] = [7, 8, 9]
    x[:, 12] = ts
    out = _host_eval(SWITCH_BODY, x)
    acc = 32.0  # i = 0: 1 + 10; i = 1: continue; i = 2: 1 + 10; i = 3: break (switch) + 10
    want = []
    for row, t in zip(x, ts):
        ti = int(t)
        if ti in (0, 1):
            r = row[3:6]
        elif ti == 2:
            r = -row[9:12]
        elif ti == 3:
            r = np.full(3, 9.0 if row[3] > 0 else 8.0)
        else:
            r = row[6:9]
        want.append(np.asarray(r, np.float32) + np.float32(acc))
    np.testing.assert_array_equal(out, np.array(want, np.float32))


@pytest.mark.parametrize("body,needle", [
    ("switch (1) { case 1: { } } return p;", "must have a default clause"),
    ("switch (1) { default: { } case 2, default: { } } return p;", "more than one default"),
    ("switch (1) { case 1, 2: { } case 2: { } default: { } } return p;", "duplicate case selector 2"),
    ("switch (t) { default: { } } return p;", "selector must be i32 or u32"),
    ("let k = i32(t); switch (1) { case k: { } default: { } } return p;", "constant expression"),
    ("switch (1i) { case 1u: { } default: { } } return p;", "does not match"),
    ("switch (1) { case 1: { continue; } default: { } } return p;", "'continue' outside of a loop"),
    ("switch (1) { case 1 return p; default: { } } return p;", "expected '{'"),
])
def test_switch_diagnostics(body, needle):
    with pytest.raises(_abi.LinonCompileError) as e:
        translate_wgsl(body)
    assert needle in e.value.message, e.value.message


def test_switch_break_without_loop_and_all_paths_return():
    # break is valid in a switch outside any loop; a switch whose every
    # clause returns ends the function
    translate_wgsl("switch (2) { case 1: { break; } default: { } } return p;")
    translate_wgsl("switch (i32(t)) { case 0: { return p; } default: { return v; } }")


def test_bitcast_and_nested_templates():
    """bitcast<T>: bit patterns reinterpreted (scalar and vector); nested
    template lists close with '>>' and '>='."""
    body = """
let b = bitcast<u32>(p.x);
let flipped = bitcast<f32>(b ^ 0x80000000u);
let one: vec2<f32>= bitcast<vec2<f32>>(vec2<i32>(1065353216, 1073741824));
let hi = f32(b >> 20u);
return vec3<f32>(hi, flipped, one.x + one.y);
"""
    x = np.zeros((4, 13), np.float32)
    x[:, 3] = [1.0, -2.5, 3.0e-3, 1.0e20]
    out = _host_eval(body, x)
    bits = x[:, 3].view(np.uint32)
    np.testing.assert_array_equal(out[:, 0], (bits >> 20).astype(np.float32))
    np.testing.assert_array_equal(out[:, 1], -x[:, 3])
    np.testing.assert_array_equal(out[:, 2], np.full(4, 3.0, np.float32))
    assert "linon_march_v1" in validate_field(body)


@pytest.mark.parametrize("body,needle", [
    ("return vec3<f32>(bitcast<f32>(vec2<u32>(1u, 2u)).x);", "different sizes"),
    ("let b = bitcast<bool>(1); return p;", "bitcast target must be"),
    ("let b = bitcast(1.0); return p;", "needs a target type"),
    ("let b = bitcast<u32>(true); return p;", "bitcast argument must be"),
])
def test_bitcast_diagnostics(body, needle):
    with pytest.raises(_abi.LinonCompileError) as e:
        translate_wgsl(body)
    assert needle in e.value.message, e.value.message


ARRAY_HELPERS = """
fn pick(a: array<vec3<f32>, 3>, i: i32) -> vec3<f32> { return a[i]; }
fn total(a: array<f32, 4>) -> f32 {
  var s = 0.0;
  for (var i = 0u; i < 4u; i++) { s += a[i]; }
  return s;
}
"""
ARRAY_BODY = """
var w = array<f32, 4>(1.0, 2.0, 3.0, 4.0);
let dirs = array(vec3<f32>(1.0, 0.0, 0.0), vec3<f32>(0.0, 1.0, 0.0), vec3<f32>(0.0, 0.0, 1.0));
var z: array<vec3<f32>, 2>;
let k = i32(t);
w[1] = w[1] * 2.0;
z[1u] = pick(dirs, k) * w[k];
let copy = w;
w[0] = 100.0;
return z[1] + vec3<f32>(total(copy), z[0].x, w[0]);
"""


def test_arrays_semantics():
    """array<T, N>: constructors (explicit and inferred), zero value, element
    assignment, value copies, by-value parameters, u32 and runtime indices
    (clamped to the array, as wgpu's default bounds-check policy does)."""
    ts = np.array([0, 1, 2, 3, 7, -5], np.float32)
    x = np.zeros((len(ts), 13), np.float32)
    x[:, 12] = ts
    out = _host_eval(ARRAY_BODY, x, ARRAY_HELPERS)
    w = np.array([1, 4, 3, 4], np.float32)  # after w[1] *= 2
    dirs = np.eye(3, dtype=np.float32)
    want = []
    for t in ts:
        k = int(t)
        z1 = dirs[min(max(k, 0), 2)] * w[min(max(k, 0), 3)]
        want.append(z1 + np.array([w.sum(), 0.0, 100.0], np.float32))
    np.testing.assert_array_equal(out, np.array(want, np.float32))
    assert "linon_march_v1" in validate_field(ARRAY_BODY, ARRAY_HELPERS)


@pytest.mark.parametrize("body,needle", [
    ("var a = array<f32, 2>(1.0, 2.0, 3.0); return p;", "needs 2 elements"),
    ("let a = array(1.0, vec2<f32>(1.0)); return p;", "different types"),
    ("let a = array<f32, 3>(1.0, 2.0, 3.0); return vec3<f32>(a[3]);", "index out of bounds"),
    ("var a: array<f32>; return p;", "runtime-sized arrays"),
    ("var a: array<array<f32, 2>, 2>; return p;", "arrays of arrays"),
    ("let n = 3; var a: array<f32, n>; return p;", "integer literal"),
    ("let a = array<f32, 2>(); let b = a + a; return p;", "cannot be applied to arrays"),
    ("let a = array<f32, 2>(); return vec3<f32>(abs(a)[0]);", "does not take an array"),
    ("let a = array<f32, 2>(); let b = -a; return p;", "cannot be applied to an array"),
    ("let a = array(); return p;", "empty array constructor"),
    ("let a = array<f32, 2>(1.0, 2.0); return vec3<f32>(a.x);", None),
])
def test_array_diagnostics(body, needle):
    with pytest.raises(_abi.LinonCompileError) as e:
        translate_wgsl(body)
    if needle:
        assert needle in e.value.message, e.value.message


STRUCT_HELPERS = """
struct Ray { o: vec3<f32>, d: vec3<f32>, w: array<f32, 2>, }
struct Pair {
  a: Ray,
  k: i32
}
fn advance(r: Ray, s: f32) -> Ray {
  var q = r;
  q.o = q.o + s * q.d;
  q.w[1] = s;
  return q;
}
fn rays() -> array<Ray, 2> {
  return array<Ray, 2>(Ray(vec3<f32>(1.0), vec3<f32>(0.0), array(0.0, 0.0)), Ray());
}
"""
STRUCT_BODY = """
var pr = Pair(Ray(p, v, array(1.0, 2.0)), 3);
let z = Pair();
let copy = pr;
pr.a = advance(pr.a, t);
pr.a.d.y = 5.0;
let rs = rays();
return pr.a.o + pr.a.d + vec3<f32>(pr.a.w[1] + copy.a.w[1], f32(pr.k) + rs[0].o.x + rs[1].o.y, f32(z.k) + z.a.o.x);
"""


def test_structs_semantics():
    """Module-scope structs: nested structs, array members, arrays of
    structs, constructors and zero values, member assignment, value copies,
    struct parameters and results."""
    rng = np.random.default_rng(3)
    x = rng.uniform(-2, 2, (16, 13)).astype(np.float32)
    out = _host_eval(STRUCT_BODY, x, STRUCT_HELPERS)
    p, v, t = x[:, 3:6], x[:, 9:12], x[:, 12:13]
    o = p + t * v
    d = v.copy()
    d[:, 1] = 5.0
    want = o + d + np.stack([t[:, 0] + 2.0, np.full(16, 3.0 + 1.0 + 0.0), np.zeros(16)], -1).astype(np.float32)
    np.testing.assert_allclose(out, want, rtol=0, atol=2e-6)
    assert "linon_march_v1" in validate_field(STRUCT_BODY, STRUCT_HELPERS)


@pytest.mark.parametrize("helpers,body,needle", [
    ("struct S { a: f32 }", "let s = S(); return vec3<f32>(s.b);", "has no member 'b'"),
    ("struct S { a: f32, b: f32 }", "let s = S(1.0); return p;", "needs 2 arguments"),
    ("struct S { a: f32 }", "let s = S(vec2<f32>(1.0)); return p;", "cannot convert"),
    ("struct S { a: f32, a: f32 }", "return p;", "duplicate member"),
    ("struct S { a: S }", "return p;", "cannot contain itself"),
    ("struct A { b: B }\nstruct B { a: A }", "return p;", "contains itself"),
    ("struct S { a: f32 }\nstruct S { b: f32 }", "return p;", "redefinition of struct"),
    ("struct S { }", "return p;", "at least one member"),
    ("struct S { a: f32 }", "let s = S(); let u = s + s; return p;", "cannot be applied to structs"),
    ("struct S { a: f32 }", "let s = S(); let u = length(s); return p;", "does not take a struct"),
    ("struct S { a: f32 }", "let s = S(); s.a = 1.0; return p;", "cannot assign to an immutable"),
])
def test_struct_diagnostics(helpers, body, needle):
    with pytest.raises(_abi.LinonCompileError) as e:
        translate_wgsl(body, helpers)
    assert needle in e.value.message, e.value.message


ALIAS_OVERRIDE_HELPERS = """
alias Vec = vec3<f32>;
alias Bend = Ray;               // used before the struct it names
alias Coeffs = array<Scalar, 3>;
alias Scalar = f32;             // used (by Coeffs) before its own declaration
struct Ray { o: Vec, d: Vec }
@id(0) override strength: f32 = 0.5;
override steps = 3;             // concrete i32 from an abstract int
override twice_strength = strength * 2.0;
fn bend(r: Bend, k: Coeffs) -> Vec {
    var acc: Vec = r.o;
    for (var i = 0; i < steps; i++) { acc = acc + k[i] * r.d; }
    return acc;
}
"""

ALIAS_OVERRIDE_BODY = """
let c = Coeffs(strength, twice_strength, 1.0);
return bend(Bend(p, v), c);
"""


def test_alias_and_override_semantics():
    """`alias` names a type (also before its declaration, also a struct);
    `override` is a pipeline constant whose default value is used (the
    engine sets no pipeline constants): a concrete scalar, from an abstract
    initialiser too."""
    rng = np.random.default_rng(4)
    x = rng.uniform(-2, 2, (12, 13)).astype(np.float32)
    out = _host_eval(ALIAS_OVERRIDE_BODY, x, ALIAS_OVERRIDE_HELPERS)
    p, v = x[:, 3:6], x[:, 9:12]
    acc = p.copy()
    for k in (np.float32(0.5), np.float32(1.0), np.float32(1.0)):
        acc = (acc + k * v).astype(np.float32)
    np.testing.assert_array_equal(out, acc)
    assert "linon_march_v1" in validate_field(ALIAS_OVERRIDE_BODY, ALIAS_OVERRIDE_HELPERS)


@pytest.mark.parametrize("helpers,needle", [
    ("alias A = B;\nalias B = A;\nfn f(x: A) -> f32 { return 1.0; }", "cyclic type alias"),
    ("alias vec3f = vec3<f32>;", "redefinition of type"),
    ("struct S { a: f32 }\nalias S = f32;", "redefinition of type"),
    ("alias A = f32;\nalias A = i32;", "redefinition of type"),
    ("alias A = Nope;\nfn f(x: A) -> f32 { return 1.0; }", "unknown type 'Nope'"),
    ("override k: f32;", "needs a default value"),
    ("override k = vec3<f32>(1.0);", "must have a scalar type"),
    ("override k: i32 = 1.5;", "cannot initialize"),
])
def test_alias_override_diagnostics(helpers, needle):
    with pytest.raises(_abi.LinonCompileError) as e:
        translate_wgsl("return p;", helpers)
    assert needle in e.value.message, e.value.message


def test_alias_constructors_of_every_kind():
    """An alias of a vector, matrix or scalar type constructs (and converts)
    like the type it names."""
    helpers = "alias V2 = vec2<f32>;\nalias M = mat2x3<f32>;\nalias S = f32;\nalias I = i32;"
    body = """
let m = M(V2(1.0, 2.0).xyx, vec3<f32>(p.x, p.y, p.z));
let s = S(I(2.75));
return m * V2(t, s) + vec3<f32>(S(3));
"""
    rng = np.random.default_rng(8)
    x = rng.uniform(-2, 2, (6, 13)).astype(np.float32)
    out = _host_eval(body, x, helpers)
    p, t = x[:, 3:6], x[:, 12]
    c0 = np.array([1.0, 2.0, 1.0], np.float32)
    want = (c0[None, :] * t[:, None] + p * np.float32(2.0) + np.float32(3.0)).astype(np.float32)
    np.testing.assert_allclose(out, want, rtol=0, atol=1e-6)
