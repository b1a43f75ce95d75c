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
# host builds of lowered fields go to the tests' scratch folder inside the
# repository (tests/conftest.py empties it at the start and end of a run)
SCRATCH = ROOT / "_build" / "tests"


def scratch_dir(prefix: str) -> Path:
    SCRATCH.mkdir(parents=True, exist_ok=True)
    return Path(tempfile.mkdtemp(prefix=prefix, dir=SCRATCH))


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
        parts.append(f"      case {fid}: {{ f{fid}::Private pv; r = f{fid}::field_function(pv, pp, p, v0, v, q[12]); }} break;")
    parts.append("      default: return 1; }")
    parts.append("    out[3*i] = r.x; out[3*i+1] = r.y; out[3*i+2] = r.z; }")
    parts.append("  return 0; }")
    d = scratch_dir("linon_fe_")
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


def _host_eval(body, x, helpers=None, calls=1):
    """Lowers one field body, compiles it for the host with g++ and
    evaluates it on inputs [n, 13] (p_prev, p, v0, v, t): one invocation per
    input (fresh var<private> state), the field called `calls` times in it,
    the last result returned."""
    code = translate_wgsl(body, helpers)
    src = "\n".join([f'#include "{RT}"', code,
                     'extern "C" void eval(const float* in, long n, float* out, int calls) {',
                     "  for (long i = 0; i < n; ++i) { const float* q = in + 13 * i;",
                     "    wgsl::vec3f pp(q[0],q[1],q[2]), p(q[3],q[4],q[5]), v0(q[6],q[7],q[8]), v(q[9],q[10],q[11]);",
                     "    linon_user::Private pv; wgsl::vec3f r;",
                     "    for (int c = 0; c < calls; ++c) r = linon_user::field_function(pv, pp, p, v0, v, q[12]);",
                     "    out[3*i] = r.x; out[3*i+1] = r.y; out[3*i+2] = r.z; } }"])
    d = scratch_dir("linon_fe1_")
    (d / "f.cpp").write_text(src)
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-shared", "-fPIC", "-o", str(d / "f.so"),
                        str(d / "f.cpp")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    h = C.CDLL(str(d / "f.so"))
    h.eval.argtypes = [C.c_void_p, C.c_long, C.c_void_p, C.c_int]
    x = np.ascontiguousarray(x, np.float32)
    out = np.zeros((len(x), 3), np.float32)
    h.eval(x.ctypes.data, len(x), out.ctypes.data, int(calls))
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


# ---- bit, float-decomposition and packing builtins (WGSL 17.5 / 17.9 / 17.10) ----
M32 = 0xFFFFFFFF


def _s32(u):
    u &= M32
    return u - (1 << 32) if u & 0x80000000 else u


def _clz(u):
    return 32 - (u & M32).bit_length()


def _ctz(u):
    u &= M32
    return 32 if u == 0 else (u & -u).bit_length() - 1


def _rev(u):
    return int(f"{u & M32:032b}"[::-1], 2)


def _flb_i(i):
    v = ~i if i < 0 else i
    return -1 if v == 0 else v.bit_length() - 1


def _ext_u(e, off, cnt):
    o = min(off, 32)
    c = min(cnt, 32 - o)
    return 0 if c == 0 else (e >> o) & ((1 << c) - 1)


def _ext_i(e, off, cnt):
    o = min(off, 32)
    c = min(cnt, 32 - o)
    if c == 0:
        return 0
    v = (e & M32) >> o & ((1 << c) - 1)
    return v - (1 << c) if v >> (c - 1) else v


def _ins(e, nb, off, cnt):
    o = min(off, 32)
    c = min(cnt, 32 - o)
    if c == 0:
        return e & M32
    mask = ((1 << c) - 1) << o
    return ((e & ~mask) | ((nb << o) & mask)) & M32


def _bits_inputs(n=3000):
    rng = np.random.default_rng(21)
    x = np.zeros((n, 13), np.float32)
    raw = rng.integers(0, 2 ** 32, (n, 3), dtype=np.uint64).astype(np.uint32)
    raw[:40] = [[0, 0, 0], [M32, M32, M32], [1, 2, 3], [0x80000000, 0x7FFFFFFF, 0x00010000]] * 10
    raw[40:80, 2] = rng.integers(0, 70, 40)  # small offsets / counts, including > 32
    x[:, 3:6] = raw.view(np.float32)
    x[:, 12] = rng.integers(0, 40, n).astype(np.float32)
    return x, raw


def test_integer_bit_builtins():
    x, raw = _bits_inputs()
    body = """
let u = bitcast<u32>(p.x);
let i = bitcast<i32>(p.y);
let w = bitcast<u32>(p.z);
let o = u32(t);
let c = w % 40u;
let a = countLeadingZeros(u) | (countOneBits(u) << 8u) | (countTrailingZeros(u) << 16u)
      | (u32(countOneBits(i)) << 24u);
return bitcast<vec3<f32>>(vec3<u32>(a, reverseBits(u), bitcast<u32>(firstLeadingBit(i))));
"""
    out = _host_eval(body, x).view(np.uint32)
    for k in range(len(x)):
        u, i = int(raw[k, 0]), _s32(int(raw[k, 1]))
        a = _clz(u) | (bin(u).count("1") << 8) | (_ctz(u) << 16) | (bin(i & M32).count("1") << 24)
        assert list(out[k]) == [a, _rev(u), _flb_i(i) & M32], k
    body2 = """
let u = bitcast<u32>(p.x);
let i = bitcast<i32>(p.y);
let w = bitcast<u32>(p.z);
let o = u32(t);
let c = w % 40u;
return bitcast<vec3<f32>>(vec3<u32>(firstTrailingBit(u) ^ (firstLeadingBit(u) << 7u),
                                    extractBits(u, o, c) ^ bitcast<u32>(extractBits(i, o, c)),
                                    insertBits(u, w, o, c) ^ bitcast<u32>(insertBits(i, bitcast<i32>(w), c, o))));
"""
    out = _host_eval(body2, x).view(np.uint32)
    for k in range(len(x)):
        u, i, w = int(raw[k, 0]), _s32(int(raw[k, 1])), int(raw[k, 2])
        o, c = int(x[k, 12]), w % 40
        ftb = M32 if u == 0 else _ctz(u)
        flb = M32 if u == 0 else u.bit_length() - 1
        e0 = (ftb ^ (flb << 7)) & M32
        e1 = (_ext_u(u, o, c) ^ (_ext_i(i, o, c) & M32)) & M32
        e2 = _ins(u, w, o, c) ^ _ins(i & M32, w, c, o)
        assert list(out[k]) == [e0, e1, e2], k
    # vectors, component-wise
    vb = "let u = bitcast<vec3<u32>>(p);\nreturn bitcast<vec3<f32>>(countOneBits(u) + reverseBits(u));"
    out = _host_eval(vb, x).view(np.uint32)
    want = [[(bin(int(q)).count("1") + _rev(int(q))) & M32 for q in r] for r in raw]
    np.testing.assert_array_equal(out, np.array(want, np.uint32))


def test_float_decomposition_builtins():
    rng = np.random.default_rng(22)
    n = 4000
    x = np.zeros((n, 13), np.float32)
    vals = np.concatenate([rng.uniform(-1e6, 1e6, n // 2), rng.standard_normal(n // 4) * 1e-3,
                           rng.uniform(-70000, 70000, n - n // 2 - n // 4)]).astype(np.float32)
    vals[:6] = [0.0, -0.0, 1.0, -2.5, 65519.0, 65520.0]
    x[:, 3] = vals
    x[:, 4] = rng.uniform(-3, 3, n).astype(np.float32)
    x[:, 12] = rng.integers(-30, 30, n).astype(np.float32)
    body = """
let f = frexp(p.x);
let m = modf(p.x);
return vec3<f32>(f.fract + f32(f.exp) * 2.0, m.fract + m.whole * 0.5, ldexp(p.y, i32(t)));
"""
    out = _host_eval(body, x)
    fr, ex = np.frexp(vals)
    mf, mw = np.modf(vals)
    want = np.stack([fr.astype(np.float32) + ex.astype(np.float32) * np.float32(2.0),
                     mf.astype(np.float32) + mw.astype(np.float32) * np.float32(0.5),
                     np.ldexp(x[:, 4], x[:, 12].astype(np.int32)).astype(np.float32)], -1)
    np.testing.assert_array_equal(out, want)
    q = _host_eval("let f = frexp(vec3<f32>(p.x, p.y, 0.0));\n"
                   "return quantizeToF16(vec3<f32>(p.x, p.y, f32(f.exp.y)));", x)
    with np.errstate(over="ignore"):
        np.testing.assert_array_equal(q[:, :2], x[:, 3:5].astype(np.float16).astype(np.float32))
    np.testing.assert_array_equal(q[:, 2], np.frexp(x[:, 4])[1].astype(np.float16).astype(np.float32))


def test_packing_builtins():
    rng = np.random.default_rng(23)
    n = 3000
    x = np.zeros((n, 13), np.float32)
    x[:, 3:6] = rng.uniform(-1.5, 1.5, (n, 3)).astype(np.float32)
    x[:, 12] = rng.uniform(-1.5, 1.5, n).astype(np.float32)
    x[:10, 3:6] = [[1, -1, 0.5], [0.00196, -0.00196, 0.0039], [2, -2, 0]] * 3 + [[1e-8, -1e-8, 65504]]
    body = """
let e = vec4<f32>(p, t);
return bitcast<vec3<f32>>(vec3<u32>(pack4x8snorm(e), pack4x8unorm(e), pack2x16float(p.xy)));
"""
    out = _host_eval(body, x).view(np.uint32)
    e4 = np.concatenate([x[:, 3:6], x[:, 12:13]], 1)

    def pk(vals, s, lo, bits):
        c = np.minimum(np.float32(1), np.maximum(np.float32(lo), vals))
        q = np.floor(np.float32(0.5) + np.float32(s) * c).astype(np.int64) & ((1 << bits) - 1)
        return sum(q[:, j] << (bits * j) for j in range(vals.shape[1]))
    h = x[:, 3:5].astype(np.float16).view(np.uint16).astype(np.int64)
    want = np.stack([pk(e4, 127, -1, 8), pk(e4, 255, 0, 8), h[:, 0] | (h[:, 1] << 16)], -1).astype(np.uint32)
    np.testing.assert_array_equal(out, want)
    body = """
let s = pack2x16snorm(p.xy);
let u = pack2x16unorm(p.yz);
return vec3<f32>(dot(unpack2x16snorm(s), vec2<f32>(1.0, 1000.0)), dot(unpack2x16unorm(u), vec2<f32>(1.0, 1000.0)),
                 unpack4x8snorm(pack4x8snorm(vec4<f32>(p, t))).w + 10.0 * unpack4x8unorm(pack4x8unorm(vec4<f32>(p, t))).x);
"""
    out = _host_eval(body, x)
    s16 = pk(x[:, 3:5], 32767, -1, 16)
    u16 = pk(x[:, 4:6], 65535, 0, 16)

    def sx(v, b):
        v = v & ((1 << b) - 1)
        return np.where(v >= 1 << (b - 1), v - (1 << b), v)
    us0 = np.maximum(sx(s16, 16).astype(np.float32) / np.float32(32767), np.float32(-1))
    us1 = np.maximum(sx(s16 >> 16, 16).astype(np.float32) / np.float32(32767), np.float32(-1))
    uu0 = (u16 & 0xFFFF).astype(np.float32) / np.float32(65535)
    uu1 = (u16 >> 16).astype(np.float32) / np.float32(65535)
    p8s = pk(e4, 127, -1, 8)
    p8u = pk(e4, 255, 0, 8)
    w3 = np.maximum(sx(p8s >> 24, 8).astype(np.float32) / np.float32(127), np.float32(-1))
    x0 = (p8u & 0xFF).astype(np.float32) / np.float32(255)
    want = np.stack([us0 + us1 * np.float32(1000), uu0 + uu1 * np.float32(1000), w3 + np.float32(10) * x0], -1)
    np.testing.assert_array_equal(out, want.astype(np.float32))
    # unpack2x16float round trip, 8-bit integer packing and packed dot products
    body = """
let a = bitcast<u32>(p.x);
let b = bitcast<u32>(p.y);
let vi = vec4<i32>(i32(t * 200.0), -3, 130, -200);
let vu = vec4<u32>(u32(abs(t) * 200.0), 3u, 300u, 255u);
let r = unpack4xI8(pack4xI8(vi)) + unpack4xI8(pack4xI8Clamp(vi)) * 1000;
let q = unpack4xU8(pack4xU8(vu)) + unpack4xU8(pack4xU8Clamp(vu)) * 1000u;
return bitcast<vec3<f32>>(vec3<u32>(dot4U8Packed(a, b), bitcast<u32>(dot4I8Packed(a, b)),
                                    bitcast<u32>(r.x + r.y + r.z * 7 + r.w * 13) ^ (q.x + q.z * 7u + q.w * 13u)));
"""
    x2 = x.copy()
    x2[:, 3:5] = rng.integers(0, 2 ** 32, (n, 2), dtype=np.uint64).astype(np.uint32).view(np.float32)
    out = _host_eval(body, x2).view(np.uint32)
    A = x2[:, 3].view(np.uint32).astype(np.int64)
    B = x2[:, 4].view(np.uint32).astype(np.int64)
    du = sum(((A >> (8 * j)) & 0xFF) * ((B >> (8 * j)) & 0xFF) for j in range(4))
    di = sum(sx(A >> (8 * j), 8) * sx(B >> (8 * j), 8) for j in range(4))
    t = x2[:, 12]
    vi = [(t * np.float32(200)).astype(np.int64), np.full(n, -3), np.full(n, 130), np.full(n, -200)]
    vu = [(np.abs(t) * np.float32(200)).astype(np.int64), np.full(n, 3), np.full(n, 300), np.full(n, 255)]
    r = [sx(v, 8) + np.clip(v, -128, 127) * 1000 for v in vi]
    q = [(v & 0xFF) + np.minimum(v, 255) * 1000 for v in vu]
    e2 = ((r[0] + r[1] + r[2] * 7 + r[3] * 13) & M32) ^ ((q[0] + q[2] * 7 + q[3] * 13) & M32)
    np.testing.assert_array_equal(out, np.stack([du & M32, di & M32, e2], -1).astype(np.uint32))
    h2 = _host_eval("return vec3<f32>(unpack2x16float(pack2x16float(p.xy)), 0.0);", x)
    np.testing.assert_array_equal(h2[:, :2], x[:, 3:5].astype(np.float16).astype(np.float32))


@pytest.mark.parametrize("body,needle", [
    ("let a = countOneBits(1.5); return p;", "needs an i32 or u32"),
    ("let a = extractBits(1u, 2, 1.5); return p;", "must be u32"),
    ("let a = extractBits(1u, 2, -1); return p;", "does not fit in u32"),
    ("let a = ldexp(p, 2); return p;", "must be vec3<i32>"),
    ("let a = pack4x8snorm(p); return p;", "must be vec4<f32>"),
    ("let f = frexp(p.x); return vec3<f32>(f.whole);", "has no member 'whole'"),
    ("let __x = 1.0; return p;", "reserved"),
])
def test_builtin_diagnostics(body, needle):
    with pytest.raises(_abi.LinonCompileError) as e:
        translate_wgsl(body)
    assert needle in e.value.message, e.value.message


ALL_NEW_BUILTINS_BODY = """
let u = bitcast<u32>(p.x);
let i = bitcast<i32>(p.y);
let a = countLeadingZeros(u) + countOneBits(u) + countTrailingZeros(u) + reverseBits(u) + firstLeadingBit(u)
      + firstTrailingBit(u) + extractBits(u, 3u, 5u) + insertBits(u, 7u, 2u, 3u);
let b = countLeadingZeros(vec2<i32>(i)) + firstLeadingBit(vec2<i32>(i)) + extractBits(vec2<i32>(i), 1u, 9u);
let f = frexp(p);
let m = modf(p.x);
let e = vec4<f32>(p, t);
let k = pack4x8snorm(e) ^ pack4x8unorm(e) ^ pack2x16snorm(p.xy) ^ pack2x16unorm(p.xy) ^ pack2x16float(p.xy)
      ^ pack4xI8(vec4<i32>(b, b)) ^ pack4xU8(unpack4xU8(u)) ^ pack4xI8Clamp(unpack4xI8(u)) ^ pack4xU8Clamp(vec4<u32>(a));
let g = unpack4x8snorm(k).xyz + unpack4x8unorm(k).xyz + vec3<f32>(unpack2x16snorm(k) + unpack2x16unorm(k)
      + unpack2x16float(k), f32(dot4U8Packed(k, u)) + f32(dot4I8Packed(k, u)));
return g + ldexp(f.fract, f.exp) + quantizeToF16(vec3<f32>(m.fract, m.whole, f32(a)));
"""


@pytest.mark.parametrize("precise", [False, True])
def test_new_builtins_compile_for_sm103a(precise):
    report = validate_field(ALL_NEW_BUILTINS_BODY, precise=precise)
    assert "linon_march_v14" in report and "sm_103a" in report


def test_f16_conversions_every_value():
    """unpack2x16float decodes every binary16 bit pattern exactly, and
    pack2x16float encodes each decoded value back to its own bits (NaNs to a
    NaN)."""
    h = np.arange(65536, dtype=np.uint32)
    words = (h[0::2] | (h[1::2] << 16)).astype(np.uint32)
    x = np.zeros((len(words), 13), np.float32)
    x[:, 3] = words.view(np.float32)
    out = _host_eval("let w = bitcast<u32>(p.x);\nlet f = unpack2x16float(w);\n"
                     "return vec3<f32>(f, bitcast<f32>(pack2x16float(f)));", x)
    ref = h.astype(np.uint16).view(np.float16).astype(np.float32)
    got = np.stack([out[:, 0], out[:, 1]], 1).reshape(-1)
    nan = np.isnan(ref)
    np.testing.assert_array_equal(got[~nan].view(np.uint32), ref[~nan].view(np.uint32))
    assert np.isnan(got[nan]).all()
    back = out[:, 2].view(np.uint32)
    lo, hi = back & 0xFFFF, back >> 16
    rt = np.stack([lo, hi], 1).reshape(-1)
    ok = nan | (rt == h)
    assert ok.all()
    nh = rt[nan]
    assert (((nh & 0x7C00) == 0x7C00) & ((nh & 0x3FF) != 0)).all()


@pytest.mark.gpu
def test_new_builtins_device_equals_host(engine):
    """The device implementations of the bit, decomposition and packing
    builtins (CUDA integer intrinsics, ldexpf / frexpf / modff) give the
    host implementations' results bit for bit (precise module, through
    linon_field_eval); so do fields with pointers, arrays of arrays,
    aliases and overrides."""
    import torch
    bodies = [
        # integer bits, as u32 bit patterns
        """let u = bitcast<u32>(p.x);
let i = bitcast<i32>(p.y);
let w = bitcast<u32>(p.z);
let o = u32(t);
let c = w % 40u;
return bitcast<vec3<f32>>(vec3<u32>(
    countLeadingZeros(u) | (countOneBits(u) << 8u) | (countTrailingZeros(u) << 16u),
    reverseBits(u) ^ bitcast<u32>(firstLeadingBit(i)) ^ firstTrailingBit(u) ^ (firstLeadingBit(u) << 3u),
    extractBits(u, o, c) ^ bitcast<u32>(extractBits(i, o, c)) ^ insertBits(u, w, o, c)));""",
        # packing and packed dot products
        """let u = bitcast<u32>(p.x);
let w = bitcast<u32>(p.z);
let e = vec4<f32>(v, t);
return bitcast<vec3<f32>>(vec3<u32>(pack4x8snorm(e) ^ pack2x16float(v.xy),
    pack4x8unorm(e) ^ pack2x16snorm(v.yz) ^ pack2x16unorm(v.xz),
    dot4U8Packed(u, w) ^ bitcast<u32>(dot4I8Packed(u, w)) ^ pack4xI8Clamp(unpack4xI8(u)) ^ pack4xU8(unpack4xU8(w))));""",
        # unpacking and decomposition, as floats
        """let u = bitcast<u32>(p.x);
let f = frexp(v);
let m = modf(v.x * 100.0);
return unpack4x8snorm(u).xyz + unpack4x8unorm(u).xyz + vec3<f32>(unpack2x16float(u), 0.0)
     + f.fract + vec3<f32>(f.exp) * 0.25 + vec3<f32>(m.fract, m.whole, ldexp(v.y, i32(t) - 20))
     + quantizeToF16(v * 1000.0);""",
    ]
    x, _ = _bits_inputs(2048)
    rng = np.random.default_rng(31)
    x[:, 9:12] = rng.uniform(-3, 3, (len(x), 3)).astype(np.float32)
    cases = [(b, None) for b in bodies]
    # pointers, arrays of arrays, aliases and overrides on the device (their
    # x arguments are the float inputs, so give p finite values)
    xf = x.copy()
    xf[:, 3:6] = rng.uniform(-2, 2, (len(x), 3)).astype(np.float32)
    cases += [(POINTER_BODY, POINTER_HELPERS), (NESTED_BODY, NESTED_HELPERS),
              (ALIAS_OVERRIDE_BODY, ALIAS_OVERRIDE_HELPERS)]
    for k, (body, helpers) in enumerate(cases):
        if helpers is not None:
            fld = engine.compile_field(body, helpers, precise=True)
            dev = engine.field_eval(fld, torch.from_numpy(xf).cuda()).cpu().numpy()
            np.testing.assert_array_equal(dev, _host_eval(body, xf, helpers))
            continue
        fld = engine.compile_field(body, precise=True)
        dev = engine.field_eval(fld, torch.from_numpy(x).cuda()).cpu().numpy()
        host = _host_eval(body, x)
        # the first two return integer bit patterns (compared as they are);
        # the last computes in floats, whose NaN payloads differ between the
        # CPU and the GPU
        both_nan = (np.isnan(dev) & np.isnan(host)) if k == 2 else np.zeros(dev.shape, bool)
        np.testing.assert_array_equal(np.where(both_nan, 0, dev.view(np.uint32)),
                                      np.where(both_nan, 0, host.view(np.uint32)))


NESTED_HELPERS = """
struct Cell { w: f32, k: array<i32, 2> }
alias Grid = array<array<f32, 3>, 2>;
fn total(g: Grid) -> f32 {
    var s = 0.0;
    for (var i = 0; i < 2; i++) { for (var j = 0; j < 3; j++) { s += g[i][j]; } }
    return s;
}
"""

NESTED_BODY = """
var g: Grid;                                         // zero value
g[1][2] = p.x;
g[0] = array<f32, 3>(1.0, p.y, 3.0);
let h = g;                                           // value copy
g[0][0] = 100.0;
let m = array(array(p.z, 2.0), array(4.0, v.x));     // inferred, abstract literals made f32
var cells = array<array<Cell, 2>, 2>();
cells[1][0] = Cell(t, array<i32, 2>(3, 4));
cells[1][0].k[1] = 7;
let i = i32(t) % 4;                                  // runtime index, clamped to [0, 1]
return vec3<f32>(total(h), m[1][1] + m[0][0] + m[i][1], cells[1][0].w + f32(cells[1][0].k[1]) + g[0][0]);
"""


def test_arrays_of_arrays_semantics():
    """array<array<T, N>, M>: zero values, element and row assignment, value
    copies, inferred nested constructors, arrays of structs in arrays,
    clamped runtime indices, aliases, function parameters."""
    rng = np.random.default_rng(9)
    x = rng.uniform(-2, 2, (24, 13)).astype(np.float32)
    x[:, 12] = rng.integers(-3, 9, 24).astype(np.float32)
    out = _host_eval(NESTED_BODY, x, NESTED_HELPERS)
    p, v, t = x[:, 3:6], x[:, 9:12], x[:, 12]
    total = ((np.float32(1.0) + p[:, 1]) + np.float32(3.0)) + np.float32(0) + np.float32(0) + p[:, 0]
    idx = np.clip(np.fmod(t.astype(np.int32), 4), 0, 1)
    m = np.stack([np.stack([p[:, 2], np.full(24, 2.0, np.float32)], -1),
                  np.stack([np.full(24, 4.0, np.float32), v[:, 0]], -1)], 1)
    col1 = m[np.arange(24), idx, 1]
    want = np.stack([total.astype(np.float32), (v[:, 0] + p[:, 2]) + col1, (t + np.float32(7.0)) + np.float32(100.0)], -1)
    np.testing.assert_allclose(out, want.astype(np.float32), rtol=0, atol=1e-6)
    assert "linon_march_v1" in validate_field(NESTED_BODY, NESTED_HELPERS)
    code = translate_wgsl(NESTED_BODY, NESTED_HELPERS)
    assert "::wgsl::arr<::wgsl::arr<float,3>,2>" in code


@pytest.mark.parametrize("body,needle", [
    ("let a = array(array(1.0, 2.0), array(1.0, 2.0, 3.0)); return p;", "array elements of different types"),
    ("var a: array<array<f32, 2>, 2>; a[0] = array<f32, 3>(1.0, 2.0, 3.0); return p;", "cannot assign"),
    ("var a: array<array<f32, 2>, 2>; let b = a[0][2]; return p;", "index out of bounds"),
])
def test_nested_array_diagnostics(body, needle):
    with pytest.raises(_abi.LinonCompileError) as e:
        translate_wgsl(body)
    assert needle in e.value.message, e.value.message


POINTER_HELPERS = """
fn split(x: f32, whole: ptr<function, f32>, frac: ptr<function, f32>) {
    *whole = floor(x);
    *frac = x - *whole;
}
fn bump(v: ptr<function, vec3<f32>>, k: f32) {
    (*v).y += k;
    v.z = v.x * 2.0;                 // pointer composite access
}
fn fill(a: ptr<function, array<f32, 3>>, s: f32) {
    for (var i = 0; i < 3; i++) { a[i] = s * f32(i); }
}
struct Acc { sum: f32, n: i32 }
fn add(acc: ptr<function, Acc>, x: f32) {
    acc.sum += x;
    (*acc).n = (*acc).n + 1;
}
"""

POINTER_BODY = """
var w = 0.0;
var f = 0.0;
split(p.x * 3.0, &w, &f);
var q = v;
bump(&q, t);
let r = &q;
r.x = (*r).x + 1.0;
var arr: array<f32, 3>;
fill(&arr, w);
var acc = Acc(0.0, 0);
add(&acc, f);
add(&acc, arr[2]);
var s = array<Acc, 2>();
add(&s[1], 5.0);
return vec3<f32>(w + f, q.y + q.z + q.x, acc.sum + f32(acc.n) + s[1].sum);
"""


def test_pointer_semantics():
    """ptr<function, T> parameters (out-parameters), '&' of variables and of
    parts of them, '*' and WGSL's pointer composite access, a pointer bound
    with 'let'."""
    rng = np.random.default_rng(12)
    x = rng.uniform(-2, 2, (20, 13)).astype(np.float32)
    out = _host_eval(POINTER_BODY, x, POINTER_HELPERS)
    p, v, t = x[:, 3:6], x[:, 9:12], x[:, 12]
    y = p[:, 0] * np.float32(3.0)
    w = np.floor(y)
    f = y - w
    q = v.copy()
    q[:, 1] = q[:, 1] + t
    q[:, 2] = q[:, 0] * np.float32(2.0)
    q[:, 0] = q[:, 0] + np.float32(1.0)
    a2 = w * np.float32(2.0)
    acc = (np.float32(0.0) + f) + a2
    want = np.stack([w + f, (q[:, 1] + q[:, 2]) + q[:, 0], (acc + np.float32(2.0)) + np.float32(5.0)], -1)
    np.testing.assert_array_equal(out, want.astype(np.float32))
    assert "linon_march_v1" in validate_field(POINTER_BODY, POINTER_HELPERS)


@pytest.mark.parametrize("helpers,body,needle", [
    ("", "let a = 1.0; let q = &a; return p;", "needs a variable"),
    ("", "var a = p; let q = &a.x; return p;", "vector component"),
    ("", "var a = 1.0; var q = &a; return p;", "only be declared with 'let'"),
    ("", "let a = *p; return p;", "'*' needs a pointer"),
    ("fn f(x: ptr<function, f32>) -> ptr<function, f32> { return x; }", "return p;", "cannot return a pointer"),
    ("struct S { a: ptr<function, f32> }", "return p;", "struct member cannot be a pointer"),
    ("fn f(x: array<ptr<function, f32>, 2>) {}", "return p;", "array element cannot be a pointer"),
    ("fn f(x: ptr<private, f32>) {}", "return p;", "only ptr<function, T>"),
    ("fn f(x: ptr<function, f32>, y: ptr<function, f32>) { *x = *y; }",
     "var a = 1.0; f(&a, &a); return p;", "aliasing"),
    ("fn f(x: ptr<function, f32>) {}", "var a = 1; f(&a); return p;", "expected ptr<function, f32>"),
])
def test_pointer_diagnostics(helpers, body, needle):
    with pytest.raises(_abi.LinonCompileError) as e:
        translate_wgsl(body, helpers or None)
    assert needle in e.value.message, e.value.message


def test_const_assert_and_directives():
    """const_assert at module and function scope (checked at translation,
    no code), the diagnostic and requires directives, @diagnostic and
    @must_use attributes."""
    helpers = """
requires pointer_composite_access, packed_4x8_integer_dot_product;
diagnostic(off, derivative_uniformity);
const N = 3;
const_assert N > 2 && !(N == 4);
const_assert 1.5 < 2.0;
@must_use @diagnostic(warning, derivative_uniformity) fn twice(x: f32) -> f32 { return 2.0 * x; }
"""
    code = translate_wgsl("const_assert N * 2 == 6;\nconst_assert true || false;\nreturn p * twice(t);", helpers)
    assert "const_assert" not in code and "u_twice" in code


@pytest.mark.parametrize("helpers,body,needle", [
    ("const_assert 1 > 2;", "return p;", "const_assert failed"),
    ("", "const_assert p.x > 0.0; return p;", "needs a constant expression"),
    ("", "const_assert 1; return p;", "needs a bool expression"),
    ("requires no_such_extension;", "return p;", "unknown language extension"),
    ("diagnostic(loud, derivative_uniformity);", "return p;", "unknown diagnostic severity"),
    ("enable f16;", "return p;", "SHADER_F16"),
])
def test_const_assert_and_directive_diagnostics(helpers, body, needle):
    with pytest.raises(_abi.LinonCompileError) as e:
        translate_wgsl(body, helpers or None)
    assert needle in e.value.message, e.value.message


def test_integer_division_modulo_and_shifts():
    """WGSL's integer '/' and '%' (a / 0 = a, a % 0 = 0, most negative i32
    over -1), shifts by the amount's low 5 bits (also vectors, i32 << u32),
    and '%' with a vector and a scalar (integer and float)."""
    rng = np.random.default_rng(41)
    n = 2000
    x = np.zeros((n, 13), np.float32)
    ai = rng.integers(-2 ** 31, 2 ** 31, n, dtype=np.int64)
    bi = rng.integers(-9, 10, n, dtype=np.int64)
    ai[:6] = [-2 ** 31, -2 ** 31, 7, -7, 0, 2 ** 31 - 1]
    bi[:6] = [-1, 0, 0, 0, 0, -1]
    sh = rng.integers(0, 70, n, dtype=np.int64)
    x[:, 3] = ai.astype(np.int32).view(np.float32)
    x[:, 4] = bi.astype(np.int32).view(np.float32)
    x[:, 5] = sh.astype(np.uint32).view(np.float32)
    x[:, 9:12] = rng.uniform(-5, 5, (n, 3)).astype(np.float32)
    body = """
let a = bitcast<i32>(p.x);
let b = bitcast<i32>(p.y);
let s = bitcast<u32>(p.z);
let ua = bitcast<u32>(a);
let ub = bitcast<u32>(b);
let va = vec2<i32>(a, b) / vec2<i32>(b, 3) + vec2<i32>(a, 7) % b;
let q = a / b ^ (a % b) * 3;
return bitcast<vec3<f32>>(vec3<u32>(bitcast<u32>(q) ^ (ua / ub) ^ ((ua % ub) << 7u),
                                    bitcast<u32>(a << s) ^ bitcast<u32>(a >> s) ^ (ua >> s),
                                    bitcast<u32>(va.x ^ va.y) ^ bitcast<u32>((vec2<i32>(a) << vec2<u32>(s, 1u)).x)));
"""
    out = _host_eval(body, x).view(np.uint32)

    def s32(v):
        v &= M32
        return v - (1 << 32) if v & 0x80000000 else v

    def div(a, b):
        if b == 0 or (a == -2 ** 31 and b == -1):
            return a
        q = abs(a) // abs(b)
        return q if (a >= 0) == (b > 0) else -q

    def mod(a, b):
        if b == 0 or (a == -2 ** 31 and b == -1):
            return 0
        return a - div(a, b) * b

    def udiv(a, b):
        return a if b == 0 else a // b

    def umod(a, b):
        return 0 if b == 0 else a % b

    for k in range(n):
        a, b, s = int(ai[k]), int(bi[k]), int(sh[k]) & 31
        ua, ub = a & M32, b & M32
        q = s32(div(a, b) ^ (mod(a, b) * 3))
        e0 = (q & M32) ^ udiv(ua, ub) ^ ((umod(ua, ub) << 7) & M32)
        e1 = ((ua << s) & M32) ^ ((a >> s) & M32) ^ (ua >> s)
        va0 = s32(div(a, b) + mod(a, b))
        va1 = s32(div(b, 3) + mod(7, b))
        e2 = ((va0 ^ va1) & M32) ^ ((ua << s) & M32)
        assert list(out[k]) == [e0 & M32, e1 & M32, e2 & M32], k
    fb = "return vec3<f32>((v % 2.0).x, (3.0 % v).y, f32((vec3<i32>(7, -7, 9) % 4).y + (11 / vec2<i32>(2, 0)).y));"
    out = _host_eval(fb, x)
    v = x[:, 9:12]
    want = np.stack([v[:, 0] - np.float32(2.0) * np.trunc(v[:, 0] / np.float32(2.0)),
                     np.float32(3.0) - v[:, 1] * np.trunc(np.float32(3.0) / v[:, 1]),
                     np.full(n, -3.0 + 11.0, np.float32)], -1).astype(np.float32)
    np.testing.assert_array_equal(out, want)
    with pytest.raises(_abi.LinonCompileError) as e:
        translate_wgsl("let a = 1 << 40; return p;")
    assert "shift amount out of range" in e.value.message
    with pytest.raises(_abi.LinonCompileError):
        translate_wgsl("let a = 1u << 2i; return p;")  # the amount must be u32


def test_vector_complement_and_bitwise_ops():
    x, raw = _bits_inputs(200)
    body = """let u = bitcast<vec3<u32>>(p);
let i = bitcast<vec3<i32>>(p);
return bitcast<vec3<f32>>((~u) ^ bitcast<vec3<u32>>(~i & i) ^ (u | vec3<u32>(1u)));"""
    out = _host_eval(body, x).view(np.uint32)
    u = raw.astype(np.int64)
    want = ((~u) & M32) ^ 0 ^ (u | 1)
    np.testing.assert_array_equal(out, want.astype(np.uint32))


def test_every_accepted_operator_combination_compiles():
    """Each binary operator over every pair of scalar / vec2 operand types
    (f32, i32, u32, bool), and each unary operator: the front end accepts
    exactly the combinations WGSL defines, and everything it accepts
    compiles (host g++ and NVRTC for sm_103a)."""
    types = ["f32", "i32", "u32", "bool", "vec2<f32>", "vec2<i32>", "vec2<u32>", "vec2<bool>"]
    binops = ["+", "-", "*", "/", "%", "&", "|", "^", "<<", ">>", "<", "<=", ">", ">=", "==", "!=", "&&", "||"]
    num = {"f32", "i32", "u32"}

    def kind(t):
        return t.replace("vec2<", "").replace(">", "")

    def wgsl_defines(a, b, op):
        ka, kb, va, vb = kind(a), kind(b), a.startswith("vec"), b.startswith("vec")
        if op in ("+", "-", "*", "/", "%"):
            return ka == kb and ka in num                       # scalar/vector mixes allowed
        if op in ("<", "<=", ">", ">="):
            return ka == kb and ka in num and va == vb
        if op in ("==", "!="):
            return ka == kb and va == vb
        if op in ("&", "|"):
            return ka == kb and va == vb and ka in ("i32", "u32", "bool")
        if op == "^":
            return ka == kb and va == vb and ka in ("i32", "u32")
        if op in ("<<", ">>"):
            return ka in ("i32", "u32") and kb == "u32" and va == vb
        return ka == kb == "bool" and not va and not vb           # && ||

    lines = []
    for a in types:
        for b in types:
            for op in binops:
                stmt = f"{{ let x = {a}(); let y = {b}(); let z{len(lines)} = x {op} y; }}"
                try:
                    translate_wgsl(stmt + "\nreturn p;")
                    ok = True
                except _abi.LinonCompileError:
                    ok = False
                assert ok == wgsl_defines(a, b, op), (a, op, b, ok)
                if ok:
                    lines.append(stmt)
    for a in types:
        for op in ["-", "!", "~"]:
            stmt = f"{{ let x = {a}(); let z = {op}x; }}"
            try:
                translate_wgsl(stmt + "\nreturn p;")
                ok = True
            except _abi.LinonCompileError:
                ok = False
            k = kind(a)
            assert ok == ((op == "-" and k in ("f32", "i32")) or (op == "!" and k == "bool")
                          or (op == "~" and k in ("i32", "u32"))), (op, a, ok)
            if ok:
                lines.append(stmt)
    assert len(lines) == 136
    body = "\n".join(lines) + "\nreturn p;"
    _host_eval(body, np.zeros((2, 13), np.float32))           # compiles for the host
    assert "linon_march_v14" in validate_field(body)          # and for the GPU, fast
    assert "linon_march_v1" in validate_field(body, precise=True)  # and precise modules


def test_every_accepted_builtin_call_compiles():
    """The numeric builtins called with one to three arguments of each
    scalar / vector type (and the extra shapes of extractBits, insertBits,
    ldexp, select, mix): every call the front end accepts compiles for the
    host and for sm_103a."""
    names = ("abs acos acosh asin asinh atan atanh atan2 ceil clamp cos cosh countLeadingZeros countOneBits "
             "countTrailingZeros cross degrees determinant distance dot exp exp2 extractBits faceForward "
             "firstLeadingBit firstTrailingBit floor fma fract frexp insertBits inverseSqrt ldexp length log log2 "
             "max min mix modf normalize pow quantizeToF16 radians reflect refract reverseBits round saturate sign "
             "sin sinh smoothstep sqrt step tan tanh transpose trunc select all any").split()
    types = [f"{v}{k}" for v in ("", "vec2<", "vec3<", "vec4<") for k in ("f32", "i32", "u32", "bool")]
    types = [t + (">" if t.startswith("vec") else "") for t in types]
    lines = []
    for n in names:
        for t in types:
            for args in (f"{t}()", f"{t}(), {t}()", f"{t}(), {t}(), {t}()", f"{t}(), 1u, 2u",
                         f"{t}(), {t}(), 1u, 2u", f"{t}(), 2", f"{t}(), {t}(), true", f"{t}(), {t}(), 0.5"):
                stmt = f"{{ let z{len(lines)} = {n}({args}); }}"
                try:
                    translate_wgsl(stmt + "\nreturn p;")
                except _abi.LinonCompileError:
                    continue
                lines.append(stmt)
    assert len(lines) > 250, len(lines)
    body = "\n".join(lines) + "\nreturn p;"
    _host_eval(body, np.zeros((2, 13), np.float32))
    assert "linon_march_v14" in validate_field(body)
    assert "linon_march_v1" in validate_field(body, precise=True)
    v = _host_eval("return vec3<f32>(f32(dot(vec4<i32>(1, -2, 3, 4), vec4<i32>(5, 6, -7, 8))),"
                   " f32(dot(vec2<u32>(3u, 4u), vec2<u32>(5u, 6u))), 0.0);", np.zeros((1, 13), np.float32))
    np.testing.assert_array_equal(v[0], [5 - 12 - 21 + 32, 39, 0])


def test_i32_arithmetic_wraps():
    """i32 + - * and unary - wrap on overflow, as WGSL defines (the generated
    code computes them in u32: no undefined behaviour on the host or GPU)."""
    x = np.zeros((1, 13), np.float32)
    x[0, 3:6] = np.array([2 ** 31 - 1, -2 ** 31, 65536], np.int32).view(np.float32)
    body = """let m = bitcast<i32>(p.x);
let n = bitcast<i32>(p.y);
let k = bitcast<i32>(p.z);
let v = vec2<i32>(m, n) + vec2<i32>(1, -1);
return bitcast<vec3<f32>>(vec3<i32>(m + 1, (-n) ^ (k * k), v.x ^ v.y ^ (n - 1) ^ (vec2<i32>(k) * k).y));"""
    out = _host_eval(body, x).view(np.int32)[0]
    i32min = -2 ** 31
    assert out[0] == i32min                                   # INT_MAX + 1
    assert out[1] == (i32min ^ 0)                             # -INT_MIN = INT_MIN; 65536 * 65536 = 0
    assert out[2] == (i32min ^ (2 ** 31 - 1) ^ (2 ** 31 - 1) ^ 0)


def test_fuzzed_fields_never_crash_and_compile_when_accepted():
    """Seeded token mutations of the predefined fields and of this file's
    test bodies: the front end returns a status for every one (no crash, no
    hang), and every mutant it accepts compiles for the host."""
    import random
    import re as _re
    rng = random.Random(2024)
    lib = _abi.load()
    pool = [(predefined_source(i), None) for i in range(1, 15)]
    pool += [(POINTER_BODY, POINTER_HELPERS), (NESTED_BODY, NESTED_HELPERS),
             (ALIAS_OVERRIDE_BODY, ALIAS_OVERRIDE_HELPERS), (ALL_NEW_BUILTINS_BODY, None),
             (SWITCH_BODY, None), (STRUCT_BODY, STRUCT_HELPERS), (PRIVATE_BODY, PRIVATE_HELPERS)]
    toks = ["(", ")", ";", ",", ".", "&", "*", "-", "!", "~", "+", "%", "/", "<<", ">>", "^", "|", "&&", "==", "<",
            "let", "var", "1", "1.5", "2u", "-3", "p", "v", "t", "x", "i32", "f32", "u32", "vec2", "vec3<i32>",
            "vec3<u32>", "select", "abs", "max", "dot", "countOneBits", "frexp", "[0]", ".xy", "true"]
    out = C.create_string_buffer(1 << 20)
    log = C.create_string_buffer(1 << 16)
    accepted = {}
    for _ in range(2500):
        body, helpers = rng.choice(pool)
        mut_helpers = helpers is not None and rng.random() < 0.5
        words = _re.findall(r"\w+|[^\w\s]+|\s+", helpers if mut_helpers else body)
        for _k in range(rng.randint(1, 3)):
            i = rng.randrange(len(words))
            r = rng.random()
            if r < 0.35:
                del words[i]
            elif r < 0.7:
                words.insert(i, rng.choice(toks))
            else:
                words[i] = rng.choice(toks)
        m = "".join(words)
        b, h = (body, m) if mut_helpers else (m, helpers)
        st = lib.linon_wgsl_translate(b.encode(), h.encode() if h else None, out, len(out), log, len(log))
        assert st in (_abi.LINON_OK, _abi.LINON_ECOMPILE)
        if st == _abi.LINON_OK:
            accepted[out.value] = True
    assert len(accepted) > 50
    d = scratch_dir("linon_fuzz_")
    files = []
    for k, code in enumerate(accepted):
        f = d / f"m{k}.cpp"
        f.write_text(f'#include "{RT}"\n' + code.decode())
        files.append(f)
    failures = []
    for k in range(0, len(files), 32):
        procs = [(f, subprocess.Popen(["g++", "-std=c++17", "-fsyntax-only", str(f)], stderr=subprocess.PIPE,
                                      text=True)) for f in files[k:k + 32]]
        for f, p in procs:
            _, err = p.communicate(timeout=120)
            if p.returncode != 0:
                failures.append((f.read_text()[-600:], err[:600]))
    assert not failures, failures[:2]


PRIVATE_HELPERS = """
var<private> calls: u32 = 0u;
var<private> acc: vec3<f32>;
var<private> hist: array<f32, 4>;
fn note(x: f32) {
    hist[calls % 4u] = x;
    acc += vec3<f32>(x, 1.0, 0.0);
}
"""
PRIVATE_BODY = """
calls += 1u;
note(t * f32(calls));
return acc + vec3<f32>(hist[0] + hist[1] + hist[2] + hist[3], f32(calls), 0.0);
"""


def test_private_variables_persist_within_an_invocation():
    """var<private>: one state per invocation (one ray), initialised from
    its initialiser or zero, kept across the field's calls in that
    invocation, written by helper functions."""
    x = np.zeros((3, 13), np.float32)
    x[:, 12] = [1.0, 2.0, 0.5]
    for calls in (1, 3, 6):
        out = _host_eval(PRIVATE_BODY, x, PRIVATE_HELPERS, calls=calls)
        for row, t in zip(out, x[:, 12]):
            vals = [np.float32(t) * np.float32(c) for c in range(1, calls + 1)]
            acc_x = np.float32(0)
            for v in vals:
                acc_x = np.float32(acc_x + v)
            hist = [0.0] * 4
            for c, v in enumerate(vals, start=1):
                hist[c % 4] = v
            h = np.float32(np.float32(np.float32(hist[0] + hist[1]) + hist[2]) + hist[3])
            np.testing.assert_array_equal(row, [acc_x + h, np.float32(calls) + np.float32(calls), 0.0])
    assert "linon_multi_fk" in validate_field(PRIVATE_BODY, PRIVATE_HELPERS, batched=True)


@pytest.mark.parametrize("helpers,needle", [
    ("var<workgroup> w: f32;", "only var<private>"),
    ("var<private> w;", "needs a type or an initializer"),
    ("var<private> w: f32 = 1.0;\nconst c = w * 2.0;\nfn f() -> f32 { return c; }", "module initializers must be constant"),
    ("var<private> w: f32 = 1.0;\nvar<private> z: f32 = w;", "module initializers must be constant"),
])
def test_private_variable_diagnostics(helpers, needle):
    with pytest.raises(_abi.LinonCompileError) as e:
        translate_wgsl("return p;", helpers)
    assert needle in e.value.message, e.value.message


CALLER_HELPERS = """
var<private> n: u32;
fn euler(p0: vec3<f32>, v0: vec3<f32>, h: f32) -> vec3<f32> {
  var p = p0;
  for (var i = 0; i < 3; i++) {
    p = p + h * field_function(p, p, v0, v0, f32(i));
  }
  return p;
}
"""


def test_helper_calls_the_field_function():
    """A helper may call the field function (the shader's own march loop,
    main_view.wgsl:229-279, is such a helper); the call passes the
    invocation's private state, and a cycle through the field function is
    rejected as recursion."""
    code = translate_wgsl("n += 1u;\nreturn v * 2.0 + vec3<f32>(t, f32(n), 0.0);", CALLER_HELPERS)
    src = "\n".join([f'#include "{RT}"', code,
                     'extern "C" void run(float* out) {',
                     "  linon_user::Private pv;",
                     "  wgsl::vec3f r = linon_user::u_euler(pv, wgsl::vec3f(1.f, 2.f, 3.f), wgsl::vec3f(0.5f, 0.f, 1.f), 0.25f);",
                     "  out[0] = r.x; out[1] = r.y; out[2] = r.z; out[3] = float(pv.u_n); }"])
    d = scratch_dir("linon_fe2_")
    (d / "f.cpp").write_text(src)
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-shared", "-fPIC", "-o", str(d / "f.so"),
                        str(d / "f.cpp")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    out = np.zeros(4, np.float32)
    C.CDLL(str(d / "f.so")).run(C.c_void_p(out.ctypes.data))
    p = np.float32([1, 2, 3])
    for i in range(3):
        k = np.float32([0.5, 0, 1]) * np.float32(2) + np.float32([i, i + 1, 0])
        p = (p + np.float32(0.25) * k).astype(np.float32)
    np.testing.assert_array_equal(out, list(p) + [3.0])
    body = "n += 1u;\nreturn v * 2.0 + vec3<f32>(t, f32(n), 0.0);"
    assert "linon_march_v14" in validate_field(body, CALLER_HELPERS)  # NVRTC, sm_103a
    assert "linon_multi_fk" in validate_field(body, CALLER_HELPERS, batched=True)
    with pytest.raises(_abi.LinonCompileError) as e:
        translate_wgsl("return euler(p, v, 0.1);", CALLER_HELPERS)
    assert "recursion" in str(e.value)


@pytest.mark.parametrize("name,has_pair", [("linear", True), ("twist", True), ("lens", True), ("lorenz_scaled", True),
                                           ("rotation", True), ("translation_x", True), ("lorenz", True),
                                           ("mirage_spherical", False), ("mirage_plane_sigmoid", False)])
def test_pair_form_of_the_predefined_fields(name, has_pair):
    """Fields whose arithmetic is lane-wise compile in pair form (two rays
    per thread, packed FP32 pairs) for sm_103a; fields that branch on a value
    (the mirages' refraction) have none and keep one ray per thread."""
    from linon_gb300 import _abi
    from linon_gb300.engine import predefined_source, validate_field
    log = validate_field(predefined_source(_abi.FIELD_IDS[name]))
    assert ("pair form: compiles" in log) == has_pair, log[-400:]
    assert ("pair form: not available" in log) == (not has_pair)


def test_pair_form_rejects_a_branch_on_a_value():
    from linon_gb300.engine import validate_field
    log = validate_field("if (p.x < 0.0) { return v; }\nreturn v0;")
    assert "pair form: not available" in log
    # precise modules have no pair form at all
    log = validate_field("return v0;", precise=True)
    assert "pair form" not in log
    # nor fields with var<private> state: a private integer would be one
    # value for both rays of a thread
    log = validate_field("count = count + 1;\nreturn v0 * f32(count);", helpers="var<private> count: i32;")
    assert "pair form: not available" in log


def test_cli_validates_a_users_field_files(tmp_path):
    """`python -m linon_gb300 validate --body F [--helpers G]`: a user's
    edited field and helper files go through the front end and NVRTC (the
    reference's reload of an edited shader, src/main.rs:206-222); a rejected
    body prints the diagnostics and exits with status 1."""
    import sys
    (tmp_path / "body.wgsl").write_text("return rotateY(v0, 0.5 * p.y) + my_shift(p);\n")
    (tmp_path / "helpers.wgsl").write_text("fn my_shift(q: vec3<f32>) -> vec3<f32> { return 0.01 * q; }\n")
    (tmp_path / "bad.wgsl").write_text("return q;\n")
    cmd = [sys.executable, "-m", "linon_gb300", "validate"]
    r = subprocess.run(cmd + ["--body", str(tmp_path / "body.wgsl"), "--helpers", str(tmp_path / "helpers.wgsl")],
                       cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert "registers" in r.stdout
    r = subprocess.run(cmd + ["--body", str(tmp_path / "bad.wgsl")], cwd=ROOT, capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 1
    assert "no definition in scope for identifier: 'q'" in r.stdout and "line 1, column 8" in r.stdout
