"""WGSL front end: lowering, diagnostics, FLOP counts, NVRTC compile (CPU only).

The generated CUDA C is also compiled for the host with g++ (device/wgsl_rt.cuh
is host/device code) and evaluated against the oracle's hand-written field
functions: without FMA contraction both are the same IEEE operations in the
same order, so every predefined field must agree bit for bit.
"""
import ctypes as C
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


def test_validate_rejects_front_end_errors():
    validate_field("return v;")
    with pytest.raises(_abi.LinonCompileError):
        validate_field("return undefined_thing;")
