"""The C ABI library: loads without a GPU, exports every declared symbol,
data layouts match the reference's uniforms, host-only entry points work."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from linon_gb300 import _abi, outline_indices
from linon_gb300.engine import predefined_name, predefined_source

HEADER = Path(__file__).resolve().parents[1] / "include" / "linon.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(linon_[a-z0-9_]+)\s*\(", text)))


def test_every_declared_symbol_is_exported(lib):
    names = declared_functions()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n
    # and every declared symbol has a ctypes prototype
    assert set(names) == set(_abi.PROTOTYPES), set(names) ^ set(_abi.PROTOTYPES)


def test_rust_binding_declares_every_function():
    """The Rust FFI binding a maintainer would add declares
    exactly the header's functions."""
    text = (HEADER.parents[1] / "INTEGRATION.md").read_text()
    rust = sorted(set(re.findall(r"pub fn (linon_[a-z0-9_]+)\(", text)))
    assert rust == declared_functions(), set(rust) ^ set(declared_functions())


_C_TO_RUST = {"float": "f32", "double": "f64", "int32_t": "i32", "uint32_t": "u32", "int64_t": "i64",
              "uint64_t": "u64", "size_t": "usize", "uint8_t": "u8"}


def _c_structs():
    """Field lists of the header's typedef structs: (name, base type, element
    count, pointer kind) in declaration order."""
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    out = {}
    for m in re.finditer(r"typedef struct (linon_\w+) \{(.*?)\} \1;", text, re.S):
        fields = []
        for decl in m.group(2).split(";"):
            decl = decl.strip()
            if not decl:
                continue
            d = re.match(r"(const\s+)?(\w+)\s*(\*?)\s*(.*)", decl)
            const, base, ptr, names = d.groups()
            for nm in names.split(","):
                a = re.match(r"\s*(\w+)\s*(?:\[(\d+)\])?", nm)
                ty = _C_TO_RUST.get(base, base)
                kind = ("*const " if const else "*mut ") if ptr else ""
                fields.append((a.group(1), ty, int(a.group(2) or 1), kind))
        out[m.group(1)] = fields
    return out


def _rust_structs():
    text = (HEADER.parents[1] / "INTEGRATION.md").read_text()
    out = {}
    for m in re.finditer(r"pub struct (linon_\w+) \{(.*?)\}", text, re.S):
        body = re.sub(r"//[^\n]*", "", m.group(2))
        if "_p: [u8; 0]" in body:
            continue
        fields = []
        for f in re.finditer(r"pub (\w+): ([^,]+?)\s*(?:,|$)", body.strip()):
            ty, n, kind = f.group(2).strip(), 1, ""
            pm = re.match(r"(\*mut |\*const )(\w+)$", ty)
            if pm:
                kind, ty = pm.group(1), pm.group(2)
            while True:  # [T; N] and [[T; N]; M] flatten to T x N*M
                am = re.match(r"\[(.*); (\d+)\]$", ty)
                if not am:
                    break
                ty, n = am.group(1).strip(), n * int(am.group(2))
            fields.append((f.group(1), ty, n, kind))
        out[m.group(1)] = fields
    return out


def test_rust_structs_match_header():
    """Every struct of the Rust binding in INTEGRATION.md has the header's
    fields in the header's order, with the same scalar types, element counts
    and pointer constness, and its constants have the header's values."""
    c, rust = _c_structs(), _rust_structs()
    assert len(c) >= 11 and set(c) == set(rust), set(c) ^ set(rust)
    for name, fields in c.items():
        assert rust[name] == fields, (name, rust[name], fields)
    text = HEADER.read_text()
    vals = {m.group(1): int(m.group(2)) for m in re.finditer(r"\b(LINON_[A-Z0-9_]+)\s*=\s*(-?\d+)", text)}
    vals.update({m.group(1): int(m.group(2)) for m in re.finditer(r"#define\s+(LINON_[A-Z0-9_]+)\s+(\d+)", text)})
    consts = re.findall(r"pub const (LINON_[A-Z0-9_]+): \w+ = (-?\d+);",
                        (HEADER.parents[1] / "INTEGRATION.md").read_text())
    assert len(consts) >= 15
    for k, v in consts:
        assert vals[k] == int(v), k


def test_ctypes_structs_match_header():
    """The Python binding's ctypes structures have the header's fields in the
    header's order, with the same scalar types and element counts (pointers
    as void pointers)."""
    py = {"linon_camera": _abi.Camera, "linon_settings": _abi.Settings, "linon_ray_sample": _abi.RaySample,
          "linon_march_params": _abi.MarchParams, "linon_frame": _abi.Frame, "linon_view": _abi.View,
          "linon_batch_tuning": _abi.BatchTuning, "linon_request": _abi.Request,
          "linon_serve_config": _abi.ServeConfig, "linon_result": _abi.Result,
          "linon_serve_counters": _abi.ServeStats}
    names = {v: k for k, v in py.items()}
    # size_t and uint64_t are one ctypes type on LP64 Linux: compare both as u64
    scalars = {C.c_float: "f32", C.c_double: "f64", C.c_int32: "i32", C.c_uint32: "u32", C.c_int64: "i64",
               C.c_uint64: "u64", C.c_size_t: "u64", C.c_uint8: "u8"}
    c = _c_structs()
    assert set(py) == set(c)
    for name, cls in py.items():
        got = []
        for fname, ftype in cls._fields_:
            n = 1
            while hasattr(ftype, "_length_") and ftype is not C.c_void_p:
                n, ftype = n * ftype._length_, ftype._type_
            if ftype is C.c_void_p:
                got.append((fname, "ptr", n))
            else:
                got.append((fname, names.get(ftype) or scalars[ftype], n))
        want = [(f, "ptr" if kind else ("u64" if ty == "usize" else ty), n) for f, ty, n, kind in c[name]]
        assert got == want, (name, got, want)


def test_constants_match_header():
    """Every LINON_* enum value and #define the Python bindings restate has
    the header's value."""
    text = HEADER.read_text()
    vals = {m.group(1): int(m.group(2)) for m in re.finditer(r"\b(LINON_[A-Z0-9_]+)\s*=\s*(-?\d+)", text)}
    vals.update({m.group(1): int(m.group(2)) for m in re.finditer(r"#define\s+(LINON_[A-Z0-9_]+)\s+(\d+)", text)})
    checked = 0
    for name, v in vals.items():
        if hasattr(_abi, name):
            assert getattr(_abi, name) == v, name
            checked += 1
    assert checked >= 12
    assert vals["LINON_VALIDATE_BATCHED"] == _abi.LINON_VALIDATE_BATCHED == 2
    fields = {k[len("LINON_FIELD_"):].lower(): v for k, v in vals.items()
              if k.startswith("LINON_FIELD_") and k != "LINON_FIELD_COUNT"}
    assert fields == _abi.FIELD_IDS
    assert vals["LINON_FIELD_COUNT"] == _abi.FIELD_COUNT


def test_struct_layouts():
    assert C.sizeof(_abi.Camera) == 112       # CameraUniform, main_view.rs:12-19
    assert C.sizeof(_abi.Settings) == 24      # Settings, main_view.rs:43-51
    assert C.sizeof(_abi.RaySample) == 32     # RaySample, main_view.wgsl:55-58
    assert _abi.Settings.lyapunov_scaling.offset == 20
    assert _abi.Camera.view_matrix.offset == 48


def test_reference_params(lib):
    p = _abi.reference_params()
    assert (p.h_initial, p.t_max, p.max_steps, p.adaptive) == (pytest.approx(0.1), 5.0, 0, 1)
    assert (p.h_fine, p.h_fine_above) == (pytest.approx(0.001), pytest.approx(0.002))
    assert (p.focal_length, p.viewport_height) == (pytest.approx(0.035), pytest.approx(0.025))
    # the Python restatement the workload builders (and the CPU reference
    # leg of bench.py) use is byte-identical to the library's defaults
    assert bytes(_abi.shader_params()) == bytes(p)


def test_reference_leg_does_not_map_the_engine_library():
    # building the benchmark workloads and the oracle's inputs must not load
    # liblinon.so (the CPU reference leg stands alone)
    import subprocess
    import sys
    code = ("import sys; sys.path.insert(0, '.');"
            "from linon_gb300 import workloads as wl, _abi;"
            "w = wl.frames_1080p(); v = wl.batch_uneven(64); l = wl.lyapunov_1024(); s = wl.plain_small();"
            "maps = open('/proc/self/maps').read();"
            "assert _abi._lib is None and 'liblinon.so' not in maps, 'engine library mapped'")
    r = subprocess.run([sys.executable, "-c", code], cwd=str(_abi._PKG.parent), capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_plain_c_caller(lib, tmp_path):
    """The header is strict C99 and the library links and answers a plain C
    program (the host-only entry points; no GPU): the boundary a Rust, Go or
    C caller binds."""
    import subprocess
    d = tmp_path
    src = d / "caller.c"
    src.write_text("""
#include <stdio.h>
#include <string.h>
#include "linon.h"
_Static_assert(sizeof(linon_camera) == 112, "CameraUniform");
_Static_assert(sizeof(linon_settings) == 24, "Settings");
_Static_assert(sizeof(linon_ray_sample) == 32, "RaySample");
int main(void) {
  linon_march_params p;
  memset(&p, 0xff, sizeof p);
  linon_march_params_reference(&p);
  char out[4096], log[1024];
  int st = linon_wgsl_translate("return v0;", NULL, out, sizeof out, log, sizeof log);
  linon_ctx* ctx = NULL;
  int bad = linon_create(0, 0, &ctx);
  printf("%d %.3f %.3f %d %d %d %s|%s\\n", linon_abi_version(), p.h_initial, p.t_max, p.max_steps, st,
         bad != LINON_OK && ctx == NULL, linon_status_string(LINON_ECOMPILE),
         linon_predefined_name(LINON_FIELD_LORENZ) ? linon_predefined_name(LINON_FIELD_LORENZ) : "?");
  return 0;
}
""")
    inc = HEADER.parent
    libdir = Path(_abi.LIB_PATH).parent
    exe = d / "caller"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", f"-I{inc}", str(src),
                        f"-L{libdir}", "-llinon", f"-Wl,-rpath,{libdir}", "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120,
                       env={"CUDA_VISIBLE_DEVICES": "", "PATH": "/usr/bin:/bin"})
    assert r.returncode == 0, r.stderr[-2000:]
    ver, h, tmax, steps, st, failed_cleanly, rest = r.stdout.split(" ", 6)
    assert int(ver) == _abi.load().linon_abi_version()
    assert (float(h), float(tmax), int(steps)) == (0.1, 5.0, 0)
    assert int(st) == _abi.LINON_OK and int(failed_cleanly) == 1
    status, name = rest.strip().split("|")
    assert status and name == predefined_name(_abi.FIELD_IDS["lorenz"])


def test_status_strings_and_predefined(lib):
    assert lib.linon_abi_version() == 2
    assert lib.linon_status_string(_abi.LINON_ECOMPILE) == b"field function compilation failed"
    assert predefined_name(3) == "Mirage (spherical sigmoid)"
    assert predefined_name(9) == "Roessler attractor"
    assert predefined_source(7) == "return normalize(v0 + rotateZ(v0, PI * t));"
    assert lib.linon_predefined_source(99) is None


def test_outline_indices_restated():
    """src/ray_samples.rs:29-49 restated in numpy: 4 sides x 99 quads x 4 tris."""
    idx = outline_indices()
    assert idx.shape == (4 * 99 * 4, 3)
    exp = []
    for a, b, c in ((0, 1, 2), (2, 3, 4), (4, 5, 6), (6, 7, 0)):
        for i in range(99):
            A, B, Cc = a * 100 + i, b * 100 + i, c * 100 + i
            exp += [(A, B + 1, A + 1), (A, B, B + 1), (B, Cc, B + 1), (Cc, Cc + 1, B + 1)]
    np.testing.assert_array_equal(idx, np.array(exp, np.uint16))


def test_create_without_gpu_fails_cleanly(lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    ctx = C.c_void_p()
    st = lib.linon_create(0, 0, C.byref(ctx))
    assert st in (_abi.LINON_ECUDA, _abi.LINON_EINVAL)
    assert ctx.value is None
    assert lib.linon_last_error()


def test_null_arguments_rejected(lib):
    assert lib.linon_render(None, None, None, None, None, None) == _abi.LINON_EINVAL
    assert lib.linon_scene_upload(None, None, 0, None, 0, None, 0) == _abi.LINON_EINVAL
    assert lib.linon_destroy(None) == _abi.LINON_OK
