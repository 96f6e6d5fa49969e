"""The WGSL-to-C++ translation used to run the reference shader on the host (CPU).

A small compute module written here exercises the semantics the translation
must keep, independently of the reference checkout: abstract-numeric
constant expressions folded in binary64 and converted to f32 once (WGSL's
rule, which differs from f32 arithmetic: 0.1 / 0.3 folds to 0x3eaaaaab, the
f32 division gives 0x3eaaaaaa), saturating f32 -> integer conversions,
bit-reinterpreting integer conversions, wrapping i32 arithmetic, swizzles,
vector arithmetic and comparisons, loops with break and continue, struct
constructors, and atomics across host threads.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

MODULE = r"""
const SCALE: f32 = 2.5;
const FOLDED = 0.1 / 0.3;
struct Pair { a: vec4<f32>, b: vec4<f32>, }
struct Acc { count: atomic<u32>, total: atomic<i32>, }
@group(0) @binding(0) var<storage, read_write> out_f: array<f32>;
@group(0) @binding(1) var<storage, read_write> out_u: array<u32>;
@group(0) @binding(2) var<storage, read_write> out_i: array<i32>;
@group(0) @binding(3) var<storage, read_write> acc: array<Acc>;
@group(0) @binding(4) var<storage, read_write> pairs: array<Pair>;

fn scaled(v: vec3<f32>) -> vec3<f32> {
    return v * SCALE + vec3<f32>(0.5);
}

@compute @workgroup_size(64)
fn probe(@builtin(global_invocation_id) gid: vec3<u32>) {
    let i = gid.x;
    if (i != 0u) {
        return;
    }
    let a = 0.1;
    let b = 0.3;
    out_f[0] = FOLDED;                 // folded in binary64: RN32(0.1 / 0.3)
    out_f[1] = f32(a) / f32(b);        // let-bound: f32 values, f32 division
    let big = 3.0e9 + f32(i);          // runtime values: constant ones out of
    let m1 = i32(i) - 1;               // range would not compile as WGSL
    out_i[0] = i32(big);               // saturates
    out_i[1] = i32(-big);
    out_u[0] = u32(f32(m1) - 0.5);     // saturates at 0
    out_u[1] = u32(m1);                // reinterprets the bits
    out_i[2] = i32(0xFFFFFFFEu);
    var w = 2147483647;
    w += 1;                            // wraps
    out_i[3] = w;
    let v = scaled(vec3<f32>(1.0, 2.0, 3.0));
    out_f[2] = v.z;
    let q = vec4<f32>(v.xy, 7.0, 8.0);
    out_f[3] = dot(q.xyz, vec3<f32>(1.0, 1.0, 1.0));
    let lo = vec3<i32>(1, -2, 3) < vec3<i32>(0);
    out_u[2] = select(0u, 1u, any(lo));
    out_u[3] = select(0u, 1u, all(lo));
    var s = 0u;
    for (var k = 0u; k < 10u; k++) {
        if (k == 2u) { continue; }
        if (k == 6u) { break; }
        s += k;
    }
    out_u[4] = s;                      // 0 + 1 + 3 + 4 + 5
    var n = 0u;
    loop {
        n += 3u;
        if (n > 10u) { break; }
    }
    out_u[5] = n;
    var p = pairs[0];
    p.b = vec4<f32>(p.a.w, p.a.z, p.a.y, p.a.x);
    p.a.y = -p.a.y;
    pairs[0] = Pair(p.a * 2.0, p.b);
    out_f[4] = clamp(-4.0, -1.0, 1.0);
    out_f[5] = fract(-1.25);
    out_f[6] = round(2.5);             // ties to even
}

@compute @workgroup_size(256)
fn count(@builtin(global_invocation_id) gid: vec3<u32>) {
    atomicAdd(&acc[gid.x % 4u].count, 1u);
    atomicAdd(&acc[gid.x % 4u].total, i32(gid.x) - 500);
}
"""

HARNESS = r"""
extern "C" void bind(void *f, void *u, void *i, void *a, void *p) {
  w_out_f = (float *)f; w_out_u = (uint32_t *)u; w_out_i = (int32_t *)i;
  w_acc = (T_Acc *)a; w_pairs = (T_Pair *)p;
}
extern "C" void run(const char *name, uint32_t invocations) {
  for (const auto &e : wgsl_entries) {
    if (std::strcmp(e.name, name) != 0) continue;
#pragma omp parallel for
    for (int64_t x = 0; x < (int64_t)invocations; x++) e.fn(wgsl::make<uint32_t, 3>((uint32_t)x, 0u, 0u));
  }
}
"""


@pytest.fixture(scope="module")
def lib(tmp_path_factory):
    from oracle import wgsl_ref, wgsl_transpile
    d = str(tmp_path_factory.mktemp("wgsl_t"))
    src = os.path.join(d, "m.cpp")
    with open(src, "w") as fh:
        fh.write("#include <cstring>\n" + wgsl_transpile.transpile(MODULE) + HARNESS)
    so = os.path.join(d, "m.so")
    cmd = ["g++", *wgsl_ref.CXXFLAGS, "-I", wgsl_ref.HERE, "-I", wgsl_ref.MATH_DIR, src, "-o", so]
    res = subprocess.run(cmd, capture_output=True, text=True)
    assert res.returncode == 0, res.stderr
    L = C.CDLL(so)
    L.run.argtypes = [C.c_char_p, C.c_uint32]
    return L


def test_translation_semantics(lib):
    f = np.zeros(8, np.float32)
    u = np.zeros(8, np.uint32)
    i = np.zeros(8, np.int32)
    acc = np.zeros(8, np.uint32)
    pairs = np.array([[1, 2, 3, 4, 0, 0, 0, 0]], np.float32)
    lib.bind(*(x.ctypes.data_as(C.c_void_p) for x in (f, u, i, acc, pairs)))
    lib.run(b"probe", 64)
    assert f[0] == np.float32(0.1 / 0.3) and f.view(np.uint32)[0] == 0x3EAAAAAB
    assert f[1] == np.float32(0.1) / np.float32(0.3) and f.view(np.uint32)[1] == 0x3EAAAAAA
    assert list(i[:4]) == [2**31 - 1, -2**31, -2, -2**31]
    assert list(u[:2]) == [0, 0xFFFFFFFF]
    assert f[2] == np.float32(3.0) * np.float32(2.5) + np.float32(0.5)
    assert f[3] == np.float32(3.0) + np.float32(5.5) + np.float32(7.0)
    assert list(u[2:6]) == [1, 0, 13, 12]
    assert list(pairs[0]) == [2, -4, 6, 8, 4, 3, 2, 1]  # b copied before a.y is negated
    assert list(f[4:7]) == [-1.0, 0.75, 2.0]


def test_atomics_across_host_threads(lib):
    f = np.zeros(8, np.float32)
    u = np.zeros(8, np.uint32)
    i = np.zeros(8, np.int32)
    acc = np.zeros(8, np.uint32)
    pairs = np.zeros((1, 8), np.float32)
    lib.bind(*(x.ctypes.data_as(C.c_void_p) for x in (f, u, i, acc, pairs)))
    n = 100000
    lib.run(b"count", n)
    x = np.arange(n, dtype=np.int64)
    for k in range(4):
        assert acc[2 * k] == np.sum(x % 4 == k)
        assert acc[2 * k + 1].view(np.int32) == np.int32(np.sum(x[x % 4 == k] - 500) % 2**32)
