"""The reference shader's compute passes, translated and run on the host (test infrastructure only).

``build()`` translates ``src/rainbow_fmm.wgsl`` of the reference checkout
(``RFMM_REFERENCE_DIR``, default ``/root/reference``) with
``wgsl_transpile.py`` into ``oracle/_ref/rainbow_fmm_wgsl.gen.cpp`` and
compiles it with ``wgsl_ref_harness.cpp`` (the native harness's dispatch
sequence, native/main.rs) into ``oracle/_ref/libwgsl_ref.so``.  Nothing of
the reference is stored in the repository: where the checkout is absent
(the GPU machine), the translation generated earlier into ``oracle/_ref/``
is compiled if it is there, else ``available()`` is False.  The fixture
generator and the CPU tests use it to produce and check the golden digests
that pin the oracle and the CUDA path to the reference's own code;
``bench.py``'s CPU legs time it beside the oracle port.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libwgsl_ref.so")
GEN = os.path.join(OUT_DIR, "rainbow_fmm_wgsl.gen.cpp")
MATH_DIR = os.path.join(os.path.dirname(HERE), "fmm-rainbow_gb300", "csrc")
REF_DIR = os.environ.get("RFMM_REFERENCE_DIR", "/root/reference")
SHADER = os.path.join(REF_DIR, "src", "rainbow_fmm.wgsl")

CXXFLAGS = ["-std=c++17", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
            "-fno-finite-math-only", "-fwrapv", "-Wall", "-Wno-unused-function",
            "-Wno-unused-variable", "-Wno-unused-but-set-variable"]


def shader_available() -> bool:
    """The reference checkout is present (translation can be regenerated)."""
    return os.path.exists(SHADER)


def available() -> bool:
    """The translation can be built: from the checkout, or from a translation
    generated earlier into oracle/_ref/ (machines without the checkout)."""
    return shader_available() or os.path.exists(GEN)


def _compile(shader_text, gen_path: str, lib_path: str) -> str:
    """Translate `shader_text` into gen_path (None: use gen_path as it is) and
    compile it with the harness into lib_path."""
    from . import wgsl_transpile
    os.makedirs(OUT_DIR, exist_ok=True)
    if shader_text is not None:
        with open(gen_path, "w") as fh:
            fh.write(wgsl_transpile.transpile(shader_text))
    tmp = lib_path + ".tmp%d" % os.getpid()
    cmd = ["g++", *CXXFLAGS, "-I", HERE, "-I", MATH_DIR, "-include", gen_path,
           os.path.join(HERE, "wgsl_ref_harness.cpp"), "-o", tmp]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("reference harness build failed:\n%s\n%s" % (" ".join(cmd), res.stderr))
    os.replace(tmp, lib_path)
    return lib_path


def build(force: bool = False) -> str:
    """Translate the reference shader and compile the harness.  Without the
    checkout, compile the translation generated earlier into oracle/_ref/."""
    if not available():
        raise FileNotFoundError("reference shader not found: %s" % SHADER)
    deps = [os.path.join(HERE, "wgsl_transpile.py"), os.path.join(HERE, "wgsl_runtime.hpp"),
            os.path.join(HERE, "wgsl_ref_harness.cpp"), os.path.join(MATH_DIR, "rfmm_math.h")]
    if shader_available():
        deps.append(SHADER)
    else:
        deps = [GEN] + deps[1:]
    if (not force and os.path.exists(LIB)
            and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps)):
        return LIB
    if shader_available():
        with open(SHADER) as fh:
            return _compile(fh.read(), GEN, LIB)
    return _compile(None, GEN, LIB)


def build_variant(shader_text: str, tag: str) -> C.CDLL:
    """Compile an edited copy of the shader text (tests plant mistakes this way)."""
    path = _compile(shader_text, os.path.join(OUT_DIR, "variant_%s.gen.cpp" % tag),
                    os.path.join(OUT_DIR, "libwgsl_variant_%s.so" % tag))
    return _bind(C.CDLL(path))


class RefConfig(C.Structure):
    """The uniform values the native harness writes (native/main.rs:39-86), settable."""

    _fields_ = [
        ("count", C.c_uint32), ("depth", C.c_uint32), ("cells", C.c_uint32), ("scale", C.c_float),
        ("dt", C.c_float), ("gravity", C.c_float), ("softening", C.c_float), ("speed", C.c_float),
        ("control_point", C.c_float * 4), ("control_axis_mode", C.c_float * 4),
        ("control_strength", C.c_float), ("control_radius", C.c_float),
    ]


_lib = None


def _bind(L):
    vp, P = C.c_void_p, C.POINTER(RefConfig)
    L.wref_seed.argtypes = [vp, P]
    L.wref_solve_fields.argtypes = [vp, vp, vp, P]
    L.wref_frames.argtypes = [vp, vp, vp, P, C.c_uint32]
    L.wref_set_threads.argtypes = [C.c_int]
    for f in (L.wref_seed, L.wref_solve_fields, L.wref_frames, L.wref_set_threads):
        f.restype = C.c_int
    return L


def lib():
    global _lib
    if _lib is None:
        _lib = _bind(C.CDLL(build()))
    return _lib


def config(n, depth, cells, scale, dt=0.0009, gravity=0.34, softening=0.012, speed=1.0,
           control_point=(0.0, 0.0, 0.0, 0.0), control_axis_mode=(0.0, 0.0, 0.0, 0.0),
           control_strength=0.7, control_radius=0.22) -> RefConfig:
    """Defaults are the native harness's values (native/main.rs:55-81)."""
    c = RefConfig()
    c.count, c.depth, c.cells, c.scale = n, depth, cells, scale
    c.dt, c.gravity, c.softening, c.speed = dt, gravity, softening, speed
    c.control_point[:] = list(control_point)
    c.control_axis_mode[:] = list(control_axis_mode)
    c.control_strength, c.control_radius = control_strength, control_radius
    return c


def set_threads(n: int) -> int:
    """Host threads for the translated dispatches (<= 0: all)."""
    return lib().wref_set_threads(n)


class RefState:
    """Particle, moment and field buffers driven through the translated passes."""

    def __init__(self, particles: np.ndarray, cfg: RefConfig, library=None):
        self.cfg = cfg
        self.lib = library
        self.particles = np.ascontiguousarray(particles).copy()
        assert self.particles.nbytes == 32 * cfg.count
        self.moments = np.zeros(cfg.cells * 4, np.uint32)
        self.fields = np.zeros(cfg.cells * 12, np.float32)

    def _ptrs(self):
        return (self.particles.ctypes.data_as(C.c_void_p), self.moments.ctypes.data_as(C.c_void_p),
                self.fields.ctypes.data_as(C.c_void_p))

    def solve_fields(self):
        _ok((self.lib or lib()).wref_solve_fields(*self._ptrs(), C.byref(self.cfg)))

    def frames(self, k: int):
        _ok((self.lib or lib()).wref_frames(*self._ptrs(), C.byref(self.cfg), k))


def seed(cfg: RefConfig, like: np.ndarray | None = None) -> np.ndarray:
    """The reference galaxy of cfg.count bodies (raw 32-byte records)."""
    out = np.zeros(cfg.count * 8, np.float32) if like is None else np.empty_like(like)
    _ok(lib().wref_seed(out.ctypes.data_as(C.c_void_p), C.byref(cfg)))
    return out


def _ok(status: int) -> None:
    if status != 0:
        raise RuntimeError("the translated shader lacks an entry point the harness dispatches")
