"""ctypes bindings for the CPU oracle (test infrastructure only).

Only the tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` import this module.  It wraps ``rfmm_oracle.c``, the CPU
restatement of the reference's compute passes (src/rainbow_fmm.wgsl:100-771,
frame order native/main.rs:411-421), and exposes numpy views of the three
reference buffer layouts: Particle 32 B, Moment 16 B, Field 48 B.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_oracle

PARTICLE_DTYPE = np.dtype([("pos", "<f4", 3), ("hue", "<f4"), ("vel", "<f4", 3), ("exc", "<f4")])
MOMENT_DTYPE = np.dtype([("count", "<u4"), ("sum", "<i4", 3)])
FIELD_DTYPE = np.dtype([("a", "<f4", 4), ("j0", "<f4", 4), ("j1", "<f4", 4)])
assert PARTICLE_DTYPE.itemsize == 32 and MOMENT_DTYPE.itemsize == 16 and FIELD_DTYPE.itemsize == 48

ADAPTIVE_LEAF_CAPACITY = 16
WORLD_HALF_EXTENT = np.float32(1.6)


class OParams(C.Structure):
    """Compute-relevant subset of `struct Params` (src/rainbow_fmm.wgsl:18-50)."""

    _fields_ = [
        ("n", C.c_uint32),
        ("depth", C.c_uint32),
        ("scale", C.c_float),
        ("dt", C.c_float),
        ("gravity", C.c_float),
        ("softening", C.c_float),
        ("speed", C.c_float),
        ("control_point", C.c_float * 4),
        ("control_axis_mode", C.c_float * 4),
        ("control_strength", C.c_float),
        ("control_radius", C.c_float),
        ("near_mode", C.c_uint32),  # 0 reference near field, 1 exact P2P
    ]


class ORenderParams(C.Structure):
    """Camera and image parameters of the headless render (the solver's rfmm_render_params)."""

    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("instances", C.c_uint32),
                ("yaw", C.c_float), ("pitch", C.c_float), ("zoom", C.c_float),
                ("point_size", C.c_float), ("exposure", C.c_float)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        L = C.CDLL(path)
        u32, f32, vp = C.c_uint32, C.c_float, C.c_void_p
        P = C.POINTER(OParams)
        sig = {
            "oracle_level_cells": (u32, [u32]),
            "oracle_level_offset": (u32, [u32]),
            "oracle_total_cells": (u32, [u32]),
            "oracle_depth_for_particles": (u32, [u32]),
            "oracle_fixed_point_scale": (f32, [u32]),
            "oracle_clamp_particle_count": (u32, [u32]),
            "oracle_linear_work_bound": (C.c_uint64, [u32, u32]),
            "oracle_clear": (None, [vp, u32]),
            "oracle_deposit": (None, [vp, vp, P]),
            "oracle_upward": (None, [vp, P]),
            "oracle_m2l_all": (None, [vp, vp, P]),
            "oracle_near_all": (None, [vp, vp, P]),
            "oracle_downward": (None, [vp, vp, P]),
            "oracle_integrate": (None, [vp, vp, vp, P]),
            "oracle_initialize": (None, [vp, P]),
            "oracle_solve_fields": (None, [vp, vp, vp, P]),
            "oracle_step": (None, [vp, vp, vp, P, u32]),
            "oracle_fnv1a": (u32, [vp, C.c_size_t]),
            "oracle_m2l_targets": (u32, [vp, P, vp, u32]),
            "oracle_sample_cells": (None, [vp, vp, P, vp]),
            "oracle_leaf_of": (u32, [vp, u32]),
            "oracle_direct_sum_f64": (None, [vp, u32, vp, u32, C.c_double, C.c_double, vp]),
            "oracle_accelerations": (None, [vp, vp, vp, P, vp]),
            "oracle_set_threads": (C.c_int, [C.c_int]),
            "oracle_render": (None, [vp, P, C.POINTER(ORenderParams), vp, vp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.c_void_p)


def plan(n: int):
    """Unclamped planner (src/lib.rs:45-69), as the native harness uses it."""
    L = lib()
    depth = L.oracle_depth_for_particles(n)
    return depth, L.oracle_total_cells(depth), L.oracle_fixed_point_scale(n)


def make_params(n, dt=0.0009, gravity=0.34, softening=0.012, speed=1.0, depth=None, scale=None,
                control_point=(0.0, 0.0, 0.0, 0.0), control_axis_mode=(0.0, 0.0, 0.0, 0.0),
                control_strength=0.7, control_radius=0.22, near_mode=0) -> OParams:
    """Params with the native harness's defaults (native/main.rs:57-81)."""
    d, _, s = plan(n)
    p = OParams()
    p.n = n
    p.depth = d if depth is None else depth
    p.scale = s if scale is None else scale
    p.dt, p.gravity, p.softening, p.speed = dt, gravity, softening, speed
    p.control_point[:] = control_point
    p.control_axis_mode[:] = control_axis_mode
    p.control_strength, p.control_radius = control_strength, control_radius
    p.near_mode = near_mode
    return p


class OracleState:
    """Particle, moment and field buffers driven by the oracle passes."""

    def __init__(self, particles: np.ndarray, params: OParams):
        assert particles.dtype == PARTICLE_DTYPE
        self.params = params
        self.particles = np.ascontiguousarray(particles).copy()
        cells = lib().oracle_total_cells(params.depth)
        self.moments = np.zeros(cells, MOMENT_DTYPE)
        self.fields = np.zeros(cells, FIELD_DTYPE)  # wgpu zero-initialises

    def solve_fields(self):
        lib().oracle_solve_fields(_ptr(self.particles), _ptr(self.moments), _ptr(self.fields),
                                  C.byref(self.params))

    def step(self, steps: int = 1):
        lib().oracle_step(_ptr(self.particles), _ptr(self.moments), _ptr(self.fields),
                          C.byref(self.params), steps)

    def integrate(self):
        lib().oracle_integrate(_ptr(self.particles), _ptr(self.moments), _ptr(self.fields),
                               C.byref(self.params))

    def accelerations(self) -> np.ndarray:
        """FMM acceleration of every body from the current moments/fields."""
        out = np.zeros((self.params.n, 3), np.float32)
        lib().oracle_accelerations(_ptr(self.particles), _ptr(self.moments), _ptr(self.fields),
                                   C.byref(self.params), _ptr(out))
        return out

    def m2l_targets(self) -> np.ndarray:
        cap = len(self.moments)
        out = np.zeros(cap, np.uint32)
        k = lib().oracle_m2l_targets(_ptr(self.moments), C.byref(self.params), _ptr(out), cap)
        return out[:k].copy()

    def sample_cells(self) -> np.ndarray:
        out = np.zeros(self.params.n, np.uint32)
        lib().oracle_sample_cells(_ptr(self.particles), _ptr(self.moments), C.byref(self.params),
                                  _ptr(out))
        return out


def initialize(n: int, params: OParams | None = None) -> np.ndarray:
    """The reference's seeded galaxy (src/rainbow_fmm.wgsl:232-374)."""
    p = params or make_params(n)
    out = np.zeros(n, PARTICLE_DTYPE)
    lib().oracle_initialize(_ptr(out), C.byref(p))
    return out


def fnv1a(buf: np.ndarray) -> int:
    """FNV-1a over the buffer's bytes (native/main.rs:152-163)."""
    b = np.ascontiguousarray(buf)
    return int(lib().oracle_fnv1a(_ptr(b), b.nbytes))


def direct_sum_f64(particles: np.ndarray, targets: np.ndarray, gravity: float, eps: float):
    """FP64 softened direct sum on the given targets, equal masses 1/N."""
    t = np.ascontiguousarray(targets, dtype=np.uint32)
    out = np.zeros((len(t), 3), np.float64)
    p = np.ascontiguousarray(particles)
    lib().oracle_direct_sum_f64(_ptr(p), len(p), _ptr(t), len(t), gravity, eps, _ptr(out))
    return out


def render(particles: np.ndarray, params: OParams, width=1280, height=720, instances=0, yaw=-0.18,
           pitch=-0.14, zoom=1.78, point_size=5.0, exposure=1.0):
    """RGBA8 image (height, width, 4) and the fixed-point accumulation
    ((height+1)//2, (width+1)//2, 4) of the display passes (wgsl:780-1009)."""
    r = ORenderParams(width, height, instances, yaw, pitch, zoom, point_size, exposure)
    img = np.zeros((height, width, 4), np.uint8)
    acc = np.zeros(((height + 1) // 2, (width + 1) // 2, 4), np.uint64)
    p = np.ascontiguousarray(particles)
    lib().oracle_render(_ptr(p), C.byref(params), C.byref(r), _ptr(img), _ptr(acc))
    return img, acc


def set_threads(n: int) -> int:
    return lib().oracle_set_threads(n)
