"""Python host mirror of the GB300 FMM solver C ABI.

The reference drives its solver from JavaScript/Rust host code that calls the
planner exports (src/lib.rs:88-157) and encodes WGSL passes
(app.js:525-648, native/main.rs:353-421).  This module binds the same planner
exports and the `rfmm_*` dispatch-sequence ABI of ``lib/librfmm.so`` through
ctypes, with numpy views of the reference buffer layouts.  It is what the
tests, the bench and a Python host call; there is no fallback: if the shared
library is missing, importing the solver raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB_PATH = os.environ.get("RFMM_LIB") or os.path.join(PKG, "lib", "librfmm.so")

PARTICLE_DTYPE = np.dtype([("pos", "<f4", 3), ("hue", "<f4"), ("vel", "<f4", 3), ("exc", "<f4")])
MOMENT_DTYPE = np.dtype([("count", "<u4"), ("sum", "<i4", 3)])
FIELD_DTYPE = np.dtype([("a", "<f4", 4), ("j0", "<f4", 4), ("j1", "<f4", 4)])

RFMM_OK = 0
RFMM_ERR_INVALID = -1
RFMM_ERR_TIMEOUT = -5
STATUS = {
    0: "ok", -1: "invalid argument", -2: "CUDA runtime error", -3: "device memory exhausted",
    -4: "call out of order", -5: "kernel wait timed out", -6: "no sm_103 CUDA device",
    -7: "kernel reported an error", -8: "request exceeds the memory budget",
}
BUF_PARTICLES, BUF_MOMENTS, BUF_FIELDS = 0, 1, 2
NEAR_REFERENCE, NEAR_P2P = 0, 1
FLOAT_EXACT, FLOAT_FAST = 0, 1
PHASES = ("clear", "deposit", "upward", "m2l", "downward", "near", "integrate")

# Every symbol the headers in include/ declare, with its ctypes signature.
_u32, _f32, _vp, _sz, _i = C.c_uint32, C.c_float, C.c_void_p, C.c_size_t, C.c_int


class Params(C.Structure):
    """`rfmm_params` (include/rfmm.h)."""

    _fields_ = [
        ("dt", C.c_float),
        ("gravity", C.c_float),
        ("softening", C.c_float),
        ("speed", C.c_float),
        ("control_point", C.c_float * 4),
        ("control_axis_mode", C.c_float * 4),
        ("control_strength", C.c_float),
        ("control_radius", C.c_float),
        ("fixed_point_scale", C.c_float),
        ("depth", C.c_uint32),
    ]


class ServerConfig(C.Structure):
    _fields_ = [("memory_budget_bytes", C.c_uint64), ("max_bodies", C.c_uint32),
                ("max_slots", C.c_uint32), ("max_chunk_steps", C.c_uint32),
                ("staging_bytes", C.c_uint64), ("float_mode", C.c_uint32), ("timeline", C.c_uint32)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_uint64), ("completed", C.c_uint64), ("queued", C.c_uint64),
                ("in_flight", C.c_uint64), ("slots", C.c_uint32), ("slot_capacity", C.c_uint32),
                ("device_bytes", C.c_uint64), ("p50_ms", C.c_double), ("p99_ms", C.c_double),
                ("mean_ms", C.c_double), ("max_ms", C.c_double),
                ("body_steps_per_s", C.c_double), ("body_steps", C.c_double),
                ("chunks", C.c_uint64), ("mean_active_slots", C.c_double),
                ("pageable_inputs", C.c_uint64), ("worker_gpu_wait_ms", C.c_double),
                ("worker_admit_ms", C.c_double), ("worker_lists_ms", C.c_double),
                ("worker_step_ms", C.c_double), ("worker_retire_ms", C.c_double),
                ("gpu_step_ms", C.c_double), ("gpu_between_ms", C.c_double)]


class Tuning(C.Structure):
    """`rfmm_tuning` (include/rfmm.h): launch shapes; results never depend on them."""

    _fields_ = [("upward_ctas_per_sm", C.c_uint32), ("m2l_ctas_per_sm", C.c_uint32),
                ("l2l_ctas_per_sm", C.c_uint32), ("integrate_ctas_per_sm", C.c_uint32),
                ("integrate_dynamic", C.c_uint32), ("resort_interval", C.c_uint32),
                ("graph_steps", C.c_uint32), ("pdl", C.c_uint32), ("m2l_compact", C.c_uint32),
                ("m2l_lanes", C.c_uint32), ("l2l_lanes", C.c_uint32), ("upward_warps", C.c_uint32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Timeline(C.Structure):
    """`rfmm_timeline` (include/rfmm.h): step kernels as they ran inside the graphs."""

    _fields_ = [("steps", C.c_uint32), ("launches", C.c_uint32 * 6), ("busy_ms", C.c_double * 6),
                ("gap_ms", C.c_double * 6), ("span_ms", C.c_double)]

    def as_dict(self):
        kinds = KERNEL_KINDS
        return {"steps": self.steps, "span_ms": self.span_ms,
                "kinds": {k: {"launches": self.launches[i], "busy_ms": self.busy_ms[i],
                              "gap_ms": self.gap_ms[i]} for i, k in enumerate(kinds)}}


class Diagnostics(C.Structure):
    _fields_ = [("kinetic", C.c_double), ("potential", C.c_double), ("total", C.c_double),
                ("momentum", C.c_double * 3), ("angular_momentum", C.c_double * 3)]


class RenderParams(C.Structure):
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("instances", C.c_uint32),
                ("yaw", C.c_float), ("pitch", C.c_float), ("zoom", C.c_float),
                ("point_size", C.c_float), ("exposure", C.c_float)]


class Plan(C.Structure):
    _fields_ = [("particles", C.c_uint32), ("depth", C.c_uint32), ("cells", C.c_uint32),
                ("fixed_point_scale", C.c_float)]


_P = C.POINTER(Params)
SIGNATURES = {
    # include/rainbow_fmm.h
    "rainbow_api_version": (_u32, []),
    "rainbow_shader_ptr": (_vp, []),
    "rainbow_shader_len": (_sz, []),
    "rainbow_algorithm_ptr": (_vp, []),
    "rainbow_algorithm_len": (_sz, []),
    "rainbow_depth_for_particles": (_u32, [_u32]),
    "rainbow_level_cells": (_u32, [_u32]),
    "rainbow_level_offset": (_u32, [_u32]),
    "rainbow_total_cells": (_u32, [_u32]),
    "rainbow_clamp_particle_count": (_u32, [_u32]),
    "rainbow_fixed_point_scale": (_f32, [_u32]),
    "rainbow_linear_work_lo": (_u32, [_u32, _u32]),
    "rainbow_plan_depth_unclamped": (_u32, [_u32]),
    "rainbow_plan_scale_unclamped": (_f32, [_u32]),
    "rainbow_plan_work_bound_unclamped": (C.c_uint64, [_u32, _u32]),
    # include/rfmm.h
    "rfmm_default_params": (None, [_P]),
    "rfmm_status_string": (C.c_char_p, [_i]),
    "rfmm_create": (_i, [_u32, _P, C.POINTER(_vp)]),
    "rfmm_destroy": (_i, [_vp]),
    "rfmm_set_stream": (_i, [_vp, _vp]),
    "rfmm_get_plan": (_i, [_vp, C.POINTER(Plan)]),
    "rfmm_set_params": (_i, [_vp, _P]),
    "rfmm_upload_particles": (_i, [_vp, _vp, _sz]),
    "rfmm_upload_particles_device": (_i, [_vp, _vp, _sz]),
    "rfmm_seed_galaxy": (_i, [_vp]),
    "rfmm_solve_fields": (_i, [_vp]),
    "rfmm_step": (_i, [_vp, _u32]),
    "rfmm_sync": (_i, [_vp]),
    "rfmm_download": (_i, [_vp, _i, _vp, _sz]),
    "rfmm_download_device": (_i, [_vp, _i, _vp, _sz]),
    "rfmm_digest": (_i, [_vp, _i, C.POINTER(_u32)]),
    "rfmm_phase_times": (_i, [_vp, C.POINTER(_f32)]),
    "rfmm_check_finite": (_i, [_vp, _u32, C.POINTER(_u32), C.POINTER(_f32)]),
    "rfmm_set_resort_interval": (_i, [_vp, _u32]),
    "rfmm_set_near_mode": (_i, [_vp, _u32]),
    "rfmm_set_float_mode": (_i, [_vp, _u32]),
    "rfmm_batch_set_float_mode": (_i, [_vp, _u32]),
    "rfmm_device_error": (_i, [_vp, C.POINTER(_u32), C.POINTER(_u32)]),
    "rfmm_profile_steps": (_i, [_vp, _u32, C.POINTER(_f32), C.POINTER(_u32)]),
    "rfmm_launch_count": (_i, [_vp, C.POINTER(C.c_uint64)]),
    "rfmm_set_timeline": (_i, [_vp, _u32]),
    "rfmm_get_timeline": (_i, [_vp, C.POINTER(Timeline)]),
    "rfmm_batch_set_timeline": (_i, [_vp, _u32]),
    "rfmm_batch_get_timeline": (_i, [_vp, C.POINTER(Timeline)]),
    "rfmm_solve_fields_noalloc": (_i, [_vp, _u32, _P, _vp, _vp, _vp]),
    "rfmm_noalloc_device_error": (_i, [C.POINTER(_u32), C.POINTER(_u32), _vp]),
    "rfmm_batch_create": (_i, [_u32, C.POINTER(_u32), _P, C.POINTER(_vp)]),
    "rfmm_batch_destroy": (_i, [_vp]),
    "rfmm_batch_set_stream": (_i, [_vp, _vp]),
    "rfmm_batch_get_plan": (_i, [_vp, _u32, C.POINTER(Plan)]),
    "rfmm_batch_set_params": (_i, [_vp, _u32, _P]),
    "rfmm_batch_upload": (_i, [_vp, _u32, _vp, _sz]),
    "rfmm_batch_upload_device": (_i, [_vp, _u32, _vp, _sz]),
    "rfmm_batch_upload_device_all": (_i, [_vp, _vp]),
    "rfmm_batch_download_all": (_i, [_vp, _i, _vp]),
    "rfmm_check_wait_timeout": (_i, [_vp, _u32]),
    "rfmm_batch_seed_galaxy": (_i, [_vp, _u32]),
    "rfmm_batch_commit": (_i, [_vp]),
    "rfmm_batch_solve_fields": (_i, [_vp]),
    "rfmm_batch_step": (_i, [_vp, _u32]),
    "rfmm_batch_sync": (_i, [_vp]),
    "rfmm_batch_download": (_i, [_vp, _u32, _i, _vp, _sz]),
    "rfmm_batch_download_device": (_i, [_vp, _u32, _i, _vp, _sz]),
    "rfmm_batch_digest": (_i, [_vp, _u32, _i, C.POINTER(_u32)]),
    "rfmm_batch_launch_count": (_i, [_vp, C.POINTER(C.c_uint64)]),
    "rfmm_batch_profile_steps": (_i, [_vp, _u32, C.POINTER(_f32), C.POINTER(_u32)]),
    "rfmm_batch_set_resort_interval": (_i, [_vp, _u32]),
    "rfmm_batch_set_near_mode": (_i, [_vp, _u32]),
    "rfmm_accelerations": (_i, [_vp, _vp, _sz]),
    "rfmm_force_error": (_i, [_vp, _u32, C.c_uint64, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "rfmm_get_diagnostics": (_i, [_vp, C.POINTER(Diagnostics)]),
    "rfmm_batch_force_error": (_i, [_vp, _u32, _u32, C.c_uint64, C.POINTER(C.c_double),
                                    C.POINTER(C.c_double)]),
    "rfmm_default_render_params": (None, [C.POINTER(RenderParams)]),
    "rfmm_render": (_i, [_vp, C.POINTER(RenderParams), _vp, _sz]),
    "rfmm_render_device": (_i, [_vp, C.POINTER(RenderParams), _vp, _sz]),
    "rfmm_get_tuning": (_i, [_vp, C.POINTER(Tuning)]),
    "rfmm_set_tuning": (_i, [_vp, C.POINTER(Tuning)]),
    "rfmm_autotune": (_i, [_vp, _u32, C.POINTER(Tuning)]),
    "rfmm_batch_get_tuning": (_i, [_vp, C.POINTER(Tuning)]),
    "rfmm_batch_set_tuning": (_i, [_vp, C.POINTER(Tuning)]),
    "rfmm_batch_autotune": (_i, [_vp, _u32, C.POINTER(Tuning)]),
    "rfmm_server_create": (_i, [C.POINTER(ServerConfig), C.POINTER(_vp)]),
    "rfmm_server_destroy": (_i, [_vp]),
    "rfmm_server_submit": (_i, [_vp, _vp, _u32, _P, _u32, C.POINTER(C.c_uint64)]),
    "rfmm_server_submit_at": (_i, [_vp, _vp, _u32, _P, _u32, C.c_double, C.POINTER(C.c_uint64)]),
    "rfmm_server_clock": (_i, [C.POINTER(C.c_double)]),
    "rfmm_server_status": (_i, [_vp, C.c_uint64, C.POINTER(_i)]),
    "rfmm_server_wait": (_i, [_vp, C.c_uint64, _u32]),
    "rfmm_server_result": (_i, [_vp, C.c_uint64, _vp, _sz]),
    "rfmm_server_get_stats": (_i, [_vp, C.POINTER(ServerStats)]),
    "rfmm_server_get_timeline": (_i, [_vp, C.POINTER(Timeline)]),
}
KERNEL_KINDS = ("upward", "m2l", "l2l_near", "integrate", "resort", "near_p2p")

_lib = None


class RFMMError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        super().__init__("%s failed: %s (%d)" % (what, STATUS.get(status, "unknown"), status))


def lib() -> C.CDLL:
    """Load ``lib/librfmm.so``; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError("librfmm.so is not built (%s); run the package build first" % LIB_PATH)
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(status: int, what: str) -> None:
    if status != RFMM_OK:
        raise RFMMError(status, what)


def default_params(**kw) -> Params:
    p = Params()
    lib().rfmm_default_params(C.byref(p))
    for k, v in kw.items():
        if k in ("control_point", "control_axis_mode"):
            getattr(p, k)[:] = v
        else:
            setattr(p, k, v)
    return p


def default_render_params(**kw) -> RenderParams:
    p = RenderParams()
    lib().rfmm_default_render_params(C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    return p


# ------------------------------------------------------------------ planner

def api_version() -> int:
    return lib().rainbow_api_version()


def shader_text() -> str:
    L = lib()
    return C.string_at(L.rainbow_shader_ptr(), L.rainbow_shader_len()).decode()


def algorithm() -> str:
    L = lib()
    return C.string_at(L.rainbow_algorithm_ptr(), L.rainbow_algorithm_len()).decode()


def plan_unclamped(n: int):
    """(depth, cells, scale) as the native harness plans it (native/main.rs:89-92)."""
    L = lib()
    d = L.rainbow_plan_depth_unclamped(n)
    return d, L.rainbow_level_offset(d + 1), L.rainbow_plan_scale_unclamped(n)


# ------------------------------------------------------------------- solver

def solve_fields_noalloc(particles_ptr: int, n: int, params: Params | None, moments_ptr: int,
                         fields_ptr: int, stream_ptr: int | None = None) -> None:
    """Allocation-free field solve on caller-owned device buffers (n <= 131072)."""
    _check(lib().rfmm_solve_fields_noalloc(particles_ptr, n, C.byref(params) if params else None,
                                           moments_ptr, fields_ptr, stream_ptr or None),
           "rfmm_solve_fields_noalloc")


def noalloc_device_error(stream_ptr: int | None = None):
    """(status, code, info) of the last allocation-free solve on this device,
    read after the work queued on the stream."""
    code, info = C.c_uint32(), C.c_uint32()
    st = lib().rfmm_noalloc_device_error(C.byref(code), C.byref(info), stream_ptr or None)
    return st, code.value, info.value


class Solver:
    """One scene of N bodies resident on the GPU (the `rfmm_*` handle)."""

    def __init__(self, n: int, params: Params | None = None, **kw):
        if params is None:
            params = default_params(**kw)
        self._h = C.c_void_p()
        _check(lib().rfmm_create(n, C.byref(params), C.byref(self._h)), "rfmm_create")
        self.n = n
        plan = Plan()
        _check(lib().rfmm_get_plan(self._h, C.byref(plan)), "rfmm_get_plan")
        self.depth, self.cells, self.scale = plan.depth, plan.cells, plan.fixed_point_scale

    def close(self):
        if self._h:
            lib().rfmm_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def handle(self):
        return self._h

    def set_params(self, params: Params):
        _check(lib().rfmm_set_params(self._h, C.byref(params)), "rfmm_set_params")

    def set_stream(self, stream_ptr: int | None):
        _check(lib().rfmm_set_stream(self._h, stream_ptr or None), "rfmm_set_stream")

    def upload(self, particles: np.ndarray):
        a = np.ascontiguousarray(particles)
        assert a.dtype == PARTICLE_DTYPE and len(a) == self.n
        _check(lib().rfmm_upload_particles(self._h, a.ctypes.data, a.nbytes), "rfmm_upload_particles")

    def upload_device(self, ptr: int, nbytes: int):
        _check(lib().rfmm_upload_particles_device(self._h, ptr, nbytes), "rfmm_upload_particles_device")

    def upload_host_ptr(self, ptr: int, nbytes: int):
        _check(lib().rfmm_upload_particles(self._h, ptr, nbytes), "rfmm_upload_particles")

    def seed_galaxy(self):
        _check(lib().rfmm_seed_galaxy(self._h), "rfmm_seed_galaxy")

    def solve_fields(self):
        _check(lib().rfmm_solve_fields(self._h), "rfmm_solve_fields")

    def step(self, steps: int = 1):
        _check(lib().rfmm_step(self._h, steps), "rfmm_step")

    def sync(self):
        _check(lib().rfmm_sync(self._h), "rfmm_sync")

    def set_resort_interval(self, steps: int):
        _check(lib().rfmm_set_resort_interval(self._h, steps), "rfmm_set_resort_interval")

    def set_near_mode(self, mode: int):
        _check(lib().rfmm_set_near_mode(self._h, mode), "rfmm_set_near_mode")

    def set_float_mode(self, mode: int):
        _check(lib().rfmm_set_float_mode(self._h, mode), "rfmm_set_float_mode")

    def download(self, which: int = BUF_PARTICLES) -> np.ndarray:
        dtype, count = {BUF_PARTICLES: (PARTICLE_DTYPE, self.n), BUF_MOMENTS: (MOMENT_DTYPE, self.cells),
                        BUF_FIELDS: (FIELD_DTYPE, self.cells)}[which]
        out = np.empty(count, dtype)
        _check(lib().rfmm_download(self._h, which, out.ctypes.data, out.nbytes), "rfmm_download")
        return out

    def check_wait_timeout(self, polls: int = 1024) -> int:
        """Run the bounded-wait self-check; returns the status code (ERR_TIMEOUT expected)."""
        return lib().rfmm_check_wait_timeout(self._h, polls)

    def download_host_ptr(self, which: int, ptr: int, nbytes: int):
        _check(lib().rfmm_download(self._h, which, ptr, nbytes), "rfmm_download")

    def download_device(self, which: int, ptr: int, nbytes: int):
        _check(lib().rfmm_download_device(self._h, which, ptr, nbytes), "rfmm_download_device")

    def particles(self) -> np.ndarray:
        return self.download(BUF_PARTICLES)

    def moments(self) -> np.ndarray:
        return self.download(BUF_MOMENTS)

    def fields(self) -> np.ndarray:
        return self.download(BUF_FIELDS)

    def digest(self, which: int) -> int:
        out = C.c_uint32()
        _check(lib().rfmm_digest(self._h, which, C.byref(out)), "rfmm_digest")
        return out.value

    def phase_times(self) -> dict:
        ms = (C.c_float * 7)()
        _check(lib().rfmm_phase_times(self._h, ms), "rfmm_phase_times")
        return dict(zip(PHASES, list(ms)))

    def check_finite(self, probe: int = 8192):
        bad, mx = C.c_uint32(), C.c_float()
        _check(lib().rfmm_check_finite(self._h, probe, C.byref(bad), C.byref(mx)), "rfmm_check_finite")
        return bad.value, mx.value

    def profile_steps(self, steps: int):
        """Per-kernel-kind device ms and launch counts over `steps` frames."""
        ms = (C.c_float * len(KERNEL_KINDS))()
        cnt = (C.c_uint32 * len(KERNEL_KINDS))()
        _check(lib().rfmm_profile_steps(self._h, steps, ms, cnt), "rfmm_profile_steps")
        return {k: (ms[i], cnt[i]) for i, k in enumerate(KERNEL_KINDS)}

    def launch_count(self) -> int:
        out = C.c_uint64()
        _check(lib().rfmm_launch_count(self._h, C.byref(out)), "rfmm_launch_count")
        return out.value

    def set_timeline(self, on: bool):
        _check(lib().rfmm_set_timeline(self._h, 1 if on else 0), "rfmm_set_timeline")

    def timeline(self) -> dict:
        t = Timeline()
        _check(lib().rfmm_get_timeline(self._h, C.byref(t)), "rfmm_get_timeline")
        return t.as_dict()

    def accelerations(self) -> np.ndarray:
        """(N, 4) float32: FMM ax, ay, az, phi of the current positions (caller order)."""
        out = np.empty((self.n, 4), np.float32)
        _check(lib().rfmm_accelerations(self._h, out.ctypes.data, out.nbytes), "rfmm_accelerations")
        return out

    def force_error(self, targets: int = 4096, seed: int = 1):
        rms, mx = C.c_double(), C.c_double()
        _check(lib().rfmm_force_error(self._h, targets, seed, C.byref(rms), C.byref(mx)),
               "rfmm_force_error")
        return rms.value, mx.value

    def render(self, **kw) -> np.ndarray:
        """(height, width, 4) uint8 image of the current bodies (row 0 at the top)."""
        p = default_render_params(**kw)
        out = np.empty((p.height, p.width, 4), np.uint8)
        _check(lib().rfmm_render(self._h, C.byref(p), out.ctypes.data, out.nbytes), "rfmm_render")
        return out

    def render_device(self, params, device_ptr, nbytes):
        _check(lib().rfmm_render_device(self._h, C.byref(params), device_ptr, nbytes),
               "rfmm_render_device")

    def diagnostics(self) -> dict:
        d = Diagnostics()
        _check(lib().rfmm_get_diagnostics(self._h, C.byref(d)), "rfmm_get_diagnostics")
        return {"kinetic": d.kinetic, "potential": d.potential, "total": d.total,
                "momentum": list(d.momentum), "angular_momentum": list(d.angular_momentum)}

    def tuning(self) -> Tuning:
        t = Tuning()
        _check(lib().rfmm_get_tuning(self._h, C.byref(t)), "rfmm_get_tuning")
        return t

    def set_tuning(self, t: Tuning):
        _check(lib().rfmm_set_tuning(self._h, C.byref(t)), "rfmm_set_tuning")

    def autotune(self, steps_per_trial: int = 20) -> Tuning:
        t = Tuning()
        _check(lib().rfmm_autotune(self._h, steps_per_trial, C.byref(t)), "rfmm_autotune")
        return t

    def device_error(self):
        code, info = C.c_uint32(), C.c_uint32()
        _check(lib().rfmm_device_error(self._h, C.byref(code), C.byref(info)), "rfmm_device_error")
        return code.value, info.value


class Batch:
    """Many independent scenes stepped together (the `rfmm_batch_*` handle)."""

    def __init__(self, sizes, params=None):
        sizes = [int(x) for x in sizes]
        arr = (C.c_uint32 * len(sizes))(*sizes)
        prm = None
        if params is not None:
            prm = (Params * len(sizes))(*params)
        self._h = C.c_void_p()
        _check(lib().rfmm_batch_create(len(sizes), arr, prm, C.byref(self._h)), "rfmm_batch_create")
        self.sizes = sizes
        self.plans = []
        for i in range(len(sizes)):
            plan = Plan()
            _check(lib().rfmm_batch_get_plan(self._h, i, C.byref(plan)), "rfmm_batch_get_plan")
            self.plans.append((plan.depth, plan.cells, plan.fixed_point_scale))

    def close(self):
        if self._h:
            lib().rfmm_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_stream(self, stream_ptr):
        _check(lib().rfmm_batch_set_stream(self._h, stream_ptr or None), "rfmm_batch_set_stream")

    def set_resort_interval(self, steps):
        _check(lib().rfmm_batch_set_resort_interval(self._h, steps), "rfmm_batch_set_resort_interval")

    def set_near_mode(self, mode):
        _check(lib().rfmm_batch_set_near_mode(self._h, mode), "rfmm_batch_set_near_mode")

    def set_float_mode(self, mode):
        _check(lib().rfmm_batch_set_float_mode(self._h, mode), "rfmm_batch_set_float_mode")

    def upload(self, scene, particles):
        a = np.ascontiguousarray(particles)
        assert a.dtype == PARTICLE_DTYPE and len(a) == self.sizes[scene]
        _check(lib().rfmm_batch_upload(self._h, scene, a.ctypes.data, a.nbytes), "rfmm_batch_upload")

    def upload_device(self, scene, ptr, nbytes):
        _check(lib().rfmm_batch_upload_device(self._h, scene, ptr, nbytes), "rfmm_batch_upload_device")

    def download_all_into(self, which, ptrs):
        """Every scene's buffer `which` into host addresses ptrs[s], one synchronisation."""
        assert len(ptrs) == len(self.sizes)
        arr = (C.c_void_p * len(ptrs))(*ptrs)
        _check(lib().rfmm_batch_download_all(self._h, which, arr), "rfmm_batch_download_all")

    def upload_device_all(self, ptrs):
        """Every scene at once: ptrs[s] is the device address of scene s's bodies."""
        assert len(ptrs) == len(self.sizes)
        arr = (C.c_void_p * len(ptrs))(*ptrs)
        _check(lib().rfmm_batch_upload_device_all(self._h, arr), "rfmm_batch_upload_device_all")

    def commit(self):
        _check(lib().rfmm_batch_commit(self._h), "rfmm_batch_commit")

    def solve_fields(self):
        _check(lib().rfmm_batch_solve_fields(self._h), "rfmm_batch_solve_fields")

    def step(self, steps=1):
        _check(lib().rfmm_batch_step(self._h, steps), "rfmm_batch_step")

    def sync(self):
        _check(lib().rfmm_batch_sync(self._h), "rfmm_batch_sync")

    def download(self, scene, which=BUF_PARTICLES):
        depth, cells, _ = self.plans[scene]
        dtype, count = {BUF_PARTICLES: (PARTICLE_DTYPE, self.sizes[scene]),
                        BUF_MOMENTS: (MOMENT_DTYPE, cells), BUF_FIELDS: (FIELD_DTYPE, cells)}[which]
        out = np.empty(count, dtype)
        _check(lib().rfmm_batch_download(self._h, scene, which, out.ctypes.data, out.nbytes),
               "rfmm_batch_download")
        return out

    def digest(self, scene, which):
        out = C.c_uint32()
        _check(lib().rfmm_batch_digest(self._h, scene, which, C.byref(out)), "rfmm_batch_digest")
        return out.value

    def launch_count(self):
        out = C.c_uint64()
        _check(lib().rfmm_batch_launch_count(self._h, C.byref(out)), "rfmm_batch_launch_count")
        return out.value

    def set_timeline(self, on):
        _check(lib().rfmm_batch_set_timeline(self._h, 1 if on else 0), "rfmm_batch_set_timeline")

    def timeline(self):
        t = Timeline()
        _check(lib().rfmm_batch_get_timeline(self._h, C.byref(t)), "rfmm_batch_get_timeline")
        return t.as_dict()

    def force_error(self, scene, targets=1024, seed=1):
        rms, mx = C.c_double(), C.c_double()
        _check(lib().rfmm_batch_force_error(self._h, scene, targets, seed, C.byref(rms), C.byref(mx)),
               "rfmm_batch_force_error")
        return rms.value, mx.value

    def tuning(self):
        t = Tuning()
        _check(lib().rfmm_batch_get_tuning(self._h, C.byref(t)), "rfmm_batch_get_tuning")
        return t

    def set_tuning(self, t):
        _check(lib().rfmm_batch_set_tuning(self._h, C.byref(t)), "rfmm_batch_set_tuning")

    def autotune(self, steps_per_trial=10):
        t = Tuning()
        _check(lib().rfmm_batch_autotune(self._h, steps_per_trial, C.byref(t)), "rfmm_batch_autotune")
        return t

    def profile_steps(self, steps):
        ms = (C.c_float * len(KERNEL_KINDS))()
        cnt = (C.c_uint32 * len(KERNEL_KINDS))()
        _check(lib().rfmm_batch_profile_steps(self._h, steps, ms, cnt), "rfmm_batch_profile_steps")
        return {k: (ms[i], cnt[i]) for i, k in enumerate(KERNEL_KINDS)}


class Server:
    """Continuous-batching solve server (the `rfmm_server_*` handle)."""

    def __init__(self, max_bodies, memory_budget_bytes=8 << 30, max_slots=0, max_chunk_steps=0,
                 staging_bytes=0, float_mode=FLOAT_EXACT, timeline=False):
        cfg = ServerConfig(memory_budget_bytes, max_bodies, max_slots, max_chunk_steps,
                           staging_bytes, float_mode, 1 if timeline else 0)
        self._h = C.c_void_p()
        _check(lib().rfmm_server_create(C.byref(cfg), C.byref(self._h)), "rfmm_server_create")
        self._n = {}

    def close(self):
        if self._h:
            lib().rfmm_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def submit(self, particles, steps, params=None):
        a = np.ascontiguousarray(particles)
        assert a.dtype == PARTICLE_DTYPE
        rid = C.c_uint64()
        _check(lib().rfmm_server_submit(self._h, a.ctypes.data, len(a),
                                        C.byref(params) if params is not None else None, steps,
                                        C.byref(rid)), "rfmm_server_submit")
        self._n[rid.value] = len(a)
        return rid.value

    def submit_at(self, particles, steps, params, arrival_s):
        """Submit with an explicit arrival time on the server clock (see clock())."""
        a = np.ascontiguousarray(particles)
        assert a.dtype == PARTICLE_DTYPE
        rid = C.c_uint64()
        _check(lib().rfmm_server_submit_at(self._h, a.ctypes.data, len(a),
                                           C.byref(params) if params is not None else None, steps,
                                           arrival_s, C.byref(rid)), "rfmm_server_submit_at")
        self._n[rid.value] = len(a)
        return rid.value

    @staticmethod
    def clock():
        t = C.c_double()
        _check(lib().rfmm_server_clock(C.byref(t)), "rfmm_server_clock")
        return t.value

    def status(self, rid):
        st = C.c_int()
        _check(lib().rfmm_server_status(self._h, rid, C.byref(st)), "rfmm_server_status")
        return st.value

    def wait(self, rid, timeout_ms=60000):
        _check(lib().rfmm_server_wait(self._h, rid, timeout_ms), "rfmm_server_wait")

    def result(self, rid):
        out = np.empty(self._n.pop(rid), PARTICLE_DTYPE)
        _check(lib().rfmm_server_result(self._h, rid, out.ctypes.data, out.nbytes),
               "rfmm_server_result")
        return out

    def stats(self):
        st = ServerStats()
        _check(lib().rfmm_server_get_stats(self._h, C.byref(st)), "rfmm_server_get_stats")
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def timeline(self) -> dict:
        """The step kernels' in-graph timeline (server created with timeline=True)."""
        t = Timeline()
        _check(lib().rfmm_server_get_timeline(self._h, C.byref(t)), "rfmm_server_get_timeline")
        return t.as_dict()
