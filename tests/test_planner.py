"""Planner known-answer tests: the reference's own unit tests (src/lib.rs:163-217)
run against the library's C ABI (include/rainbow_fmm.h) and the oracle's
restatement, plus the exported functions' clamping (src/lib.rs:113-157)."""
import math

import numpy as np
import pytest

U32_MAX = 0xFFFFFFFF
F32_HALF = float(np.float32(1.6))


@pytest.fixture(scope="module")
def L(rfmm_mod):
    return rfmm_mod.lib()


def py_scale(n):
    worst = n * F32_HALF
    return float(np.float32(2.0 ** math.floor(math.log2(0.82 * 2147483647 / max(worst, 1.0)))))


def py_depth(n):
    target = -(-n // 8)
    d = 4
    while d < 6 and 8 ** d < target:
        d += 1
    return d


def test_octree_layout_is_contiguous(L, oracle_mod):  # lib.rs:164-172
    O = oracle_mod.lib()
    for level in range(0, 7):
        assert L.rainbow_level_offset(level) + L.rainbow_level_cells(level) == L.rainbow_level_offset(level + 1)
        assert O.oracle_level_offset(level) + O.oracle_level_cells(level) == O.oracle_level_offset(level + 1)
    assert L.rainbow_total_cells(6) == 299_593
    assert O.oracle_total_cells(6) == 299_593


def test_million_particle_plan_uses_depth_six(L, oracle_mod):  # lib.rs:175-179
    O = oracle_mod.lib()
    assert L.rainbow_plan_depth_unclamped(1 << 20) == 6
    assert L.rainbow_depth_for_particles(1 << 20) == 6
    assert O.oracle_depth_for_particles(1 << 20) == 6
    assert L.rainbow_level_cells(6) == 262_144
    assert L.rainbow_clamp_particle_count(U32_MAX) == 1 << 23
    assert O.oracle_clamp_particle_count(U32_MAX) == 1 << 23


def test_multi_million_plans_stay_cache_resident(L, oracle_mod):  # lib.rs:182-189
    O = oracle_mod.lib()
    for n in (1 << 21, 1 << 22, 1 << 23):
        assert L.rainbow_plan_depth_unclamped(n) == 6
        assert O.oracle_depth_for_particles(n) == 6
    assert L.rainbow_total_cells(6) == 299_593


def test_fixed_point_scale_stays_inside_i32(L, oracle_mod):  # lib.rs:192-203
    O = oracle_mod.lib()
    for n in (1 << 14, 1 << 20, 1 << 21, 1 << 22, 1 << 23):
        for scale in (L.rainbow_plan_scale_unclamped(n), O.oracle_fixed_point_scale(n)):
            worst = n * F32_HALF * scale
            assert worst < 2147483647, (n, worst)
            assert math.log2(scale) == int(math.log2(scale))


def test_work_bound_is_linear_for_a_fixed_depth(L, oracle_mod):  # lib.rs:206-210
    O = oracle_mod.lib()
    a = L.rainbow_plan_work_bound_unclamped(1 << 18, 6)
    b = L.rainbow_plan_work_bound_unclamped(1 << 19, 6)
    assert b - a == 3 * (1 << 18)
    assert O.oracle_linear_work_bound(1 << 19, 6) - O.oracle_linear_work_bound(1 << 18, 6) == 3 * (1 << 18)
    assert L.rainbow_linear_work_lo(1 << 19, 6) - L.rainbow_linear_work_lo(1 << 18, 6) == 3 * (1 << 18)


def test_shader_payload_is_present(rfmm_mod):  # lib.rs:213-217, payload = kernel source
    text = rfmm_mod.shader_text()
    assert "k_m2l" in text and "k_integrate" in text
    assert len(text) > 10_000


def test_api_version_and_algorithm(rfmm_mod):
    assert rfmm_mod.api_version() == 1
    assert rfmm_mod.algorithm() == "Sparse p=1 Cartesian FMM / BLDTT-inspired adaptive hierarchy"


def test_exported_functions_clamp_like_the_reference(L):  # lib.rs:113-157
    assert L.rainbow_level_cells(7) == 0 and L.rainbow_level_cells(6) == 8 ** 6
    assert L.rainbow_level_offset(8) == 0 and L.rainbow_level_offset(7) == (8 ** 7 - 1) // 7
    assert L.rainbow_total_cells(0) == 4681 and L.rainbow_total_cells(9) == 299_593
    assert L.rainbow_depth_for_particles(0) == 4           # clamped to 2^14
    assert L.rainbow_clamp_particle_count(5) == 1 << 14
    assert L.rainbow_fixed_point_scale(0) == py_scale(1 << 14)
    assert L.rainbow_fixed_point_scale(U32_MAX) == py_scale(1 << 23)
    assert L.rainbow_linear_work_lo(1 << 20, 2) == (3 * (1 << 20) + 199 * 4681) & U32_MAX


def test_plan_sweep_matches_python_restatement(L, oracle_mod):
    O = oracle_mod.lib()
    rng = np.random.default_rng(5)
    ns = sorted(set([1, 2, 7, 8, 9, 4095, 4096, 4097, 32768, 32769, 262144, 262145]
                    + rng.integers(1, 1 << 23, 2000).tolist()))
    for n in ns:
        assert L.rainbow_plan_depth_unclamped(n) == py_depth(n) == O.oracle_depth_for_particles(n), n
        assert L.rainbow_plan_scale_unclamped(n) == py_scale(n) == O.oracle_fixed_point_scale(n), n
