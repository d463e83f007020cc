"""Failure detection without a GPU fault: a bounded device wait that runs out
reports GBPT_ERR_TIMEOUT and leaves the context usable; device allocations
made to fail on the host give GBPT_ERR_OOM at every point of a renderer's
set-up, and the library works again once they succeed."""
import ctypes

import numpy as np
import pytest

from helpers import scene_arrays


def test_fault_injection_switch_without_gpu(gb):
    L = gb._native.load()
    assert L.gbpt_test_fail_allocations(5) == 0
    assert L.gbpt_test_fail_allocations(-1) == 0


@pytest.mark.gpu
def test_bounded_wait_runs_out_and_context_survives(gbdev):
    L = gbdev._native.load()
    ms = ctypes.c_double(0.0)
    st = L.gbpt_selftest_wait_timeout(ctypes.addressof(ms))
    assert st == 4, st  # GBPT_ERR_TIMEOUT
    assert "ran out" in L.gbpt_last_error_string().decode()
    assert 10.0 < ms.value < 60000.0, ms.value
    (v, t, m), cam = scene_arrays("cornell")
    s = gbdev.RTScene(v, t, m).build_bvh()
    img = gbdev.RTRenderer(32, 32, 0, gbdev.default_params()).render(s, cam)
    assert np.isfinite(img).all() and img.max() > 0


@pytest.mark.gpu
def test_failed_allocations_are_reported_and_recovered(gbdev):
    L = gbdev._native.load()
    (v, t, m), cam = scene_arrays("cornell")
    s = gbdev.RTScene(v, t, m).build_bvh()
    s.trace_rays(np.array([[0.5, 0.5, 0.5, 0.0, 0.0, 1.0]], np.float32))  # uploads the scene first
    want = gbdev.RTRenderer(24, 24, 1, gbdev.default_params()).render(s, cam).copy()
    failures = 0
    try:
        for after in range(0, 60, 3):
            L.gbpt_test_fail_allocations(after)
            r = gbdev.RTRenderer(24, 24, 1, gbdev.default_params())
            try:
                r.render(s, cam)
            except gbdev.GbptError as e:
                assert e.status == 2, e  # GBPT_ERR_OOM
                failures += 1
            finally:
                L.gbpt_test_fail_allocations(-1)
                r.close()
    finally:
        L.gbpt_test_fail_allocations(-1)
    assert failures >= 5
    got = gbdev.RTRenderer(24, 24, 1, gbdev.default_params()).render(s, cam)
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))
