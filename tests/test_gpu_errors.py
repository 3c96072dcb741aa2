"""Device error paths: every bounded loop of the kernels reports through a
status word that the host turns into an error code, and the CUDA context
stays usable afterwards.  The limits are made to run out on purpose through
debug hooks (a lowered traversal step or stack bound; a completion barrier
that nothing arrives on), never by a fault or an endless wait.  Also the
film's fixed-point range: contributions it cannot hold are counted and the
render fails instead of returning a wrapped image."""
import ctypes as C
import dataclasses

import numpy as np
import pytest

from cpppt import scenes

pytestmark = pytest.mark.gpu


def _scene():
    return scenes.soup(seed=2, n_spheres=60, freq=3, width=32, height=32, extent=6.0)


def test_traversal_step_limit_is_reported(gpu_lib):
    from cpppt.lib import GpuScene, PtError
    sc = _scene()
    gs = GpuScene(sc)
    rays = scenes.hit_ray_batch(sc, 4096, seed=3)
    want = gs.trace_closest(rays)
    L = gpu_lib
    assert L.pt_debug_traversal_limits(gs.h, 2, 0) == 0
    with pytest.raises(PtError) as e:
        gs.trace_closest(rays)
    assert e.value.status == 4 and "step limit" in str(e.value)
    with pytest.raises(PtError) as e:
        gs.render(4, max_depth=4, seed=1)
    assert e.value.status == 4 and "step limit" in str(e.value)
    assert L.pt_debug_traversal_limits(gs.h, 0, 0) == 0  # defaults again: same answers as before
    got = gs.trace_closest(rays)
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1].view(np.uint32), want[1].view(np.uint32))
    assert np.isfinite(gs.render(4, max_depth=4, seed=1)).all()


def test_traversal_stack_overflow_is_reported(gpu_lib):
    from cpppt.lib import GpuScene, PtError
    sc = _scene()
    gs = GpuScene(sc)
    rays = scenes.hit_ray_batch(sc, 4096, seed=4)
    L = gpu_lib
    assert L.pt_debug_traversal_limits(gs.h, 0, 1) == 0
    with pytest.raises(PtError) as e:
        gs.trace_closest(rays)
    assert e.value.status == 4 and "stack overflow" in str(e.value)
    with pytest.raises(PtError):
        gs.trace_any(rays)
    assert L.pt_debug_traversal_limits(gs.h, 0, 0) == 0
    idx, _, _, _ = gs.trace_closest(rays)
    assert (idx >= 0).mean() > 0.3
    assert L.pt_debug_traversal_limits(gs.h, -1, 0) == 1  # out of range: PT_ERR_INVALID
    assert L.pt_debug_traversal_limits(gs.h, 0, 65) == 1


def test_tensor_wait_timeout_is_reported(gpu_lib):
    from cpppt import lib
    from tests.test_gpu_nn import HI, LO, random_inputs, random_weights
    L = gpu_lib
    st = L.pt_debug_tensor_wait_timeout()
    assert st == 2, st
    assert b"tensor-core completion wait timed out" in L.pt_last_error()
    # the context is still usable: the tensor-core forward pass runs
    out = lib.nn_forward(random_weights(1), LO, HI, random_inputs(512, 2))
    assert np.isfinite(out).all()


def _bright(intensity):
    sc = scenes.cornell(32, 32)
    params = sc.mat_params.copy()
    params[sc.mat_kind == scenes.EMISSIVE, 5] = intensity
    return dataclasses.replace(sc, mat_params=params)


def test_film_overflow_fails_the_render(gpu_lib):
    from cpppt.lib import GpuScene, PtError
    ok = GpuScene(_bright(17.0))
    ok.render(64, max_depth=8, seed=1)
    assert ok.stats()["film_overflow"] == 0
    # one contribution alone beyond the 32.32 range (4e9 >= 2^31)
    gs = GpuScene(_bright(4e9))
    with pytest.raises(PtError) as e:
        gs.render(16, max_depth=8, seed=1)
    assert e.value.status == 4 and "film overflow" in str(e.value)
    assert gs.stats()["film_overflow"] > 0
    # contributions that fit one by one, but whose per-pixel sum does not:
    # 64 samples of an emitter seen directly at 1e8 add up to 6.4e9 > 2^31
    gs = GpuScene(_bright(1e8))
    with pytest.raises(PtError) as e:
        gs.render(64, max_depth=1, seed=1)
    assert e.value.status == 4
    assert gs.stats()["film_overflow"] > 0
    # the same emitter at 8 samples fits (8e8 < 2^31): nothing is counted
    gs.render(8, max_depth=1, seed=1)
    assert gs.stats()["film_overflow"] == 0
