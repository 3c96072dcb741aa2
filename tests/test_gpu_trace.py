"""Closest-hit / any-hit parity of the CUDA traversal with the reference.

The golden fixtures hold the reference's own answers (BVH::intersect and
intersect_any run by oracle/ref_harness.cpp); larger batches are checked
against the oracle port, which test_oracle_pins.py pins to the reference
bit for bit.  The bar is bit-exact primitive ids and distances."""
import numpy as np
import pytest

from cpppt import scenes
from tests.golden.make_golden import SMALL_SCENES

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", sorted(SMALL_SCENES))
def test_closest_matches_reference_fixture(gpu_lib, golden, name):
    from cpppt.lib import GpuScene
    g = golden(f"{name}_ref.npz")
    sc = SMALL_SCENES[name]()
    gs = GpuScene(sc)
    idx, t, beta, gamma = gs.trace_closest(g["rays"])
    assert np.array_equal(idx, g["hit_index"]), np.nonzero(idx != g["hit_index"])[0][:10]
    assert np.array_equal(t.view(np.uint32), g["hit_t"].view(np.uint32))


@pytest.mark.parametrize("name", sorted(SMALL_SCENES))
def test_any_matches_reference_fixture(gpu_lib, golden, name):
    from cpppt.lib import GpuScene
    g = golden(f"{name}_ref.npz")
    gs = GpuScene(SMALL_SCENES[name]())
    occ = gs.trace_any(g["shadow_rays"])
    assert np.array_equal(occ, g["occluded"])


def test_closest_matches_oracle_large_batch(gpu_lib):
    from cpppt.lib import GpuScene
    from oracle.oracle import Oracle
    sc = scenes.soup(seed=2, n_spheres=400, freq=4, width=64, height=64)
    rays = scenes.hit_ray_batch(sc, 1 << 16, seed=11)
    oi, ot = Oracle("port").scene(sc).trace_closest(rays)
    gi, gt, _, _ = GpuScene(sc).trace_closest(rays)
    assert (oi >= 0).mean() > 0.9
    assert np.array_equal(gi, oi)
    assert np.array_equal(gt.view(np.uint32), ot.view(np.uint32))


@pytest.mark.parametrize("config", ["cornell256", "soup1M"])
def test_full_size_ray_batch_matches_oracle(gpu_lib, config):
    """2^20 rays (seed 6: camera, secondary, edge/vertex and axis-parallel
    rays) on the Cornell box and on the 1M-triangle soup: closest-hit ids and
    distances bit-exact, any-hit answers identical for max_t around the hit."""
    from cpppt.lib import GpuScene
    from oracle.oracle import Oracle
    sc = scenes.cornell(256, 256) if config == "cornell256" else scenes.soup(seed=2)
    rays = scenes.hit_ray_batch(sc, 1 << 20, seed=6)
    osc = Oracle("port").scene(sc)
    oi, ot = osc.trace_closest(rays)
    gs = GpuScene(sc)
    gi, gt, _, _ = gs.trace_closest(rays)
    assert (oi >= 0).mean() > 0.5
    bad = np.nonzero(gi != oi)[0]
    assert bad.size == 0, (bad.size, bad[:8])
    assert np.array_equal(gt.view(np.uint32), ot.view(np.uint32))
    sh = rays.copy()
    rng = np.random.default_rng(7)
    hit = oi >= 0
    sh[hit, 6] = ot[hit] * rng.uniform(0.5, 1.5, size=hit.sum()).astype(np.float32)
    oo = osc.trace_any(sh)
    go = gs.trace_any(sh)
    assert 0.2 < oo.mean() < 0.9
    assert np.array_equal(go, oo)


def test_empty_and_degenerate_inputs(gpu_lib):
    from cpppt.lib import GpuScene
    sc = scenes.cornell(16, 16)
    gs = GpuScene(sc)
    idx, t, _, _ = gs.trace_closest(np.zeros((0, 7), np.float32))
    assert idx.size == 0
    # rays pointing away from everything and zero-length max_t
    rays = np.array([[0.5, 0.5, 5.0, 0, 0, 1, np.inf], [0.5, 0.5, 0.5, 0, 1, 0, 0.0]], np.float32)
    idx, t, _, _ = gs.trace_closest(rays)
    assert idx[0] == -1 and idx[1] == -1
