"""Image parity of the GPU PT+NEE+MIS with the reference's PathtracerMIS.

The GPU draws its own (counter-based) random numbers, so parity is
statistical:

* Cornell box 256x256, 16384 spp, depth 8 against the reference's own
  16k-spp render (tests/golden/cornell256_16k_ref.npz: 16 replicas x 1024
  spp): relMSE < 1e-3 with relMSE = mean (x - ref)^2 / (ref^2 + 1e-2), and a
  per-tile z-test on the means (16x16-pixel tiles, standard errors from the
  replicas of both sides).
* Scenes with GGX, dielectric and occluded light against the oracle port
  (pinned to the reference bit for bit) at small size: per-tile z-test.
"""
import os

import numpy as np
import pytest

from cpppt import scenes
from tests.golden.make_golden import SMALL_SCENES

pytestmark = pytest.mark.gpu


def rel_mse(x, ref):
    return float(np.mean((x - ref) ** 2 / (ref ** 2 + 1e-2)))


def tile_means(imgs, tile):
    R, H, W, C = imgs.shape
    return imgs.reshape(R, H // tile, tile, W // tile, tile, C).mean(axis=(2, 4))


def ztest(tiles_a, tiles_b):
    """z per tile and channel from replica means (R_a x T x T x 3, R_b x ...)."""
    ma, mb = tiles_a.mean(0), tiles_b.mean(0)
    va = tiles_a.var(0, ddof=1) / tiles_a.shape[0]
    vb = tiles_b.var(0, ddof=1) / tiles_b.shape[0]
    return (ma - mb) / np.sqrt(va + vb + 1e-20)


def check_z(z, max_abs=5.5, frac3=0.02):
    z = z.reshape(-1)
    assert np.isfinite(z).all()
    assert np.abs(z).max() < max_abs, f"max |z| {np.abs(z).max():.2f}"
    assert (np.abs(z) > 3).mean() <= frac3, f"{(np.abs(z) > 3).mean():.3f} of tiles beyond 3 sigma"


def test_cornell_16k_matches_reference(gpu_lib, golden):
    from cpppt.lib import GpuScene
    path = os.path.join(os.path.dirname(__file__), "golden", "cornell256_16k_ref.npz")
    if not os.path.exists(path):
        pytest.fail("missing golden fixture cornell256_16k_ref.npz")
    g = golden("cornell256_16k_ref.npz")
    R = int(g["replicas"])
    spp = int(g["spp_per_replica"])
    tile = int(g["tile"])
    gs = GpuScene(scenes.cornell(256, 256))
    imgs = np.stack([gs.render(spp, max_depth=int(g["depth"]), seed=77 + r) for r in range(R)])
    mean = imgs.mean(0)
    rel = rel_mse(mean, g["mean"])
    assert rel < 1e-3, f"relMSE {rel:.3e}"
    check_z(ztest(tile_means(imgs, tile), g["tile_means"]))


@pytest.mark.parametrize("name", ["soup", "slitroom", "cornell"])
def test_small_scenes_match_oracle(gpu_lib, name):
    from cpppt.lib import GpuScene
    from oracle.oracle import Oracle
    sc = SMALL_SCENES[name]()
    R, tile = 8, 8
    sc = sc.with_resolution(32, 32) if name == "cornell" else sc.with_resolution(32, 16)
    ors = Oracle("port").scene(sc)
    o_imgs = np.stack([ors.render_mis(16, 10, 5000 * (r + 1))[0] for r in range(R)])  # 256 spp each
    gs = GpuScene(sc)
    g_imgs = np.stack([gs.render(1024, max_depth=10, seed=300 + r) for r in range(R)])
    check_z(ztest(tile_means(g_imgs, tile), tile_means(o_imgs, tile)))
    assert rel_mse(g_imgs.mean(0), o_imgs.mean(0)) < 0.05


SINGLE_MATERIAL = {
    # all spheres GGX, roughness U[0.05, 0.5]: alpha clamped to 0.01 below roughness 0.1
    "ggx": dict(only=1),
    # all spheres GGX, roughness U[0.3, 0.5]
    "ggx_rough": dict(only=1, rough_range=(0.3, 0.5)),
    # all spheres the terminating dielectric (IOR 1.5): only total internal reflection continues
    "dielectric": dict(only=2),
}


@pytest.mark.parametrize("name", sorted(SINGLE_MATERIAL))
def test_single_material_soups_match_oracle(gpu_lib, name):
    """Soups of one material kind packed so that the spheres fill the view
    (60 spheres in a 6-unit cube), 64x64, depth 10, against the oracle port:
    16 replicas a side of 64 spp each, per-tile z-test on 8x8 tiles of the
    grey level (the materials and the light are white, so the channels carry
    the same information: 64 values), and the whole-image mean within 4
    standard errors.  The reference's GGX eval is D G / (4 cos theta_o),
    unbounded at grazing wo, and NEE keeps its full weight towards grazing
    lights, so at alpha = 0.01 a few samples are very large: the estimator is
    heavy-tailed and skewed, so both sides take the same number of samples
    (a side with fewer samples misses the rare bright ones more often and
    reads low), and the relMSE of the mean images is only bounded for the
    rougher and the dielectric soups."""
    from cpppt.lib import GpuScene
    from oracle.oracle import Oracle
    sc = scenes.soup(seed=2, n_spheres=60, freq=3, width=64, height=64, extent=6.0, **SINGLE_MATERIAL[name])
    R, tile = 16, 8
    ors = Oracle("port").scene(sc).set_fast()
    o_imgs = np.stack([ors.render_mis(8, 10, 7000 * (r + 1))[0] for r in range(R)])  # 64 spp each
    gs = GpuScene(sc)
    g_imgs = np.stack([gs.render(64, max_depth=10, seed=900 + r) for r in range(R)])
    grey = lambda x: x.mean(axis=3, keepdims=True)
    check_z(ztest(tile_means(grey(g_imgs), tile), tile_means(grey(o_imgs), tile)), frac3=0.05)
    ga, oa = g_imgs.mean(axis=(1, 2, 3)), o_imgs.mean(axis=(1, 2, 3))
    se = np.sqrt(ga.var(ddof=1) / R + oa.var(ddof=1) / R)
    assert abs(ga.mean() - oa.mean()) < 4 * se, (ga.mean(), oa.mean(), se)
    if name != "ggx":
        assert rel_mse(g_imgs.mean(0), o_imgs.mean(0)) < 0.05


def test_full_size_soup_image_matches_oracle(gpu_lib):
    """The 1M-triangle workload of the benchmark (2000 spheres x 500
    triangles, Lambert / GGX / dielectric, four emitters, depth 10) rendered
    whole at 96x48 on the GPU and by the oracle port (culling traversal, same
    answers as the reference's): 16 replicas a side, per-tile z-test on
    12x12 tiles (96 values)."""
    from cpppt.lib import GpuScene
    from oracle.oracle import Oracle
    sc = scenes.soup(seed=2, n_spheres=2000, freq=5, width=96, height=48)
    R, tile = 16, 12
    ors = Oracle("port").scene(sc).set_fast()
    o_imgs = np.stack([ors.render_mis(6, 10, 11000 * (r + 1))[0] for r in range(R)])  # 36 spp each
    gs = GpuScene(sc)
    g_imgs = np.stack([gs.render(1024, max_depth=10, seed=1300 + r) for r in range(R)])
    assert o_imgs.mean() > 0
    check_z(ztest(tile_means(g_imgs, tile), tile_means(o_imgs, tile)))
    # whole-image mean per channel: within 4 standard errors of the replicas
    ga, oa = g_imgs.mean(axis=(1, 2)), o_imgs.mean(axis=(1, 2))
    se = np.sqrt(ga.var(0, ddof=1) / R + oa.var(0, ddof=1) / R)
    assert (np.abs(ga.mean(0) - oa.mean(0)) < 4 * se).all(), (ga.mean(0), oa.mean(0), se)


@pytest.mark.parametrize("name,integrator", [(n, i) for n in sorted(SMALL_SCENES) for i in (1, 2)
                                              if not (n == "slitroom" and i == 2)])
def test_other_integrators_match_oracle(gpu_lib, name, integrator):
    """PT_MODE_NEE (Pathtracer: NEE without MIS) and PT_MODE_PT (PurePt) on
    the same wavefront against the oracle port of the reference's own
    integrators (pinned bit-exact by test_oracle_pins).  Pure PT on the slit
    room is left out: without NEE, the light behind the slit is reached too
    rarely for a per-tile test at this size."""
    from cpppt.lib import MODE_NEE, MODE_PT, GpuScene
    from oracle.oracle import Oracle
    sc = SMALL_SCENES[name]()
    R, tile = 8, 8
    sc = sc.with_resolution(32, 32) if name == "cornell" else sc.with_resolution(32, 16)
    ors = Oracle("port").scene(sc)
    o_imgs = np.stack([ors.render_variant(integrator, 16, 10, 5000 * (r + 1))[0] for r in range(R)])
    gs = GpuScene(sc)
    mode = MODE_NEE if integrator == 1 else MODE_PT
    g_imgs = np.stack([gs.render(1024, max_depth=10, seed=300 + r, mode=mode) for r in range(R)])
    # 48 z values per scene: at most two beyond 3 sigma (these estimators have
    # heavier tails than the MIS one, so replica variances are rougher)
    check_z(ztest(tile_means(g_imgs, tile), tile_means(o_imgs, tile)), frac3=0.045)
    assert rel_mse(g_imgs.mean(0), o_imgs.mean(0)) < 0.05


def test_render_is_deterministic_and_seeded(gpu_lib):
    from cpppt.lib import GpuScene
    gs = GpuScene(scenes.cornell(32, 32))
    a = gs.render(16, max_depth=8, seed=5)
    b = gs.render(16, max_depth=8, seed=5)
    c = gs.render(16, max_depth=8, seed=6)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, c)


def test_render_stats_account_for_every_path(gpu_lib):
    from cpppt.lib import GpuScene
    gs = GpuScene(scenes.cornell(48, 40))
    gs.render(9, max_depth=8, seed=1)
    st = gs.stats()
    assert st["paths"] == 48 * 40 * 9
    assert st["closest_rays"] >= st["paths"]
    assert st["iterations"] >= 8


def test_render_loop_runs_on_the_device(gpu_lib):
    """The whole wavefront loop is one graph launch (a conditional loop whose
    control kernel ends it): the host reads the counters once per render,
    however many loop bodies ran."""
    from cpppt.lib import GpuScene
    gs = GpuScene(scenes.cornell(64, 64))
    gs.render(64, max_depth=8, seed=2)
    st = gs.stats()
    assert st["d2h_bytes"] == 128 + 64 * 64 * 3 * 4  # one WaveCounters read and the image
    assert st["kernel_launches"] > 5 * 16  # more than one loop body ran
    assert st["paths"] == 64 * 64 * 64


def test_render_argument_errors(gpu_lib):
    from cpppt.lib import GpuScene, PtError
    gs = GpuScene(scenes.cornell(8, 8))
    with pytest.raises(PtError):
        gs.render(0)
    with pytest.raises(PtError):
        gs.render(4, max_depth=0)
