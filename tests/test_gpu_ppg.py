"""SD-tree guided rendering (PPG, row a14) on the GPU against the reference's
own PPG renderer (src/renderer/ppg.h:149-215, run by the oracle harness).

Both learn their SD-tree online from their own paths, so the trees differ
sample by sample; the one-sample MIS estimator's mean does not depend on the
guide, so the images must agree statistically: per-tile z-test on replica
means.  The host tree update is pinned bit for bit in test_sdtree_host.py."""
import numpy as np
import pytest

from cpppt import scenes
from tests.test_gpu_render import check_z, tile_means, ztest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,res", [("cornell", (32, 32)), ("slitroom", (32, 16))])
def test_ppg_matches_reference_ppg(gpu_lib, name, res):
    from cpppt.lib import MODE_SDTREE, GpuScene
    from oracle import oracle as orc
    from tests.golden.make_golden import SMALL_SCENES
    if not orc.reference_available():
        pytest.fail("reference harness missing (build with __graft_entry__.build())")
    sc = SMALL_SCENES[name]().with_resolution(*res)
    R, tile, spp_axis = 8, 8, 8
    ref = orc.Oracle("reference").scene(sc)
    r_imgs = np.stack([ref.render_ppg(spp_axis, 100 * (r + 1))[0] for r in range(R)])
    gs = GpuScene(sc)
    g_imgs = np.stack([gs.render(spp_axis * spp_axis, max_depth=32, seed=50 + r, mode=MODE_SDTREE)
                       for r in range(R)])
    assert np.isfinite(g_imgs).all()
    check_z(ztest(tile_means(g_imgs, tile), tile_means(r_imgs, tile)), max_abs=6.0, frac3=0.05)


def test_ppg_learns_and_reports_stats(gpu_lib):
    from cpppt.lib import MODE_SDTREE, GpuScene
    gs = GpuScene(scenes.cornell(64, 64))
    img = gs.render(256, max_depth=16, seed=3, mode=MODE_SDTREE)
    st = gs.stats()
    # passes of 1, 2, ..., 128 spp: 255 spp worth of paths
    assert st["paths"] == 64 * 64 * 255
    assert img.mean() > 0.05 and np.isfinite(img).all()
