"""Image textures on the GPU against the reference: the textured room of
tests/texscene.py (tiled sRGB albedo, metal and roughness maps, a normal
map, an emission texture), written to files here and loaded by this
library's loader, rendered by the GPU PT + NEE + MIS and compared with the
reference's own render of the same files (tests/golden/texroom_ref.npz:
16 replicas x 64 spp, its filtering pinned to bilinear) through a per-tile
z-test on the replica means.  Also checked: every integrator and the slot
wavefront see the textures, and batched jobs give the single renders'
images."""
import numpy as np
import pytest

from tests.test_gpu_render import check_z, tile_means, ztest

pytestmark = pytest.mark.gpu


def _scene(tmp_path):
    from cpppt.lib import GpuScene
    from tests import texscene
    return GpuScene(settings_file=texscene.write(str(tmp_path)))


def test_textured_room_matches_reference(gpu_lib, golden, tmp_path):
    g = golden("texroom_ref.npz")
    R, spp, depth, tile = int(g["replicas"]), int(g["spp_per_replica"]), int(g["depth"]), int(g["tile"])
    gs = _scene(tmp_path)
    imgs = np.stack([gs.render(spp, max_depth=depth, seed=900 + r) for r in range(R)])
    assert np.isfinite(imgs).all()
    assert gs.stats()["nonfinite"] == 0
    check_z(ztest(tile_means(imgs, tile), g["tile_means"]), max_abs=6.0, frac3=0.05)
    # the textures matter: the same room with constant materials differs
    mean, ref = imgs.mean(0), g["mean"]
    assert abs(mean.mean() - ref.mean()) < 0.03 * ref.mean()


def test_textures_in_every_mode_and_batched(gpu_lib, tmp_path):
    from cpppt.lib import (FLAG_NN_FREEZE, FLAG_UNBIASED_MIS, MODE_MIS, MODE_NEE, MODE_NN, MODE_PT, GpuBatch)
    gs = _scene(tmp_path)
    base = np.stack([gs.render(64, max_depth=8, seed=10 + r) for r in range(4)]).mean(0)
    for mode, flags in [(MODE_NEE, 0), (MODE_PT, 0), (MODE_MIS, FLAG_UNBIASED_MIS), (MODE_NN, FLAG_NN_FREEZE)]:
        img = np.stack([gs.render(64, max_depth=8, seed=20 + r, mode=mode, flags=flags) for r in range(4)]).mean(0)
        assert np.isfinite(img).all()
        # all estimate the same image here (no delta lights; the camera sees
        # no emitter directly): the image means agree within noise
        assert abs(img.mean() - base.mean()) < 0.05 * base.mean(), (mode, flags)
    b = GpuBatch([gs])
    jobs = [dict(scene=0, spp=16, max_depth=8, seed=3), dict(scene=0, spp=9, max_depth=5, seed=4)]
    imgs = b.render(jobs)
    for j, img in zip(jobs, imgs):
        ref = gs.render(j["spp"], max_depth=j["max_depth"], seed=j["seed"])
        assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))


def test_batch_of_textured_and_plain_scenes(gpu_lib, tmp_path):
    """The batch arena appends every scene's textures and rebases the
    materials' texture slots: a batch of a plain scene and two textured
    rooms (one with its own copies of the files, one sharing none) gives
    each job its single render, bit for bit."""
    from cpppt import scenes
    from cpppt.lib import GpuBatch, GpuScene
    from tests import texscene
    a = GpuScene(scenes.cornell(24, 16))
    b = GpuScene(settings_file=texscene.write(str(tmp_path / "b")))
    c = GpuScene(settings_file=texscene.write(str(tmp_path / "c")))
    batch = GpuBatch([a, b, c])
    jobs = [dict(scene=1, spp=9, max_depth=6, seed=1), dict(scene=0, spp=4, max_depth=6, seed=2),
            dict(scene=2, spp=16, max_depth=8, seed=3), dict(scene=1, spp=4, max_depth=3, seed=4)]
    imgs = batch.render(jobs)
    for j, img in zip(jobs, imgs):
        ref = [a, b, c][j["scene"]].render(j["spp"], max_depth=j["max_depth"], seed=j["seed"])
        assert np.array_equal(img.view(np.uint32), ref.view(np.uint32)), j
