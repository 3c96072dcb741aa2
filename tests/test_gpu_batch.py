"""Multi-scene batches: every job's image must be bit-identical to pt_render
of the same scene with the same parameters, whatever the launch shape."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def members(gpu_lib):
    from cpppt import scenes
    from cpppt.lib import GpuScene
    scs = [
        scenes.cornell(32, 32),
        scenes.soup(seed=11, n_spheres=40, freq=3, width=24, height=16),
        scenes.slit_room(seed=4, n_boxes=20, box_subdiv=2, width=16, height=8),
        scenes.soup(seed=12, n_spheres=300, freq=4, width=40, height=24),
        scenes.cornell(8, 8),
    ]
    return [GpuScene(s) for s in scs]


JOBS = [
    dict(scene=0, spp=16, max_depth=8, seed=3),
    dict(scene=1, spp=9, max_depth=10, seed=5),
    dict(scene=2, spp=4, max_depth=12, seed=7),
    dict(scene=3, spp=7, max_depth=10, seed=9),
    dict(scene=0, spp=5, max_depth=4, rr_start=1, seed=11),  # the same scene again, other parameters
    dict(scene=4, spp=64, max_depth=8, seed=13),
]


def unbatched(members, j):
    return members[j["scene"]].render(j["spp"], max_depth=j.get("max_depth", 32), rr_start=j.get("rr_start", 3),
                                      seed=j.get("seed", 0))


def test_batch_matches_unbatched_bit_exact(members):
    from cpppt.lib import GpuBatch
    b = GpuBatch(members)
    imgs = b.render(JOBS)
    st = b.stats()
    assert st["paths"] == sum(members[j["scene"]].width * members[j["scene"]].height * j["spp"] for j in JOBS)
    for j, img in zip(JOBS, imgs):
        ref = unbatched(members, j)
        assert img.shape == ref.shape
        assert np.array_equal(img.view(np.uint32), ref.view(np.uint32)), j
        assert img.mean() > 0


@pytest.mark.parametrize("tuning", [dict(capacity=1024, iters_per_graph=2, tile_w=1, tile_h=1),
                                    dict(capacity=4096, iters_per_graph=8, tile_w=8, tile_h=4),
                                    dict(capacity=1 << 20, iters_per_graph=32, tile_w=4, tile_h=8)])
def test_launch_shape_does_not_change_images(members, tuning):
    from cpppt.lib import GpuBatch
    b = GpuBatch(members)
    ref = b.render(JOBS)
    got = b.set_tuning(**tuning)
    assert got == tuning
    imgs = b.render(JOBS)
    for a, r in zip(imgs, ref):
        assert np.array_equal(a.view(np.uint32), r.view(np.uint32))


def test_autotune_picks_a_valid_shape(members):
    from cpppt.lib import GpuBatch
    b = GpuBatch(members)
    best, rate = b.autotune(JOBS, spp_divisor=2)
    assert rate > 0
    assert best == b.tuning()
    assert best["capacity"] % 1024 == 0 and best["iters_per_graph"] % 2 == 0
    imgs = b.render(JOBS[:2])
    for j, img in zip(JOBS[:2], imgs):
        assert np.array_equal(img.view(np.uint32), unbatched(members, j).view(np.uint32))


def test_batch_loop_runs_on_the_device(members):
    """A batch render is one graph launch of the whole loop: one counter read."""
    from cpppt.lib import GpuBatch
    b = GpuBatch(members)
    b.render(JOBS, outputs=False)
    st = b.stats()
    assert st["d2h_bytes"] == 128
    assert st["paths"] == sum(members[j["scene"]].width * members[j["scene"]].height * j["spp"] for j in JOBS)


def test_device_outputs(members):
    import torch
    from cpppt.lib import GpuBatch
    b = GpuBatch(members)
    outs = [torch.zeros((members[j["scene"]].height, members[j["scene"]].width, 3), dtype=torch.float32,
                        device="cuda") for j in JOBS]
    b.render_device(JOBS, [o.data_ptr() for o in outs])
    for j, o in zip(JOBS, outs):
        assert np.array_equal(o.cpu().numpy().view(np.uint32), unbatched(members, j).view(np.uint32))


def test_batch_modes_match_unbatched(members):
    """The other integrators (PT_MODE_NEE, PT_MODE_PT) and the slot
    wavefront's unbiased MIS estimator, batched, bit-identical to pt_render."""
    from cpppt.lib import FLAG_THROUGHPUT_RR, FLAG_UNBIASED_MIS, MODE_MIS, MODE_NEE, MODE_PT, GpuBatch
    b = GpuBatch(members)
    for mode, flags in [(MODE_NEE, 0), (MODE_PT, 0), (MODE_MIS, FLAG_UNBIASED_MIS),
                        (MODE_MIS, FLAG_UNBIASED_MIS | FLAG_THROUGHPUT_RR)]:
        imgs = b.render(JOBS, mode=mode, flags=flags)
        for j, img in zip(JOBS, imgs):
            ref = members[j["scene"]].render(j["spp"], max_depth=j.get("max_depth", 32),
                                             rr_start=j.get("rr_start", 3), seed=j.get("seed", 0), mode=mode,
                                             flags=flags)
            assert np.array_equal(img.view(np.uint32), ref.view(np.uint32)), (mode, flags, j)


@pytest.fixture(scope="module")
def guided(gpu_lib):
    """Three scenes, each with its own learned guide, trained a little by
    single-scene renders (batch of 1024 records, so small renders train)."""
    from cpppt import scenes
    from cpppt.lib import MODE_NN, GpuScene
    scs = [scenes.slit_room(seed=4, n_boxes=20, box_subdiv=2, width=32, height=16),
           scenes.slit_room(seed=5, n_boxes=40, box_subdiv=2, width=24, height=24),
           scenes.cornell(16, 16)]
    gs = [GpuScene(s) for s in scs]
    for k, g in enumerate(gs):
        g.nn_reset(100 + k)
        g.nn_configure(**{**g.nn_config(), "batch": 1024})
        for r in range(4):
            g.render(16, max_depth=8, seed=50 + r, mode=MODE_NN)
        assert g.nn_stats()["steps"] > 0
    return gs


GUIDED_JOBS = [dict(scene=0, spp=16, max_depth=8, seed=1), dict(scene=2, spp=9, max_depth=6, seed=2),
               dict(scene=1, spp=4, max_depth=12, seed=3), dict(scene=0, spp=5, max_depth=3, seed=4)]


def test_frozen_guides_batched_bit_exact(guided):
    """Every job is guided by its own scene's network: with the guides frozen
    the batched images equal the single-scene guided renders bit for bit."""
    from cpppt.lib import FLAG_NN_FREEZE, FLAG_THROUGHPUT_RR, MODE_NN, GpuBatch
    b = GpuBatch(guided)
    for flags in (FLAG_NN_FREEZE, FLAG_NN_FREEZE | FLAG_THROUGHPUT_RR):
        imgs = b.render(GUIDED_JOBS, mode=MODE_NN, flags=flags)
        for j, img in zip(GUIDED_JOBS, imgs):
            ref = guided[j["scene"]].render(j["spp"], max_depth=j["max_depth"], seed=j["seed"], mode=MODE_NN,
                                            flags=flags)
            assert np.isfinite(img).all() and img.mean() > 0
            assert np.array_equal(img.view(np.uint32), ref.view(np.uint32)), (flags, j)


def test_batch_trains_each_scene_guide(guided):
    """An unfrozen batched render trains the guide of every scene it
    renders, on that scene's records, and leaves the others alone."""
    from cpppt.lib import MODE_NN, GpuBatch
    b = GpuBatch(guided)
    w0 = [g.nn_weights().copy() for g in guided]
    s0 = [g.nn_stats()["steps"] for g in guided]
    jobs = [dict(scene=0, spp=32, max_depth=8, seed=7), dict(scene=2, spp=32, max_depth=8, seed=8)]
    imgs = b.render(jobs, mode=MODE_NN)
    assert all(np.isfinite(x).all() and x.mean() > 0 for x in imgs)
    for k, g in enumerate(guided):
        trained = k in (0, 2)
        assert (g.nn_stats()["steps"] > s0[k]) == trained, k
        assert (not np.array_equal(g.nn_weights(), w0[k])) == trained, k


def test_batch_errors(members):
    from cpppt.lib import GpuBatch, PtError
    b = GpuBatch(members)
    with pytest.raises(PtError):
        b.render([dict(scene=len(members), spp=1)])
    with pytest.raises(PtError):
        b.render([dict(scene=0, spp=0)])
    with pytest.raises(PtError):
        b.set_tuning(capacity=1000)
    with pytest.raises(PtError):
        b.set_tuning(iters_per_graph=3)
    from cpppt.lib import FLAG_NN_FREEZE, FLAG_UNBIASED_MIS, MODE_MIS, MODE_NEE, MODE_SDTREE
    with pytest.raises(PtError):
        b.render([dict(scene=0, spp=1)], mode=MODE_SDTREE)
    with pytest.raises(PtError):
        b.render([dict(scene=0, spp=1)], mode=MODE_NEE, flags=FLAG_UNBIASED_MIS)
    with pytest.raises(PtError):
        b.render([dict(scene=0, spp=1)], mode=MODE_MIS, flags=FLAG_UNBIASED_MIS | FLAG_NN_FREEZE)
    with pytest.raises(PtError):
        b.render([dict(scene=0, spp=1)], mode=99)
    b.render([dict(scene=0, spp=1)])  # still usable


def test_batch_keeps_member_scenes_alive(gpu_lib):
    """pt_scene_destroy on a member of a live batch is deferred: the batch
    still renders with that scene's learned guide, and destroying the batch
    releases the scene."""
    import ctypes as C
    from cpppt import scenes
    from cpppt.lib import FLAG_NN_FREEZE, MODE_NN, GpuBatch, GpuScene
    gs = GpuScene(scenes.cornell(16, 16))
    ref = gs.render(4, max_depth=4, seed=2, mode=MODE_NN, flags=FLAG_NN_FREEZE)
    from cpppt import lib
    b = GpuBatch([gs])
    lib._lib.pt_scene_destroy(gs.h)  # destroyed through the C ABI while the batch lives
    gs.h = C.c_void_p()
    img = b.render([dict(scene=0, spp=4, max_depth=4, seed=2)], mode=MODE_NN, flags=FLAG_NN_FREEZE)[0]
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    b.close()  # releases the scene
