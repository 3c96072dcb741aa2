"""Pins the oracle (oracle/pt_oracle.c) to the reference.

tests/golden/*_ref.npz are outputs of the reference's own code (see
tests/golden/make_golden.py).  The oracle must reproduce all of them bit for
bit: BVH topology and boxes, closest-hit ids and distances, any-hit
answers, and rendered images (same mt19937 streams, same float steps)."""
import numpy as np
import pytest

from tests.golden.make_golden import SMALL_SCENES


@pytest.fixture(scope="module")
def port():
    from oracle.oracle import Oracle
    return Oracle("port")


@pytest.mark.parametrize("name", sorted(SMALL_SCENES))
def test_bvh_topology(port, golden, name):
    g = golden(f"{name}_ref.npz")
    order, boxes, parent, pparent = port.scene(SMALL_SCENES[name]()).bvh_dump()
    assert np.array_equal(order, g["leaf_order"])
    assert np.array_equal(boxes.view(np.uint32), g["node_boxes"].view(np.uint32))
    assert np.array_equal(parent, g["node_parent"])
    assert np.array_equal(pparent, g["prim_parent"])


@pytest.mark.parametrize("name", sorted(SMALL_SCENES))
def test_hits(port, golden, name):
    g = golden(f"{name}_ref.npz")
    s = port.scene(SMALL_SCENES[name]())
    idx, t = s.trace_closest(g["rays"])
    assert np.array_equal(idx, g["hit_index"])
    assert np.array_equal(t.view(np.uint32), g["hit_t"].view(np.uint32))
    assert np.array_equal(s.trace_any(g["shadow_rays"]), g["occluded"])


@pytest.mark.parametrize("name", sorted(SMALL_SCENES))
def test_render_bitwise(port, golden, name):
    g = golden(f"{name}_ref.npz")
    s = port.scene(SMALL_SCENES[name]())
    img, _ = s.render_mis(2, 8, 0)
    assert np.array_equal(img.view(np.uint32), g["render_spp2_d8"].view(np.uint32))
    img32, _ = s.render_mis(1, 32, 7)
    assert np.array_equal(img32.view(np.uint32), g["render_spp1_d32_seed7"].view(np.uint32))


@pytest.mark.parametrize("name", sorted(SMALL_SCENES))
def test_other_integrators_bitwise(port, golden, name):
    """Pathtracer (NEE without MIS) and PurePt (no NEE) of the reference."""
    g = golden(f"{name}_ref.npz")
    s = port.scene(SMALL_SCENES[name]())
    nee, _ = s.render_variant(1, 2, 8, 3)
    assert np.array_equal(nee.view(np.uint32), g["render_nee_spp2_d8_seed3"].view(np.uint32))
    pure, _ = s.render_variant(2, 2, 8, 3)
    assert np.array_equal(pure.view(np.uint32), g["render_pure_spp2_d8_seed3"].view(np.uint32))


def test_reference_harness_matches_fixture(golden):
    """When the reference can be compiled here, it still gives the fixtures."""
    from oracle import oracle as orc
    if not orc.reference_available():
        pytest.skip("reference harness not built in this environment")
    g = golden("cornell_ref.npz")
    s = orc.Oracle("reference").scene(SMALL_SCENES["cornell"]())
    idx, t = s.trace_closest(g["rays"])
    assert np.array_equal(idx, g["hit_index"])


@pytest.mark.parametrize("spp_axis,depth,seed", [(2, 8, 3), (1, 12, 40), (3, 4, 7)])
def test_textured_room_port_matches_reference(tmp_path, spp_axis, depth, seed):
    """The port's image textures (bilinear sampling, REPEAT wrap, per-hit
    metal / roughness / albedo, normal map at the first hit, emission texture
    also at the light sample) give the reference's own render of the
    textured room's files bit for bit; the texture pixels come from the
    reference's Image loader."""
    from oracle import oracle as orc
    from tests import texscene
    if not orc.reference_available():
        pytest.skip("reference harness not built here")
    ref = orc.Oracle("reference")
    settings = texscene.write(str(tmp_path))
    rs = ref.load_files(settings)
    sc, uv, tex_info, tex_px, mat_tex, mat_emit = texscene.port_inputs(str(tmp_path), ref.image_load)
    ps = orc.Oracle("port").scene(sc).set_textures(uv, tex_info, tex_px, mat_tex, mat_emit)
    want, _ = rs.render_mis(spp_axis, depth, seed, threads=1)
    got, _ = ps.render_mis(spp_axis, depth, seed)
    assert want.mean() > 0
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("name", sorted(SMALL_SCENES))
def test_culling_traversal_matches_goldens(port, golden, name):
    """The port's culling traversal (set_fast) gives the reference's answers
    on the golden ray batches and the bit-identical renders."""
    g = golden(f"{name}_ref.npz")
    s = port.scene(SMALL_SCENES[name]()).set_fast()
    idx, t = s.trace_closest(g["rays"])
    assert np.array_equal(idx, g["hit_index"])
    assert np.array_equal(t.view(np.uint32), g["hit_t"].view(np.uint32))
    assert np.array_equal(s.trace_any(g["shadow_rays"]), g["occluded"])
    img, _ = s.render_mis(2, 8, 0)
    assert np.array_equal(img.view(np.uint32), g["render_spp2_d8"].view(np.uint32))


@pytest.mark.parametrize("make", [lambda: __import__("cpppt.scenes").scenes.soup(seed=9, n_spheres=400),
                                  lambda: __import__("cpppt.scenes").scenes.slit_room(seed=4, n_boxes=150,
                                                                                      box_subdiv=2)],
                         ids=["soup200k", "slitroom29k"])
def test_culling_traversal_matches_exhaustive(port, make):
    """Larger scenes than the goldens: the culling traversal against the
    exhaustive recursion on 2^14 mixed rays (camera, secondary, edge and
    vertex aims, axis-parallel), closest and any hit, bit for bit."""
    from cpppt import scenes
    sc = make()
    rays = scenes.hit_ray_batch(sc, 1 << 14, seed=21)
    slow = port.scene(sc)
    fast = port.scene(sc).set_fast()
    i0, t0 = slow.trace_closest(rays)
    i1, t1 = fast.trace_closest(rays)
    assert (i0 >= 0).mean() > 0.5
    assert np.array_equal(i0, i1)
    assert np.array_equal(t0.view(np.uint32), t1.view(np.uint32))
    sh = rays.copy()
    sh[:, 6] = np.where(np.isfinite(t0), t0 * np.float32(0.999), np.float32(3.0))
    assert np.array_equal(slow.trace_any(sh), fast.trace_any(sh))
