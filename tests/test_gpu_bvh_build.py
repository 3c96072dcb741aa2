"""Device build of the reference-topology BVH (csrc/gpu_bvh.cu): the same
tree as BVH::build (bvh.h:151-216) -- leaf order (the tie-break ranks),
internal-node boxes in pre-order and each triangle's innermost internal
node -- bit for bit against the reference's own trees (golden fixtures), the
host build and the oracle, including -0.0 / +0.0 coordinates (the
reference's min / max keep the later of equal values) and a block of
coincident triangles (the reference's endless recursion becomes one leaf).
pt_scene_create builds every scene's tree this way, so the hit and image
tests run on it too."""
import numpy as np
import pytest

from cpppt import scenes
from tests.golden.make_golden import SMALL_SCENES

pytestmark = pytest.mark.gpu


def _same(a, b):
    order, boxes, pparent = a[:3]
    o_order, o_boxes, o_pparent = b[:3]
    assert np.array_equal(order, o_order)
    assert boxes.shape == o_boxes.shape
    assert np.array_equal(boxes.view(np.uint32), o_boxes.view(np.uint32))
    assert np.array_equal(pparent, o_pparent)


@pytest.mark.parametrize("name", sorted(SMALL_SCENES))
def test_device_build_matches_reference_fixture(gpu_lib, golden, name):
    from cpppt import lib
    g = golden(f"{name}_ref.npz")
    order, boxes, pparent, _ = lib.ref_topology_device(SMALL_SCENES[name]())
    _same((order, boxes, pparent), (g["leaf_order"], g["node_boxes"], g["prim_parent"]))


def test_device_build_matches_host_with_coincident_block(gpu_lib):
    from cpppt import lib
    sc = scenes.soup(seed=9, n_spheres=1000, freq=4, width=8, height=8)
    sc.triangles[1000:41000] = sc.triangles[7]  # 40000 coincident copies of one triangle
    dev = lib.ref_topology_device(sc)
    assert dev[3] > 10
    _same(dev, lib.ref_topology(sc))


def test_device_build_signed_zeros(gpu_lib):
    """Coordinates of 0.0 written as +0.0 and -0.0 in an irregular pattern:
    every min / max must keep the later of two equal values."""
    from cpppt import lib
    from oracle.oracle import Oracle
    sc = scenes.soup(seed=11, n_spheres=150, freq=3, width=8, height=8, extent=4.0)
    rng = np.random.default_rng(3)
    v = sc.vertices.copy()
    pick = rng.random(v.shape) < 0.25
    v[pick] = np.round(v[pick])  # many exact integers, among them zeros
    v[(v == 0) & (rng.random(v.shape) < 0.5)] = np.float32(-0.0)
    assert (np.signbit(v) & (v == 0)).sum() > 50
    sc.vertices = v
    dev = lib.ref_topology_device(sc)
    _same(dev, lib.ref_topology(sc))
    o_order, o_boxes, _, o_pparent = Oracle("port").scene(sc).bvh_dump()
    _same(dev, (o_order, o_boxes, o_pparent))


@pytest.mark.parametrize("make", [lambda: scenes.soup(seed=2),
                                  lambda: scenes.slit_room(seed=4, n_boxes=1000, box_subdiv=4)],
                         ids=["soup1M", "slitroom192k"])
def test_device_build_full_size(gpu_lib, make):
    from cpppt import lib
    sc = make()
    _same(lib.ref_topology_device(sc), lib.ref_topology(sc))


def _same_wide(sc):
    from cpppt import lib
    dn, do, dd, df = lib.wide_bvh(sc, on_device=True)
    hn, ho, hd, hf = lib.wide_bvh(sc, on_device=False)
    assert dn.shape == hn.shape, (dn.shape, hn.shape)
    assert np.array_equal(dn, hn)
    assert np.array_equal(do, ho)
    assert (dd, df) == (hd, hf)
    return dn


def _tiny(n, seed=0):
    sc = scenes.soup(seed=seed, n_spheres=4, freq=1, width=8, height=8)
    sc.triangles = sc.triangles[:n].copy()  # geometry only: the tree builds read nothing else
    return sc


@pytest.mark.parametrize("name", sorted(SMALL_SCENES))
def test_device_wide_tree_matches_host_small(gpu_lib, name):
    """Device binned-SAH build and 4-wide collapse (csrc/gpu_sah.cu): the
    host build's nodes, leaf order, depth and inflation, byte for byte."""
    _same_wide(SMALL_SCENES[name]())


@pytest.mark.parametrize("n", [1, 2, 3, 5, 17, 300])
def test_device_wide_tree_matches_host_tiny(gpu_lib, n):
    _same_wide(_tiny(n))


def test_device_wide_tree_coincident_and_flat(gpu_lib):
    """Blocks of coincident triangles (no SAH split: halved in insertion
    order, in the level-synchronous top levels for 40000 copies and inside a
    subtree for 100), a flat scene (one axis without extent) and signed
    zeros."""
    sc = scenes.soup(seed=9, n_spheres=1000, freq=4, width=8, height=8)
    sc.triangles[1000:41000] = sc.triangles[7]
    sc.triangles[50000:50100] = sc.triangles[9]
    _same_wide(sc)
    flat = scenes.soup(seed=12, n_spheres=200, freq=2, width=8, height=8)
    flat.vertices = flat.vertices.copy()
    flat.vertices[:, 2] = np.float32(3.0)
    _same_wide(flat)
    z = scenes.soup(seed=11, n_spheres=150, freq=3, width=8, height=8, extent=4.0)
    rng = np.random.default_rng(3)
    v = z.vertices.copy()
    pick = rng.random(v.shape) < 0.25
    v[pick] = np.round(v[pick])
    v[(v == 0) & (rng.random(v.shape) < 0.5)] = np.float32(-0.0)
    z.vertices = v
    _same_wide(z)


@pytest.mark.parametrize("make", [lambda: scenes.soup(seed=2),
                                  lambda: scenes.slit_room(seed=4, n_boxes=1000, box_subdiv=4)],
                         ids=["soup1M", "slitroom192k"])
def test_device_wide_tree_full_size(gpu_lib, make):
    """Full size, and the device build repeated: atomics decide only node
    numbering inside the build, never the output."""
    from cpppt import lib
    sc = make()
    nodes = _same_wide(sc)
    assert len(nodes) > 10000
    for _ in range(4):
        again = lib.wide_bvh(sc, on_device=True)[0]
        assert np.array_equal(again, nodes)
