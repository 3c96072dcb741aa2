"""Host-only checks of the C ABI library (no CUDA call)."""
import os
import re

import numpy as np
import pytest

from tests.golden.make_golden import SMALL_SCENES

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    src = open(os.path.join(ROOT, "include", "cpppt_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(pt_[a-z_]+)\s*\(", src)))


def test_library_exports_every_declared_function():
    from cpppt import lib
    L = lib.load()
    names = header_functions()
    assert len(names) >= 12
    for n in names:
        assert hasattr(L, n), n
    assert sorted(lib.EXPORTS) == names


@pytest.mark.parametrize("name", sorted(SMALL_SCENES))
def test_product_ref_topology_matches_reference(golden, name):
    """The library's own rebuild of BVH::build equals the reference's tree."""
    from cpppt import lib
    g = golden(f"{name}_ref.npz")
    order, boxes, pparent = lib.ref_topology(SMALL_SCENES[name]())
    assert np.array_equal(order, g["leaf_order"])
    assert np.array_equal(boxes.view(np.uint32), g["node_boxes"].view(np.uint32))
    assert np.array_equal(pparent, g["prim_parent"])


def test_product_ref_topology_large_matches_oracle():
    from cpppt import lib, scenes
    from oracle.oracle import Oracle
    sc = scenes.soup(seed=5, n_spheres=300, freq=4, width=8, height=8)
    order, boxes, pparent = lib.ref_topology(sc)
    o_order, o_boxes, _, o_pparent = Oracle("port").scene(sc).bvh_dump()
    assert np.array_equal(order, o_order)
    assert np.array_equal(boxes.view(np.uint32), o_boxes.view(np.uint32))
    assert np.array_equal(pparent, o_pparent)


def test_errors_are_status_codes():
    from cpppt import lib
    L = lib.load()
    import ctypes as C
    nn = C.c_int32()
    assert L.pt_debug_ref_topology(None, -1, None, None, None, 0, C.byref(nn)) == 1
    assert b"bad argument" in L.pt_last_error()


def test_parallel_ref_topology_matches_oracle():
    """Above 2 x 16384 primitives per side the library builds independent
    subtrees on separate threads and joins them in pre-order: the tree must
    stay the reference's, here on 320k triangles plus a block of coincident
    copies (the reference's endless-recursion case becomes one leaf)."""
    from cpppt import lib, scenes
    from oracle.oracle import Oracle
    sc = scenes.soup(seed=9, n_spheres=1000, freq=4, width=8, height=8)
    sc.triangles[1000:41000] = sc.triangles[7]  # 40000 coincident copies of one triangle
    order, boxes, pparent = lib.ref_topology(sc)
    o_order, o_boxes, _, o_pparent = Oracle("port").scene(sc).bvh_dump()
    assert len(order) > 300_000
    assert np.array_equal(order, o_order)
    assert np.array_equal(boxes.view(np.uint32), o_boxes.view(np.uint32))
    assert np.array_equal(pparent, o_pparent)


def test_wide_bvh_host_build_is_thread_independent():
    """The host 4-wide SAH build keeps every node's triangles in insertion
    order (stable partitions; halving in that order where no SAH split
    exists), so its bytes do not depend on how many threads build
    independent subtrees -- the property the device build relies on to
    reproduce it.  320k triangles (above the 65536-triangle threading
    threshold) plus a block of coincident copies and a smaller one."""
    from cpppt import lib, scenes
    sc = scenes.soup(seed=9, n_spheres=1000, freq=4, width=8, height=8)
    sc.triangles[1000:41000] = sc.triangles[7]   # 40000 coincident copies
    sc.triangles[50000:50100] = sc.triangles[9]  # 100 more
    n1, o1, d1, f1 = lib.wide_bvh(sc, on_device=False, host_threads=1)
    n16, o16, d16, f16 = lib.wide_bvh(sc, on_device=False, host_threads=16)
    assert np.array_equal(n1, n16) and np.array_equal(o1, o16) and d1 == d16 and f1 == f16
    assert np.array_equal(np.sort(o1), np.arange(sc.n_triangles))
    # every leaf's triangles ascend by insertion index
    refs = n1[:, 10:14].reshape(-1)
    leaves = refs[(refs != 0xFFFFFFFF) & (refs >> 31 == 1)]
    start, count = leaves & 0x7FFFFFF, ((leaves >> 27) & 15) + 1
    assert count.sum() == sc.n_triangles
    for s, c in zip(start[:5000], count[:5000]):
        assert np.all(np.diff(o1[s:s + c]) > 0)


def test_wide_bvh_debug_entry_checks_its_arguments():
    """pt_debug_wide_bvh (host build, no CUDA call): a leaf size outside
    [1, 16] is refused, an empty list gives an empty tree, and a node buffer
    that is too small gives PT_ERR_LIMIT with the node count set."""
    import ctypes as C
    from cpppt import lib, scenes
    L = lib.load()
    sc = scenes.cornell(8, 8)
    tv = np.ascontiguousarray(sc.vertices[sc.triangles].reshape(-1), np.float32)
    n = sc.n_triangles
    order = np.zeros(n, np.int32)
    nodes = np.zeros((64, 16), np.uint32)
    nn, depth, infl = C.c_int32(), C.c_int32(), C.c_float()
    args = lambda leaf, cap: (tv.ctypes.data, n, leaf, 0, 1, nodes.ctypes.data, cap, C.byref(nn),
                              order.ctypes.data, C.byref(depth), C.byref(infl))
    assert L.pt_debug_wide_bvh(*args(0, 64)) == 1 and L.pt_debug_wide_bvh(*args(17, 64)) == 1
    assert L.pt_debug_wide_bvh(*args(4, 64)) == 0
    full = nn.value
    assert full >= 2 and depth.value >= 2 and infl.value > 0
    assert np.array_equal(np.sort(order), np.arange(n))
    assert L.pt_debug_wide_bvh(*args(4, full - 1)) == 4  # PT_ERR_LIMIT
    assert nn.value == full
    assert L.pt_debug_wide_bvh(None, 0, 4, 0, 1, nodes.ctypes.data, 64, C.byref(nn), None, C.byref(depth),
                               None) == 0
    assert nn.value == 1  # a root with no children
