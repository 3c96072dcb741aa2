"""The SD-tree update (row a14) against the reference's own SDTree.

Both the reference (oracle harness, src/algorithms/sdtree.h) and the
library's host port (pt_debug_sdtree_run) receive the same rounds of splats
and run update() after each; the resulting trees -- every spatial leaf's
sampling leaves, splat counts and flux -- and the pdfs of query directions
must be identical bit for bit.  Splats are concentrated so spatial leaves
exceed the 12000 * int(2^(k/2)) split threshold and split several times."""
import numpy as np
import pytest


def make_rounds(seed, sizes):
    rng = np.random.default_rng(seed)
    rounds = []
    for n in sizes:
        # a dense cluster of positions plus a uniform background; directions
        # around one lobe; a tenth of the records carry no radiance
        pos = np.where(rng.random((n, 1)) < 0.7, rng.normal([2, 2, 2], 0.6, (n, 3)), rng.uniform(0, 10, (n, 3)))
        d = rng.normal([0.3, -0.2, 0.8], 0.5, (n, 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        rad = rng.exponential(1.0, (n, 1)) * (rng.random((n, 1)) < 0.9)
        rounds.append(np.hstack([rad, pos, d]).astype(np.float32))
    return rounds


def queries(seed, n=2000):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0, 10, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.hstack([pos, d]).astype(np.float32)


@pytest.mark.parametrize("sizes", [[5000], [30000, 60000], [20000, 50000, 120000]])
def test_sdtree_update_matches_reference(sizes):
    from cpppt import lib
    from oracle import oracle as orc
    if not orc.reference_available():
        pytest.skip("reference harness not built in this environment")
    ref_fn = orc.Oracle("reference").lib.ref_sdtree_run
    lo, hi = [0, 0, 0], [10, 10, 10]
    rounds = make_rounds(7, sizes)
    q = queries(8)
    ours = lib.sdtree_run(lo, hi, rounds, q)
    ref = lib.sdtree_run(lo, hi, rounds, q, fn=ref_fn)
    assert len(ours["leaf_counts"]) == len(ref["leaf_counts"])
    if len(sizes) > 1:
        assert len(ref["leaf_counts"]) > 1  # the spatial tree did split
    np.testing.assert_array_equal(ours["leaf_counts"], ref["leaf_counts"])
    np.testing.assert_array_equal(ours["counts"], ref["counts"])
    np.testing.assert_array_equal(ours["flux"].view(np.uint32), ref["flux"].view(np.uint32))
    np.testing.assert_array_equal(ours["leaves"].view(np.uint32), ref["leaves"].view(np.uint32))
    np.testing.assert_array_equal(ours["pdf"].view(np.uint32), ref["pdf"].view(np.uint32))


def test_fresh_sdtree_is_uniform_sphere():
    from cpppt import lib
    out = lib.sdtree_run([0, 0, 0], [1, 1, 1], [], queries(1, 10))
    assert len(out["leaf_counts"]) == 1 and out["leaf_counts"][0] == 1
    np.testing.assert_allclose(out["pdf"], 1.0 / (4 * np.pi), rtol=1e-6)
