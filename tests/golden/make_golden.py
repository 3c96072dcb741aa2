"""Generates the golden fixtures in tests/golden from the reference itself.

Run in a container where the reference sources are mounted (the oracle
harness, oracle/ref_harness.cpp, is compiled from them by
oracle/build_ref.sh):

    python tests/golden/make_golden.py            # small fixtures (seconds)
    python tests/golden/make_golden.py --c1-16k   # 16k-spp Cornell reference (~15 min on 8 cores)
    python tests/golden/make_golden.py --textures # textured room (tests/texscene.py), 16 x 64 spp

Every array stored here is an output of the reference's own code
(BVH::build, BVH::intersect / intersect_any, PathtracerMIS::render,
Pathtracer::render, PurePt::render) on the
seeded scenes of cpppt.scenes.  Inputs (rays) are stored next to the outputs
so the fixtures do not depend on numpy's random streams.
"""
from __future__ import annotations

import argparse
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "cpp-pt_gb300"))
sys.path.insert(0, ROOT)

from cpppt import scenes  # noqa: E402
from oracle import oracle as orc  # noqa: E402

SMALL_SCENES = {
    "cornell": lambda: scenes.cornell(32, 32),
    "soup": lambda: scenes.soup(seed=2, n_spheres=60, freq=3, width=24, height=16),
    "slitroom": lambda: scenes.slit_room(seed=4, n_boxes=20, box_subdiv=2, width=24, height=16),
}


def small():
    orc.build_reference()
    ref = orc.Oracle("reference")
    for name, make in SMALL_SCENES.items():
        sc = make()
        rs = ref.scene(sc)
        order, boxes, parent, pparent = rs.bvh_dump()
        rays = scenes.hit_ray_batch(sc, 4096, seed=6)
        idx, t = rs.trace_closest(rays)
        # shadow-style queries: the same rays limited to 0.999 of the hit
        sh = rays.copy()
        sh[:, 6] = np.where(np.isfinite(t), t * np.float32(0.999), np.float32(3.0))
        occ = rs.trace_any(sh)
        img, _ = rs.render_mis(2, 8, 0, threads=1)
        img32, _ = rs.render_mis(1, 32, 7, threads=1)
        # the reference's other two integrators (Pathtracer: NEE without MIS; PurePt)
        nee, _ = rs.render_variant(1, 2, 8, 3, threads=1)
        pure, _ = rs.render_variant(2, 2, 8, 3, threads=1)
        np.savez_compressed(
            os.path.join(HERE, f"{name}_ref.npz"),
            leaf_order=order, node_boxes=boxes, node_parent=parent, prim_parent=pparent,
            rays=rays, hit_index=idx, hit_t=t, shadow_rays=sh, occluded=occ,
            render_spp2_d8=img, render_spp1_d32_seed7=img32,
            render_nee_spp2_d8_seed3=nee, render_pure_spp2_d8_seed3=pure)
        print(name, sc.n_triangles, "tris;", (idx >= 0).mean(), "hit rate")


def c1_16k(replicas: int = 16, spp_axis: int = 32, depth: int = 8, tile: int = 16):
    """16 independent reference renders of the 256x256 Cornell box at
    spp_axis^2 = 1024 spp (16384 spp in total), depth 8.  Replica r seeds
    column i with i + 1000 * (r + 1).  Stores the mean image and the per-tile
    means of every replica (for the per-tile z-test)."""
    orc.build_reference()
    sc = scenes.cornell(256, 256)
    rs = orc.Oracle("reference").scene(sc)
    imgs = []
    t0 = time.time()
    for r in range(replicas):
        img, sec = rs.render_mis(spp_axis, depth, 1000 * (r + 1))
        imgs.append(img)
        print(f"replica {r}: {sec:.1f}s", flush=True)
    imgs = np.stack(imgs)
    H, W = sc.height, sc.width
    tiles = imgs.reshape(replicas, H // tile, tile, W // tile, tile, 3).mean(axis=(2, 4))
    np.savez_compressed(
        os.path.join(HERE, "cornell256_16k_ref.npz"),
        mean=imgs.mean(0).astype(np.float32), tile_means=tiles.astype(np.float32),
        replicas=replicas, spp_per_replica=spp_axis * spp_axis, depth=depth, tile=tile,
        seconds=time.time() - t0)
    print("done", time.time() - t0)


def textured(replicas: int = 16, spp_axis: int = 8, depth: int = 8, tile: int = 8):
    """The textured room of tests/texscene.py (image textures: tiled albedo,
    metal and roughness maps, normal map, emission texture), loaded by the
    reference's own Loader and rendered by its PathtracerMIS: replicas of
    spp_axis^2 spp, replica r seeding column i with i + 500 * (r + 1).
    Stores the mean image and the per-tile means of every replica."""
    import tempfile
    from tests import texscene
    orc.build_reference()
    d = tempfile.mkdtemp()
    rs = orc.Oracle("reference").load_files(texscene.write(d))
    imgs = []
    t0 = time.time()
    for r in range(replicas):
        img, _ = rs.render_mis(spp_axis, depth, 500 * (r + 1))
        imgs.append(img)
    imgs = np.stack(imgs)
    H, W = texscene.H, texscene.W
    tiles = imgs.reshape(replicas, H // tile, tile, W // tile, tile, 3).mean(axis=(2, 4))
    np.savez_compressed(
        os.path.join(HERE, "texroom_ref.npz"),
        mean=imgs.mean(0).astype(np.float32), tile_means=tiles.astype(np.float32),
        replicas=replicas, spp_per_replica=spp_axis * spp_axis, depth=depth, tile=tile)
    print("textured room", time.time() - t0, "s; mean", float(imgs.mean()))


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--c1-16k", action="store_true")
    ap.add_argument("--textures", action="store_true")
    a = ap.parse_args()
    if a.c1_16k:
        c1_16k()
    elif a.textures:
        textured()
    else:
        small()
