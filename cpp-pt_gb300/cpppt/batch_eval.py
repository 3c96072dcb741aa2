"""Batched plain PT over many seeded soup scenes in one wavefront.

    python -m cpppt.batch_eval [--scenes 64] [--seed 3] [--spp-scale 1]

Scene k: triangle count log-uniform in [min_tris, max_tris] (geodesic
spheres of 500 triangles, materials and lights as the 1M-triangle soup),
resolution uniform over {256^2, 512^2, 1024^2}, spp uniform over
{16, 64, 256} (times spp_scale), max depth 10.  Prints one JSON line per
phase: scene build, autotuning, the batched render (aggregate Mpaths/s and
Mrays/s), the same jobs rendered one pt_render call at a time, and the
bit-exact parity of the smallest jobs against their unbatched renders.
"""
from __future__ import annotations

import argparse
import json
import math
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np

from . import scenes
from .lib import GpuBatch, GpuScene


def plan(n: int, seed: int, min_tris: int, max_tris: int, spp_scale: float):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        tris = math.exp(rng.uniform(math.log(min_tris), math.log(max_tris)))
        res = int(rng.choice([256, 512, 1024]))
        spp = int(rng.choice([16, 64, 256]))
        out.append(dict(n_spheres=max(1, int(round(tris / 500))), res=res, spp=max(1, int(round(spp * spp_scale))),
                        scene_seed=1000 + k))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--scenes", type=int, default=64)
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--min-tris", type=int, default=10_000)
    ap.add_argument("--max-tris", type=int, default=2_000_000)
    ap.add_argument("--spp-scale", type=float, default=1.0)
    ap.add_argument("--depth", type=int, default=10)
    ap.add_argument("--threads", type=int, default=8)
    ap.add_argument("--autotune-div", type=int, default=32, help="0: no autotuning")
    ap.add_argument("--parity", type=int, default=8, help="smallest jobs checked against unbatched renders")
    ap.add_argument("--no-sequential", action="store_true")
    a = ap.parse_args()

    p = plan(a.scenes, a.seed, a.min_tris, a.max_tris, a.spp_scale)
    t0 = time.perf_counter()

    gen_s, create_s = [], []

    def make(q):
        t1 = time.perf_counter()
        sc = scenes.soup(seed=q["scene_seed"], n_spheres=q["n_spheres"], width=q["res"], height=q["res"])
        t2 = time.perf_counter()
        gs = GpuScene(sc)
        gen_s.append(t2 - t1)
        create_s.append(time.perf_counter() - t2)
        return gs

    with ThreadPoolExecutor(a.threads) as ex:
        members = list(ex.map(make, p))
    t_build = time.perf_counter() - t0
    tris = [m.n_triangles for m in members]
    jobs = [dict(scene=k, spp=q["spp"], max_depth=a.depth, seed=a.seed * 1000003 + k) for k, q in enumerate(p)]
    paths = sum(q["res"] * q["res"] * q["spp"] for q in p)
    print(json.dumps({"phase": "build", "scenes": a.scenes, "triangles": int(sum(tris)), "min_tris": min(tris),
                      "max_tris": max(tris), "paths": paths, "seconds": t_build,
                      "soup_generation_thread_seconds": sum(gen_s), "scene_create_thread_seconds": sum(create_s)}),
          flush=True)

    t0 = time.perf_counter()
    b = GpuBatch(members)
    t_merge = time.perf_counter() - t0
    if a.autotune_div > 0:
        t0 = time.perf_counter()
        best, rate = b.autotune(jobs, spp_divisor=a.autotune_div)
        print(json.dumps({"phase": "autotune", "tuning": best, "sample_mpaths_s": rate,
                          "seconds": time.perf_counter() - t0, "merge_seconds": t_merge}), flush=True)
    b.render(jobs, outputs=False)  # warm-up at the final shape
    t0 = time.perf_counter()
    b.render(jobs, outputs=False)
    wall = time.perf_counter() - t0
    st = b.stats()
    rays = st["closest_rays"] + st["shadow_rays"]
    print(json.dumps({"phase": "batched", "mpaths_s": st["paths"] / (st["render_ms"] * 1e3),
                      "mrays_s": rays / (st["render_ms"] * 1e3), "render_ms": st["render_ms"], "wall_s": wall,
                      "paths": st["paths"], "closest_rays": st["closest_rays"], "shadow_rays": st["shadow_rays"],
                      "kernel_launches": st["kernel_launches"], "tuning": b.tuning()}), flush=True)

    if not a.no_sequential:
        ms = 0.0
        for j in jobs:
            members[j["scene"]].render(j["spp"], max_depth=j["max_depth"], seed=j["seed"])
            ms += members[j["scene"]].stats()["render_ms"]
        print(json.dumps({"phase": "sequential", "mpaths_s": paths / (ms * 1e3), "render_ms": ms,
                          "batched_speedup": ms / st["render_ms"]}), flush=True)

    if a.parity > 0:
        order = sorted(range(len(jobs)), key=lambda k: p[k]["res"] ** 2 * p[k]["spp"])[:a.parity]
        sub = [jobs[k] for k in order]
        imgs = b.render(sub)
        same = []
        for j, img in zip(sub, imgs):
            ref = members[j["scene"]].render(j["spp"], max_depth=j["max_depth"], seed=j["seed"])
            same.append(bool(np.array_equal(img.view(np.uint32), ref.view(np.uint32))))
        print(json.dumps({"phase": "parity", "jobs": order, "bit_identical": same}), flush=True)


if __name__ == "__main__":
    main()
