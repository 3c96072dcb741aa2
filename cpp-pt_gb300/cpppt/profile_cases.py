"""Small, fixed workloads for profiling single kernels (ncu -k ... -c 1..3).

    python -m cpppt.profile_cases extend   # 1M-tri soup, 1280x720, 1 spp, depth 10 (plain PT+NEE+MIS),
                                           # kernels launched one by one (ncu-visible)
    python -m cpppt.profile_cases raycounts  # extension rays of each bounce of that render
    python -m cpppt.profile_cases nn [R]   # 200k-tri slit room, 640x360, learned guide: R renders of 4 spp
    python -m cpppt.profile_cases slit [R] # the same renders with plain PT (PT_FLAG_UNBIASED_MIS)
    python -m cpppt.profile_cases batch    # 8 soup scenes (10k-160k tris) in one batched wavefront
    python -m cpppt.profile_cases batchnn [R]    # 8 slit rooms (50k-430k tris), 640x360, one learned
                                                 # guide each, trained online: R batched renders of 2 spp
    python -m cpppt.profile_cases batchslit [R]  # the same batches with plain PT (PT_FLAG_UNBIASED_MIS)
    python -m cpppt.profile_cases c5 [R] [plain|train|frozen]  # the eight 1080p rooms of
                                                 # batch_guiding_eval (11.4M tris): R batched renders of 2 spp

Each case renders once to warm up (graph capture, allocation), then once
more: the second render is the one to capture.  Device memory stays at a
few GB.  The path state (about 180 MB for the extend case's 921,600 paths in flight) exceeds the
129 MB L2; the soup's traversal data (about 70 MB) fits in it.
"""
from __future__ import annotations

import sys
import time

from . import scenes
from .lib import FLAG_NN_FREEZE, FLAG_TIME_KERNELS, FLAG_UNBIASED_MIS, MODE_MIS, MODE_NN, GpuBatch, GpuScene


def case_extend():
    """Renders with PT_FLAG_TIME_KERNELS: the same kernels launched one by one
    (16 iterations per round) instead of inside the device-driven graph,
    whose kernel nodes ncu cannot capture (a graph with a conditional node);
    each render here takes one round, so the second render's extension
    launches start at launch 16."""
    gs = GpuScene(scenes.soup(seed=2, width=1280, height=720))
    for _ in range(2):
        gs.render(1, max_depth=10, seed=1, mode=MODE_MIS, flags=FLAG_TIME_KERNELS)
    return gs.stats()


def case_raycounts():
    """Extension rays per bounce of the extend case.  All 921,600 paths start
    in the first iteration (the wavefront holds them all), and a path's random
    numbers depend only on its pixel, sample and bounce, so a render limited
    to depth b traces exactly the first b bounces of the depth-10 render:
    rays of bounce b = closest rays at depth b+1 minus those at depth b."""
    gs = GpuScene(scenes.soup(seed=2, width=1280, height=720))
    prev, per = 0.0, []
    for d in range(1, 11):
        gs.render(1, max_depth=d, seed=1, mode=MODE_MIS)
        c = gs.stats()["closest_rays"]
        per.append(int(c - prev))
        prev = c
    return {"rays_per_bounce": per, "total": int(prev)}


def case_nn(renders: int = 2):
    gs = GpuScene(scenes.slit_room(seed=4, n_boxes=1000, box_subdiv=4, width=640, height=360))
    gs.nn_reset(7)
    for k in range(renders):
        gs.render(4, max_depth=12, seed=10 + k, mode=MODE_NN)
    return {**gs.stats(), **gs.nn_stats()}


def case_slit(renders: int = 2):
    gs = GpuScene(scenes.slit_room(seed=4, n_boxes=1000, box_subdiv=4, width=640, height=360))
    for k in range(renders):
        gs.render(4, max_depth=12, seed=10 + k, mode=MODE_MIS, flags=FLAG_UNBIASED_MIS)
    return gs.stats()


def case_batch():
    members = [GpuScene(scenes.soup(seed=300 + k, n_spheres=20 * 2 ** (k % 5), width=256 << (k % 3),
                                    height=256 << (k % 3))) for k in range(8)]
    jobs = [dict(scene=k, spp=4, max_depth=10, seed=k) for k in range(8)]
    b = GpuBatch(members)
    for _ in range(2):
        b.render(jobs, outputs=False)
    return b.stats()


def _rooms():
    members = [GpuScene(scenes.slit_room(seed=5 + k, n_boxes=1000, box_subdiv=2 + k % 5, width=640, height=360))
               for k in range(8)]
    return members, GpuBatch(members)


def case_batchnn(renders: int = 3):
    members, b = _rooms()
    for k, g in enumerate(members):
        g.nn_reset(2024 + k)
    for r in range(renders):
        b.render([dict(scene=k, spp=2, max_depth=12, seed=100 * r + k) for k in range(8)], outputs=False,
                 mode=MODE_NN)
    return {**b.stats(), "steps": sum(g.nn_stats()["steps"] for g in members)}


def case_batchslit(renders: int = 3):
    members, b = _rooms()
    for r in range(renders):
        b.render([dict(scene=k, spp=2, max_depth=12, seed=100 * r + k) for k in range(8)], outputs=False,
                 mode=MODE_MIS, flags=FLAG_UNBIASED_MIS)
    return b.stats()


def case_c5(renders: int = 2, what: str = "train"):
    from .batch_guiding_eval import plan
    members = [GpuScene(scenes.slit_room(seed=q["scene_seed"], n_boxes=1000, box_subdiv=q["box_subdiv"], width=1920,
                                         height=1080)) for q in plan(8, 5, 5e5, 4e6)]
    b = GpuBatch(members)
    for k, g in enumerate(members):
        g.nn_reset(2024 + k)
    mode, flags = (MODE_MIS, FLAG_UNBIASED_MIS) if what == "plain" else (MODE_NN, FLAG_NN_FREEZE if what == "frozen"
                                                                         else 0)
    out = []
    for r in range(renders):
        b.render([dict(scene=k, spp=2, max_depth=12, seed=100 * r + k) for k in range(8)], outputs=False,
                 mode=mode, flags=flags)
        st = b.stats()
        out.append(round(st["paths"] / (st["render_ms"] * 1e3), 1))
    return {**b.stats(), "mpaths_s_per_render": out, "steps": sum(g.nn_stats()["steps"] for g in members)}


def main():
    name = sys.argv[1] if len(sys.argv) > 1 else "extend"
    fn = {"extend": case_extend, "raycounts": case_raycounts, "nn": case_nn, "slit": case_slit, "batch": case_batch, "batchnn": case_batchnn,
          "batchslit": case_batchslit, "c5": case_c5}[name]
    t0 = time.perf_counter()
    args = [int(sys.argv[2])] if len(sys.argv) > 2 else []
    args += sys.argv[3:4]
    st = fn(*args) if name in ("nn", "slit", "batchnn", "batchslit", "c5") else fn()
    print(name, {k: v for k, v in st.items() if v}, f"{time.perf_counter() - t0:.1f}s")


if __name__ == "__main__":
    main()
