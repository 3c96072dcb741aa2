"""Small, fixed workloads for profiling single kernels (ncu -k ... -c 1..3).

    python -m cpppt.profile_cases extend   # 1M-tri soup, 1280x720, 1 spp, depth 10 (plain PT+NEE+MIS)
    python -m cpppt.profile_cases nn [R]   # 200k-tri slit room, 640x360, learned guide: R renders of 4 spp
    python -m cpppt.profile_cases slit [R] # the same renders with plain PT (PT_FLAG_UNBIASED_MIS)
    python -m cpppt.profile_cases batch    # 8 soup scenes (10k-160k tris) in one batched wavefront

Each case renders once to warm up (graph capture, allocation), then once
more: the second render is the one to capture.  Device memory stays at a
few GB.  The path state (about 400 MB at 2^21 paths in flight) exceeds the
129 MB L2; the soup's traversal data (about 70 MB) fits in it.
"""
from __future__ import annotations

import sys
import time

from . import scenes
from .lib import FLAG_UNBIASED_MIS, MODE_MIS, MODE_NN, GpuBatch, GpuScene


def case_extend():
    gs = GpuScene(scenes.soup(seed=2, width=1280, height=720))
    for _ in range(2):
        gs.render(1, max_depth=10, seed=1, mode=MODE_MIS)
    return gs.stats()


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


def main():
    name = sys.argv[1] if len(sys.argv) > 1 else "extend"
    fn = {"extend": case_extend, "nn": case_nn, "slit": case_slit, "batch": case_batch}[name]
    t0 = time.perf_counter()
    st = fn(int(sys.argv[2])) if name in ("nn", "slit") and len(sys.argv) > 2 else fn()
    print(name, {k: v for k, v in st.items() if v}, f"{time.perf_counter() - t0:.1f}s")


if __name__ == "__main__":
    main()
