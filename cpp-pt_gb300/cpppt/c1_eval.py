"""Config 1 (the reference's CPU-runnable case): the Cornell box at 256x256,
64 spp (spp_axis 8), depth 8.  Times this library's render (device time of
the call, after a warm-up) and prints one JSON line.

    python -m cpppt.c1_eval [--repeats 10]
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import scenes
from .lib import GpuScene


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--repeats", type=int, default=10)
    a = ap.parse_args()
    sc = scenes.cornell(256, 256)
    paths = sc.width * sc.height * 64
    gs = GpuScene(sc)
    gs.render(64, max_depth=8, seed=1)  # warm-up
    ms = []
    for r in range(a.repeats):
        gs.render(64, max_depth=8, seed=100 + r)
        ms.append(gs.stats()["render_ms"])
    out = {"workload": "Cornell box 256x256, 64 spp, depth 8 (36 triangles)", "paths": paths,
           "gpu_ms_median": float(np.median(ms)), "gpu_mpaths_s": paths / (float(np.median(ms)) / 1000.0) / 1e6}
    print(json.dumps(out))


if __name__ == "__main__":
    main()
