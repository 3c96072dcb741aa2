"""Equal-time comparison of learned guiding, plain PT and SD-tree guiding on
the occluded-light room (emitter behind a 0.05-wide slit, indirect light
dominates).

    python -m cpppt.guiding_eval [--budgets 10 30 60] [--ref-spp 4096]

All three estimators converge to the same image on this all-Lambert scene
(albedo <= 0.8 keeps the Russian-roulette survival below 1), so each is
scored by relMSE = mean (x - ref)^2 / (ref^2 + 1e-2) against one
high-spp reference rendered with the plain tracer (PT_FLAG_UNBIASED_MIS):

* plain  -- PT + NEE + MIS, BSDF sampling only (PT_FLAG_UNBIASED_MIS);
* nn     -- PT + NEE + MIS with the learned vMF-mixture guide, trained
            online from fresh weights inside the time budget;
* sdtree -- the reference's practical path guiding (PPG: SD-tree, no NEE),
            one render whose spp is sized to the budget.

Prints one JSON line per method and budget, then a summary with the time
each method needs to reach plain PT's relMSE at the largest budget.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import scenes
from .lib import FLAG_UNBIASED_MIS, MODE_MIS, MODE_NN, MODE_SDTREE, GpuScene


def rel_mse(x, ref):
    return float(np.mean((x - ref) ** 2 / (ref ** 2 + 1e-2)))


def progressive(gs, mode, flags, budget_s, chunk_spp, depth, seed0, ref, checkpoints):
    """Renders chunks until the budget is spent; returns [(elapsed, spp, relMSE)] at each checkpoint."""
    acc = None
    spp_total = 0
    out = []
    t0 = time.perf_counter()
    k = 0
    cps = sorted(checkpoints)
    while True:
        img = gs.render(chunk_spp, max_depth=depth, seed=seed0 + k, mode=mode, flags=flags)
        k += 1
        acc = img * chunk_spp if acc is None else acc + img * chunk_spp
        spp_total += chunk_spp
        el = time.perf_counter() - t0
        while cps and el >= cps[0]:
            out.append((cps.pop(0), spp_total, rel_mse(acc / spp_total, ref)))
        if not cps or el >= budget_s:
            break
    return out, acc / spp_total, spp_total


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--budgets", type=float, nargs="+", default=[10, 30, 60])
    ap.add_argument("--ref-spp", type=int, default=4096)
    ap.add_argument("--width", type=int, default=1280)
    ap.add_argument("--height", type=int, default=720)
    ap.add_argument("--boxes", type=int, default=1000)
    ap.add_argument("--depth", type=int, default=12)
    ap.add_argument("--chunk", type=int, default=4)
    ap.add_argument("--save", default="")
    a = ap.parse_args()
    sc = scenes.slit_room(seed=4, n_boxes=a.boxes, box_subdiv=4, width=a.width, height=a.height)
    gs = GpuScene(sc)
    # reference: plain (unbiased) PT at ref_spp, rendered in chunks
    t0 = time.perf_counter()
    ref = None
    step = 256
    for k in range(0, a.ref_spp, step):
        img = gs.render(step, max_depth=a.depth, seed=777000 + k, mode=MODE_MIS, flags=FLAG_UNBIASED_MIS)
        ref = img if ref is None else ref + img
    ref /= a.ref_spp // step
    ref_s = time.perf_counter() - t0
    print(json.dumps({"reference": {"spp": a.ref_spp, "seconds": ref_s, "mean": float(ref.mean()),
                                    "triangles": sc.n_triangles, "resolution": [a.width, a.height]}}), flush=True)
    # warm-up (graph capture, allocations, kernel loading)
    gs.render(1, max_depth=a.depth, seed=1, mode=MODE_MIS, flags=FLAG_UNBIASED_MIS)
    gs.render(1, max_depth=a.depth, seed=1, mode=MODE_NN)
    B = max(a.budgets)
    results = {}
    res_plain, img_plain, spp_plain = progressive(gs, MODE_MIS, FLAG_UNBIASED_MIS, B, a.chunk, a.depth, 10_000, ref,
                                                  a.budgets)
    results["plain"] = res_plain
    gs.nn_reset(2024)
    res_nn, img_nn, spp_nn = progressive(gs, MODE_NN, 0, B, a.chunk, a.depth, 20_000, ref, a.budgets)
    results["nn"] = res_nn
    nn_stats = gs.nn_stats()
    # SD-tree: time one pass size, then one render per budget
    t0 = time.perf_counter()
    gs.render(4, max_depth=a.depth, seed=5, mode=MODE_SDTREE)
    t4 = time.perf_counter() - t0
    res_sd = []
    for bud in a.budgets:
        spp = 4
        while spp * 2 * t4 / 3.0 * 2 < bud * 3 and spp < 1 << 16:  # passes 1..spp/2 cost ~ spp paths
            spp *= 2
        t0 = time.perf_counter()
        img = gs.render(spp, max_depth=a.depth, seed=30_000 + spp, mode=MODE_SDTREE)
        el = time.perf_counter() - t0
        res_sd.append((el, spp, rel_mse(img, ref)))
    results["sdtree"] = res_sd
    for name, rows in results.items():
        for el, spp, r in rows:
            print(json.dumps({"method": name, "seconds": el, "spp": spp, "relMSE": r}), flush=True)
    # time for each method to reach plain's relMSE at the largest budget
    target = res_plain[-1][2]
    summ = {"target_relMSE_plain_at_s": [res_plain[-1][0], target], "nn_training": nn_stats}
    for name in ("nn", "sdtree"):
        reach = [el for el, spp, r in results[name] if r <= target]
        summ[f"{name}_reaches_target_at_s"] = min(reach) if reach else None
    print(json.dumps({"summary": summ}), flush=True)
    if a.save:
        np.savez_compressed(a.save, ref=ref, plain=img_plain, nn=img_nn)


if __name__ == "__main__":
    main()
