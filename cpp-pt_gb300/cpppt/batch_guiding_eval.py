"""Learned guiding batched at scale: eight occluded-light rooms (the slit
room generator with seeds 5..12, triangle counts log-uniform in
[500k, 4M] reached by the boxes' face subdivision), 1920x1080, max depth
12, rendered as one batch (pt_batch_render_ex), each room guided by its own
network that trains online from its own paths.

    python -m cpppt.batch_guiding_eval [--budgets 10 20 40] [--ref-spp 4096]

Methods, all batched over the eight rooms except the SD-tree:

* plain  -- PT + NEE + MIS with BSDF sampling (PT_MODE_MIS |
            PT_FLAG_UNBIASED_MIS) on the batched slot wavefront;
* nn     -- the same estimator with each room's learned vMF-mixture guide,
            trained from fresh weights inside the budget;
* sdtree -- the reference's practical path guiding (SD-tree, no NEE), one
            pt_render per room, its spp sized so the eight renders fill the
            largest budget.

Each method renders chunks of spp for all rooms per call and accumulates on
the GPU; the score at a checkpoint is the mean over rooms of relMSE =
mean((x - ref)^2 / (ref^2 + 1e-2)) against a plain batched reference of
ref_spp (two independent halves give its own noise, which is subtracted in
the noise-corrected columns).  Throughput lines give Mpaths/s over each
method's renders (the library's render time: wavefront, inference and
training).  Prints JSON lines and a final summary.
"""
from __future__ import annotations

import argparse
import json
import math
import time
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import torch

from . import scenes
from .guiding_eval import rel_mse, time_to_reach
from .lib import FLAG_NN_FREEZE, FLAG_THROUGHPUT_RR, FLAG_UNBIASED_MIS, MODE_MIS, MODE_NN, MODE_SDTREE, GpuBatch, GpuScene


def plan(n: int, seed: int, min_tris: float, max_tris: float):
    """Room k: slit room of seed `seed + k`, 1000 boxes whose faces are split
    s x s (12000 s^2 + 38 triangles) with s nearest to the drawn count.  The
    counts are drawn log-uniform in [min_tris, max_tris], stratified (one
    draw in each of n equal slices of the log range, in shuffled order) so
    that a batch of a few rooms spans the range; s is kept to the splits
    whose count lies inside it (7..18 for [0.5M, 4M]: 588k..3.89M)."""
    rng = np.random.default_rng(seed)
    lo, hi = math.log(min_tris), math.log(max_tris)
    s_min = max(1, math.ceil(math.sqrt(max(0.0, min_tris - 38) / 12000.0)))
    s_max = max(s_min, math.floor(math.sqrt(max(0.0, max_tris - 38) / 12000.0)))
    slices = rng.permutation(n)
    out = []
    for k in range(n):
        tris = math.exp(lo + (hi - lo) * (slices[k] + rng.uniform()) / n)
        s = min(s_max, max(s_min, int(round(math.sqrt(tris / 12000.0)))))
        out.append(dict(scene_seed=seed + k, box_subdiv=s))
    return out


def batch_progressive(b, n_rooms, shape, mode, flags, budget, chunk, depth, seed0, refs, cps, freeze_after=None):
    """Renders chunk spp of every room per call until the budget is spent;
    returns [(seconds, spp, mean relMSE)] at the checkpoints, the
    throughput and the images."""
    H, W = shape
    outs = [torch.zeros((H, W, 3), dtype=torch.float32, device="cuda") for _ in range(n_rooms)]
    accs = [torch.zeros((H, W, 3), dtype=torch.float64, device="cuda") for _ in range(n_rooms)]
    ptrs = [o.data_ptr() for o in outs]
    spp, k, paths, ms = 0, 0, 0.0, 0.0
    snaps, cps = [], sorted(cps)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    while True:
        f = flags
        if freeze_after is not None and time.perf_counter() - t0 >= freeze_after:
            f |= FLAG_NN_FREEZE
        jobs = [dict(scene=r, spp=chunk, max_depth=depth, seed=seed0 + 1000 * k + r) for r in range(n_rooms)]
        b.render_device(jobs, ptrs, mode=mode, flags=f)
        st = b.stats()
        paths += st["paths"]
        ms += st["render_ms"]
        for a, o in zip(accs, outs):
            a += o.double() * chunk
        k += 1
        spp += chunk
        el = time.perf_counter() - t0
        while cps and el >= cps[0]:
            snaps.append((cps.pop(0), spp, [(a / spp).float() for a in accs]))
        if not cps or el >= budget:
            break
    torch.cuda.synchronize()
    rows = [(t, s, float(np.mean([rel_mse(x, r) for x, r in zip(xs, refs)]))) for t, s, xs in snaps]
    return rows, {"mpaths_s": paths / (ms * 1e3), "renders": k, "spp": spp}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--rooms", type=int, default=8)
    ap.add_argument("--seed", type=int, default=5)
    ap.add_argument("--min-tris", type=float, default=5e5)
    ap.add_argument("--max-tris", type=float, default=4e6)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--depth", type=int, default=12)
    ap.add_argument("--budgets", type=float, nargs="+", default=[10, 20, 40])
    ap.add_argument("--ref-spp", type=int, default=4096)
    ap.add_argument("--ref-step", type=int, default=64)
    ap.add_argument("--chunk", type=int, default=2)
    ap.add_argument("--nn-config", action="append", default=None,
                    help="JSON settings for every room's GpuScene.nn_configure, optionally with \"freeze_after\" "
                         "(seconds of training) and \"throughput_rr\"; repeat to compare several settings")
    ap.add_argument("--no-sdtree", action="store_true")
    ap.add_argument("--threads", type=int, default=8)
    a = ap.parse_args()

    p = plan(a.rooms, a.seed, a.min_tris, a.max_tris)
    t0 = time.perf_counter()

    def make(q):
        return GpuScene(scenes.slit_room(seed=q["scene_seed"], n_boxes=1000, box_subdiv=q["box_subdiv"],
                                         width=a.width, height=a.height))

    with ThreadPoolExecutor(a.threads) as ex:
        rooms = list(ex.map(make, p))
    b = GpuBatch(rooms)
    tris = [g.n_triangles for g in rooms]
    print(json.dumps({"phase": "build", "rooms": a.rooms, "triangles": tris, "total_triangles": int(sum(tris)),
                      "resolution": [a.width, a.height], "depth": a.depth,
                      "seconds": time.perf_counter() - t0}), flush=True)
    n, H, W = a.rooms, a.height, a.width

    # reference: plain batched renders in two independent halves (FP64 sums)
    outs = [torch.zeros((H, W, 3), dtype=torch.float32, device="cuda") for _ in range(n)]
    halves = [[torch.zeros((H, W, 3), dtype=torch.float64, device="cuda") for _ in range(n)] for _ in range(2)]
    t0 = time.perf_counter()
    steps = a.ref_spp // a.ref_step
    for q in range(steps):
        jobs = [dict(scene=r, spp=a.ref_step, max_depth=a.depth, seed=777000 + 1000 * q + r) for r in range(n)]
        b.render_device(jobs, [o.data_ptr() for o in outs], mode=MODE_MIS, flags=FLAG_UNBIASED_MIS)
        for h, o in zip(halves[q & 1], outs):
            h += o.double()
    n_a, n_b = (steps + 1) // 2, max(1, steps // 2)
    refs = [((ha + hb) / steps).float() for ha, hb in zip(halves[0], halves[1])]
    ref_noise = float(np.mean([float((((ha / n_a).float() - (hb / n_b).float()) ** 2 / (r ** 2 + 1e-2)).mean())
                               for ha, hb, r in zip(halves[0], halves[1], refs)])) / 4.0
    del halves
    torch.cuda.synchronize()
    print(json.dumps({"phase": "reference", "spp": a.ref_spp, "seconds": time.perf_counter() - t0,
                      "relMSE_noise_estimate": ref_noise}), flush=True)

    # warm-up (allocations, kernel loading) with throwaway guides
    for g in rooms:
        g.nn_reset(1)
    warm = [dict(scene=r, spp=1, max_depth=a.depth, seed=1) for r in range(n)]
    b.render(warm, outputs=False, mode=MODE_MIS, flags=FLAG_UNBIASED_MIS)
    b.render(warm, outputs=False, mode=MODE_NN, flags=FLAG_NN_FREEZE)

    B = max(a.budgets)
    cps = sorted(set([B * 2 ** (-k / 2) for k in range(0, 11)] + list(a.budgets)))
    results, thr = {}, {}
    results["plain"], thr["plain"] = batch_progressive(b, n, (H, W), MODE_MIS, FLAG_UNBIASED_MIS, B, a.chunk,
                                                       a.depth, 10_000, refs, cps)
    defaults = rooms[0].nn_config()
    nn_names = []
    for q, text in enumerate(a.nn_config or ["{}"]):
        opts = json.loads(text)
        freeze = opts.pop("freeze_after", None)
        flags = FLAG_THROUGHPUT_RR if opts.pop("throughput_rr", False) else 0
        for k, g in enumerate(rooms):
            g.nn_reset(2024 + k)
            g.nn_configure(**{**defaults, **opts})
        name = "nn" if q == 0 else f"nn{q}"
        nn_names.append(name)
        results[name], thr[name] = batch_progressive(b, n, (H, W), MODE_NN, flags, B, a.chunk, a.depth, 20_000,
                                                     refs, cps, freeze)
        thr[name].update(training_steps=[g.nn_stats()["steps"] for g in rooms], config=rooms[0].nn_config(),
                         freeze_after=freeze, throughput_rr=flags != 0)
    # the trained guides frozen: inference cost alone
    jobs = [dict(scene=r, spp=a.chunk, max_depth=a.depth, seed=5) for r in range(n)]
    b.render(jobs, outputs=False, mode=MODE_NN, flags=FLAG_NN_FREEZE)
    st = b.stats()
    thr["nn_frozen"] = {"mpaths_s": st["paths"] / (st["render_ms"] * 1e3)}
    b.render(jobs, outputs=False, mode=MODE_MIS, flags=FLAG_UNBIASED_MIS)
    st = b.stats()
    thr["plain_same_spp"] = {"mpaths_s": st["paths"] / (st["render_ms"] * 1e3)}
    for name, v in thr.items():
        print(json.dumps({"throughput": name, **v}), flush=True)

    if not a.no_sdtree:
        # one SD-tree render per room, spp a power of two sized to B / rooms
        t0 = time.perf_counter()
        rooms[0].render(4, max_depth=a.depth, seed=5, mode=MODE_SDTREE)
        t4 = time.perf_counter() - t0
        spp = 4
        while spp * 2 * t4 / 4.0 * n < B and spp < 1 << 14:
            spp *= 2
        t0 = time.perf_counter()
        errs = []
        for r, g in enumerate(rooms):
            x = g.render(spp, max_depth=a.depth, seed=30_000 + r, mode=MODE_SDTREE)
            errs.append(rel_mse(torch.from_numpy(x).cuda(), refs[r]))
        results["sdtree"] = [(time.perf_counter() - t0, spp, float(np.mean(errs)))]

    for name, rows in results.items():
        for el, spp, r in rows:
            print(json.dumps({"method": name, "seconds": el, "spp": spp, "relMSE": r}), flush=True)
    corrected = {k: [(t, s, max(r - ref_noise, 1e-12)) for t, s, r in v] for k, v in results.items()}
    summ = {"reference_noise_relMSE": ref_noise, "budgets": {}}
    for bud in a.budgets:
        pl = [r for t, _, r in results["plain"] if t == bud]
        if not pl:
            continue
        row = {"plain_relMSE": pl[0], "plain_relMSE_noise_corrected": pl[0] - ref_noise}
        for name in nn_names:
            nn = [r for t, _, r in results[name] if t == bud]
            t_nn = time_to_reach(results[name], pl[0])
            t_nc = time_to_reach(corrected[name], max(pl[0] - ref_noise, 1e-12))
            row[name] = {"relMSE": nn[0] if nn else None,
                         "relMSE_noise_corrected": None if not nn else nn[0] - ref_noise,
                         "time_fraction": None if t_nn is None else t_nn / bud,
                         "time_fraction_noise_corrected": None if t_nc is None else t_nc / bud}
        summ["budgets"][str(bud)] = row
    if "sdtree" in results:
        el, spp, r = results["sdtree"][0]
        summ["sdtree"] = {"seconds": el, "spp": spp, "relMSE": r}
    summ["throughput_mpaths_s"] = {k: v["mpaths_s"] for k, v in thr.items()}
    summ["learned"] = {k: {q: v[q] for q in ("training_steps", "config", "freeze_after", "throughput_rr")}
                       for k, v in thr.items() if k in nn_names}
    print(json.dumps({"summary": summ}), flush=True)


if __name__ == "__main__":
    main()
