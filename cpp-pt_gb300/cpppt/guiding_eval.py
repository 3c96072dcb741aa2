"""Equal-time comparison of learned guiding, plain PT and SD-tree guiding on
the occluded-light room (emitter behind a 0.05-wide slit, indirect light
dominates).

    python -m cpppt.guiding_eval [--budgets 10 30 60] [--ref-spp 16384]

All three estimators converge to the same image on this all-Lambert scene
(albedo <= 0.8 keeps the Russian-roulette survival below 1), so each is
scored by relMSE = mean over pixels and channels of (x - ref)^2 / (ref^2 +
1e-2) against one high-spp reference rendered with the plain tracer
(PT_FLAG_UNBIASED_MIS):

* plain  -- PT + NEE + MIS, BSDF sampling only (PT_FLAG_UNBIASED_MIS);
* nn     -- PT + NEE + MIS with the learned vMF-mixture guide, trained
            online from fresh weights inside the time budget (training time
            counts; optionally frozen after a given number of seconds);
* sdtree -- the reference's practical path guiding (PPG: SD-tree, no NEE),
            one render whose spp is sized to the budget;
* mis_default (--mis-default) -- the drop-in default PT_MODE_MIS (the
            reference's estimator: RR-scaled MIS weights, MIS weight at the
            last vertex).  It converges to a slightly different image, so it
            is scored against its own reference (ref_spp / 4 of the same
            estimator); its distance to the unbiased reference is printed as
            its bias.

Plain and nn accumulate chunks of spp on the GPU; relMSE is taken at
checkpoints spaced by sqrt(2) up to the largest budget.  Prints one JSON
line per method and checkpoint, then a summary: relMSE of each method at
each budget, and the time nn needs to reach plain's relMSE at that budget
(linear interpolation of log relMSE over log time between checkpoints),
both as measured and with the reference's own noise (estimated from its two
independent halves) subtracted.
"""
from __future__ import annotations

import argparse
import json
import math
import time

import numpy as np
import torch

from . import scenes
from .lib import FLAG_NN_FREEZE, FLAG_THROUGHPUT_RR, FLAG_UNBIASED_MIS, MODE_MIS, MODE_NN, MODE_SDTREE, GpuScene


def rel_mse(x: torch.Tensor, ref: torch.Tensor) -> float:
    return float(((x - ref) ** 2 / (ref ** 2 + 1e-2)).mean())


def progressive(gs, mode, flags, budget_s, chunk_spp, depth, seed0, ref, checkpoints, freeze_after=None):
    """Renders chunks until the budget is spent, accumulating on the GPU;
    returns [(seconds, spp, relMSE)] at the checkpoints and the final image.
    freeze_after: seconds after which the learned guide stops training."""
    H, W = ref.shape[:2]
    img = torch.zeros((H, W, 3), dtype=torch.float32, device="cuda")
    acc = torch.zeros((H, W, 3), dtype=torch.float64, device="cuda")
    spp_total, k = 0, 0
    snaps = []
    cps = sorted(checkpoints)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    while True:
        f = flags
        if freeze_after is not None and time.perf_counter() - t0 >= freeze_after:
            f |= FLAG_NN_FREEZE
        gs.render_device(img.data_ptr(), chunk_spp, max_depth=depth, seed=seed0 + k, mode=mode, flags=f)
        acc += img.double() * chunk_spp
        k += 1
        spp_total += chunk_spp
        el = time.perf_counter() - t0
        while cps and el >= cps[0]:
            snaps.append((cps.pop(0), spp_total, (acc / spp_total).float().clone()))
        if not cps or el >= budget_s:
            break
    torch.cuda.synchronize()
    out = [(t, spp, rel_mse(x, ref)) for t, spp, x in snaps]
    return out, (acc / spp_total).float(), spp_total


def time_to_reach(rows, target):
    """First time the (log time, log relMSE) curve crosses target."""
    prev = None
    for t, _, r in rows:
        if r <= target:
            if prev is None:
                return t
            t0, r0 = prev
            a = (math.log(target) - math.log(r0)) / (math.log(r) - math.log(r0))
            return math.exp(math.log(t0) + a * (math.log(t) - math.log(t0)))
        prev = (t, r)
    return None


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--budgets", type=float, nargs="+", default=[10, 30, 60])
    ap.add_argument("--ref-spp", type=int, default=16384)
    ap.add_argument("--width", type=int, default=1280)
    ap.add_argument("--height", type=int, default=720)
    ap.add_argument("--boxes", type=int, default=1000)
    ap.add_argument("--depth", type=int, default=12)
    ap.add_argument("--chunk", type=int, default=8)
    ap.add_argument("--nn-config", action="append", default=None,
                    help="JSON settings for GpuScene.nn_configure, optionally with \"freeze_after\": seconds "
                         "after which training stops, \"seed\" (weights and render seeds) and \"throughput_rr\"; "
                         "repeat to compare several learned guides")
    ap.add_argument("--no-sdtree", action="store_true")
    ap.add_argument("--plain-trr", action="store_true",
                    help="also run plain PT with Russian roulette on the throughput (method plain_trr)")
    ap.add_argument("--mis-default", action="store_true",
                    help="also run the drop-in default PT_MODE_MIS, scored against its own reference")
    ap.add_argument("--save", default="")
    a = ap.parse_args()
    sc = scenes.slit_room(seed=4, n_boxes=a.boxes, box_subdiv=4, width=a.width, height=a.height)
    gs = GpuScene(sc)
    H, W = a.height, a.width
    # reference: plain (unbiased) PT at ref_spp, accumulated on the GPU in FP64
    # as two independent halves; relMSE(half A, half B) / 4 estimates the
    # reference's own noise, which adds to every method's measured relMSE
    img = torch.zeros((H, W, 3), dtype=torch.float32, device="cuda")
    halves = [torch.zeros((H, W, 3), dtype=torch.float64, device="cuda") for _ in range(2)]
    t0 = time.perf_counter()
    step = 256
    for q, k in enumerate(range(0, a.ref_spp, step)):
        gs.render_device(img.data_ptr(), step, max_depth=a.depth, seed=777000 + k, mode=MODE_MIS,
                         flags=FLAG_UNBIASED_MIS)
        halves[q & 1] += img.double()
    n_steps = a.ref_spp // step
    ref = ((halves[0] + halves[1]) / n_steps).float()
    ha = (halves[0] / ((n_steps + 1) // 2)).float()
    hb = (halves[1] / max(1, n_steps // 2)).float()
    ref_noise = float(((ha - hb) ** 2 / (ref ** 2 + 1e-2)).mean()) / 4.0
    torch.cuda.synchronize()
    ref_s = time.perf_counter() - t0
    print(json.dumps({"reference": {"spp": a.ref_spp, "seconds": ref_s, "mean": float(ref.mean()),
                                    "relMSE_noise_estimate": ref_noise, "triangles": sc.n_triangles,
                                    "resolution": [W, H], "depth": a.depth}}), flush=True)
    ref_def = None
    if a.mis_default:
        # the default estimator's own reference, also as two halves
        hd = [torch.zeros((H, W, 3), dtype=torch.float64, device="cuda") for _ in range(2)]
        nd = max(2, (a.ref_spp // 4) // step)
        t0 = time.perf_counter()
        for q in range(nd):
            gs.render_device(img.data_ptr(), step, max_depth=a.depth, seed=888000 + q * step, mode=MODE_MIS, flags=0)
            hd[q & 1] += img.double()
        ref_def = ((hd[0] + hd[1]) / nd).float()
        da = (hd[0] / ((nd + 1) // 2)).float()
        db = (hd[1] / max(1, nd // 2)).float()
        def_noise = float(((da - db) ** 2 / (ref_def ** 2 + 1e-2)).mean()) / 4.0
        print(json.dumps({"reference_mis_default": {"spp": nd * step, "seconds": time.perf_counter() - t0,
                                                    "relMSE_noise_estimate": def_noise,
                                                    "bias_relMSE_vs_unbiased": rel_mse(ref_def, ref),
                                                    "mean": float(ref_def.mean())}}), flush=True)
    # warm-up (graph capture, allocations, kernel loading)
    gs.render_device(img.data_ptr(), 1, max_depth=a.depth, seed=1, mode=MODE_MIS, flags=FLAG_UNBIASED_MIS)
    gs.render_device(img.data_ptr(), 1, max_depth=a.depth, seed=1, mode=MODE_NN, flags=FLAG_NN_FREEZE)
    B = max(a.budgets)
    cps = sorted(set([B * 2 ** (-k / 2) for k in range(0, 13)] + list(a.budgets)))
    results = {}
    res_plain, img_plain, _ = progressive(gs, MODE_MIS, FLAG_UNBIASED_MIS, B, a.chunk, a.depth, 10_000, ref, cps)
    results["plain"] = res_plain
    if ref_def is not None:
        results["mis_default"], _, _ = progressive(gs, MODE_MIS, 0, B, a.chunk, a.depth, 15_000, ref_def, cps)
    if a.plain_trr:
        results["plain_trr"], _, _ = progressive(gs, MODE_MIS, FLAG_UNBIASED_MIS | FLAG_THROUGHPUT_RR, B, a.chunk,
                                                 a.depth, 10_000, ref, cps)
    nn_runs = {}
    defaults = gs.nn_config()
    for q, text in enumerate(a.nn_config or ["{}"]):
        opts = json.loads(text)
        freeze = opts.pop("freeze_after", None)
        seed = int(opts.pop("seed", 0))
        flags = FLAG_THROUGHPUT_RR if opts.pop("throughput_rr", False) else 0
        gs.nn_reset(2024 + seed)
        cfg = gs.nn_configure(**{**defaults, **opts})
        rows, img_nn, _ = progressive(gs, MODE_NN, flags, B, a.chunk, a.depth, 20_000 + 100_000 * seed, ref, cps,
                                      freeze)
        name = "nn" if q == 0 else f"nn{q}"
        results[name] = rows
        nn_runs[name] = {"config": cfg, "freeze_after": freeze, "seed": seed, "throughput_rr": flags != 0,
                         "training": gs.nn_stats()}
    if not a.no_sdtree:
        # SD-tree (PPG): one render per budget; passes of 1, 2, 4, ... spp cost ~2x the last pass
        t0 = time.perf_counter()
        gs.render(4, max_depth=a.depth, seed=5, mode=MODE_SDTREE)
        t4 = time.perf_counter() - t0
        res_sd = []
        for bud in a.budgets:
            spp = 4
            while spp * 2 * t4 / 4.0 < bud and spp < 1 << 16:
                spp *= 2
            t0 = time.perf_counter()
            x = gs.render(spp, max_depth=a.depth, seed=30_000 + spp, mode=MODE_SDTREE)
            el = time.perf_counter() - t0
            res_sd.append((el, spp, rel_mse(torch.from_numpy(x).cuda(), ref)))
        results["sdtree"] = res_sd
    for name, rows in results.items():
        for el, spp, r in rows:
            print(json.dumps({"method": name, "seconds": el, "spp": spp, "relMSE": r}), flush=True)
    summ = {"learned": nn_runs, "reference_noise_relMSE": ref_noise, "budgets": {}}
    corrected = {k: [(t, spp, max(r - ref_noise, 1e-12)) for t, spp, r in v] for k, v in results.items()}
    for bud in a.budgets:
        p = [r for t, _, r in res_plain if t == bud]
        if not p:
            continue
        pc = p[0] - ref_noise
        row = {"plain_relMSE": p[0], "plain_relMSE_noise_corrected": pc}
        for name in nn_runs:
            n = [r for t, _, r in results[name] if t == bud]
            t_nn = time_to_reach(results[name], p[0])
            t_nc = time_to_reach(corrected[name], max(pc, 1e-12))
            row[name] = {"relMSE": n[0] if n else None, "seconds_to_plain_relMSE": t_nn,
                         "time_fraction": None if t_nn is None else t_nn / bud,
                         "relMSE_noise_corrected": None if not n else n[0] - ref_noise,
                         "time_fraction_noise_corrected": None if t_nc is None else t_nc / bud}
        if "mis_default" in results:
            d = [r for t, _, r in results["mis_default"] if t == bud]
            if d:
                row["mis_default_relMSE_vs_own_reference"] = d[0]
                for name in nn_runs:
                    t_d = time_to_reach(results[name], d[0])
                    row[name]["time_fraction_vs_mis_default"] = None if t_d is None else t_d / bud
        if "sdtree" in results:
            sd = [r for (el, spp, r), b2 in zip(results["sdtree"], a.budgets) if b2 == bud]
            row["sdtree_relMSE"] = sd[0] if sd else None
        summ["budgets"][str(bud)] = row
    print(json.dumps({"summary": summ}), flush=True)
    if a.save:
        np.savez_compressed(a.save, ref=ref.cpu().numpy(), plain=img_plain.cpu().numpy(),
                            nn=img_nn.cpu().numpy())


if __name__ == "__main__":
    main()
