"""Benchmark of the PT+NEE+MIS hot path (Mpaths/s).

Default workload: the 1M-triangle seeded soup -- 2000 geodesic spheres of
500 triangles in a closed room, Lambert / GGX / dielectric materials, four
unit emitters of radiance 20 -- rendered at 1920x1080, max depth 10.  One
step = `--spp-per-step` samples per pixel over the full frame in one
pt_render call (default 64: a full 256-spp render is four steps).  Each call
ends with the wavefront draining its last paths over about ten iterations
at low occupancy; 64 spp per call amortise that like a full render does (4
spp per call measured 245 Mpaths/s, 16 spp 272, 64 spp 279).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Our arm: `value` is device-resident throughput (scene on the GPU, image left
in device memory), timed per step with the CUDA events the library records
on its own stream; L2 is flushed (a 512 MB write) between steps.  `e2e` goes
through pt_render with the image copied to a pinned host buffer every step.
The reference arm times the reference's own CPU renderer (oracle/_ref, or the
oracle port when the reference could not be compiled) on a bounded sample of
the same scene with all host threads.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "cpp-pt_gb300"))
sys.path.insert(0, ROOT)

METRIC = "Mpaths/s plain PT+NEE+MIS (1M-tri soup, 1920x1080, depth 10)"
UNIT = "Mpaths/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--spp-per-step", type=int, default=64)
    ap.add_argument("--spheres", type=int, default=2000)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--depth", type=int, default=10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-sample", default="320x180x16", help="WxHxSPP of the CPU baseline sample (~10-30 s)")
    ap.add_argument("--ref-step-sample", default="320x180x4", help="WxHxSPP of one reference-arm step")
    return ap.parse_args()


def workload(a):
    from cpppt import scenes
    return scenes.soup(seed=2, n_spheres=a.spheres, freq=5, width=a.width, height=a.height)


def config(a, sc, extra=None):
    c = {"workload": f"soup {a.spheres} spheres x 500 tris = {sc.n_triangles} tris, {a.width}x{a.height}, "
                     f"depth {a.depth}, {a.spp_per_step} spp per step (full render: 256 spp)",
         "triangles": sc.n_triangles, "resolution": [a.width, a.height], "max_depth": a.depth,
         "spp_per_step": a.spp_per_step, "rr_start": 3, "materials": "lambert/ggx/dielectric",
         "l2": "flushed between timed steps (512 MB write)", "parallelism": f"replicas x{a.gpus}"}
    if extra:
        c.update(extra)
    return c


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_baseline(sc, a, repeats=1):
    """Times the reference's own renderer (or the oracle port) on the host
    cores on a bounded sample of the same scene; returns the JSON object."""
    from oracle import oracle as orc
    w, h, spp = (int(x) for x in a.cpu_sample.split("x"))
    sub = sc.with_resolution(w, h)
    kind = "reference" if orc.reference_available() else "port"
    o = orc.Oracle(kind)
    t0 = time.time()
    s = o.scene(sub)
    setup = time.time() - t0
    cores = os.cpu_count() or 1
    secs = []
    for r in range(repeats):
        ax = int(round(spp ** 0.5))
        _, sec = s.render_mis(ax, a.depth, 1000 * (r + 1), threads=cores)
        secs.append(sec)
    paths = w * h * ax * ax
    val = paths / float(np.mean(secs)) / 1e6
    cpu = "unknown"
    try:
        for l in open("/proc/cpuinfo"):
            if l.lower().startswith(("model name", "cpu part")):
                cpu = l.split(":", 1)[1].strip()
                break
    except OSError:
        pass
    return {"value": val, "unit": UNIT, "cores": cores, "kind": kind,
            "sample": f"{w}x{h} x {ax * ax} spp of the same scene, depth {a.depth} "
                      f"({paths} paths, {float(np.mean(secs)):.2f} s render; scene+BVH build {setup:.1f} s); "
                      f"cpu: {cpu}"}


def run_reference(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sc = workload(a)
    a.cpu_sample = a.ref_step_sample
    base = cpu_baseline(sc, a, repeats=1)  # includes the one-time scene build
    w, h, spp = (int(x) for x in a.cpu_sample.split("x"))
    from oracle import oracle as orc
    kind = base["kind"]
    s = orc.Oracle(kind).scene(sc.with_resolution(w, h))
    ax = int(round(spp ** 0.5))
    cores = os.cpu_count() or 1
    for i in range(a.warmup):
        s.render_mis(ax, a.depth, 7000 + i, threads=cores)
    secs = []
    for i in range(a.steps):
        _, sec = s.render_mis(ax, a.depth, 9000 + 1000 * i, threads=cores)
        secs.append(sec)
    paths = w * h * ax * ax
    ms = 1000.0 * float(np.mean(secs))
    val = paths / (ms / 1000.0) / 1e6
    base["value"] = val
    out = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps,
           "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f32", "data": "synthetic (seeded generator)",
           "config": config(a, sc, {"reference_sample": base["sample"]}),
           "cpu_baseline": base,
           "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def aggregate(dist, paths: float, rays: float, ms: float, device: str = "cpu"):
    """Whole-job throughput over the ranks (replicas): every rank's paths
    and rays summed, over the slowest rank's time.  Returns (Mpaths/s,
    Mrays/s, slowest ms).  dist: torch.distributed after init, or None."""
    if dist is not None:
        import torch
        t = torch.tensor([paths, rays], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        m = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(m, op=dist.ReduceOp.MAX)
        paths, rays, ms = float(t[0]), float(t[1]), float(m[0])
    return paths / (ms / 1000.0) / 1e6, rays / (ms / 1000.0) / 1e6, ms


def run_ours(a):
    import torch
    from cpppt.lib import GpuScene, FLAG_TIME_KERNELS, FLAG_COUNT

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    sc = workload(a)
    t0 = time.time()
    gs = GpuScene(sc)
    setup_s = time.time() - t0
    npix = a.width * a.height
    out = torch.empty(npix * 3, dtype=torch.float32, device="cuda")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    spp = a.spp_per_step

    def step(i, seed_base):
        gs.render_device(out.data_ptr(), spp, max_depth=a.depth, seed=seed_base + i)
        return gs.stats()

    for i in range(a.warmup):
        step(i, 100 + 1000 * rank)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms, launches, paths, closest, shadow = [], 0.0, 0.0, 0.0, 0.0
    with ClockSampler(local) as clk:
        t_wall = time.time()
        for i in range(a.steps):
            flush.fill_(float(i))
            torch.cuda.synchronize()
            st = step(i, 5000 + 100000 * rank)
            ms.append(st["render_ms"])
            launches += st["kernel_launches"]
            paths += st["paths"]
            closest += st["closest_rays"]
            shadow += st["shadow_rays"]
        torch.cuda.synchronize()
        wall = time.time() - t_wall
    value, mrays, step_ms = aggregate(dist, paths, closest + shadow, float(np.sum(ms)), "cuda")

    # end to end through pt_render: image copied to a pinned host buffer each step
    host = torch.empty((a.height, a.width, 3), dtype=torch.float32).pin_memory().numpy()
    e2e_ms, h2d, d2h = [], 0.0, 0.0
    for i in range(max(2, a.steps // 2)):
        flush.fill_(float(i))
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        gs.render(spp, max_depth=a.depth, seed=7000 + i, out=host)
        e2e_ms.append((time.perf_counter() - t1) * 1000.0)
        st = gs.stats()
        h2d += st["h2d_bytes"]
        d2h += st["d2h_bytes"]
    n_e2e = len(e2e_ms)
    e2e_val, _, _ = aggregate(dist, paths / a.steps, 0.0, float(np.mean(e2e_ms)), "cuda")

    # roofline of the dominant kernel (closest-hit extension): algorithmic
    # bytes from a counting render, duration from an event-timed render of
    # the same work (same seed -> the same rays)
    gs.render_device(out.data_ptr(), spp, max_depth=a.depth, seed=4242, flags=FLAG_COUNT)
    cnt = gs.stats()
    gs.render_device(out.data_ptr(), spp, max_depth=a.depth, seed=4242, flags=FLAG_TIME_KERNELS)
    tim = gs.stats()
    node_b, tri_b, ray_b, hit_b = 64, 48, 32, 16
    alg_bytes = cnt["extend_nodes"] * node_b + cnt["extend_tris"] * tri_b + cnt["closest_rays"] * (ray_b + hit_b)
    n_launch = tim["iterations"]
    achieved = alg_bytes / (tim["trace_closest_ms"] / 1000.0) / 1e9
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    # DRAM (and L2) bytes per extension ray measured by ncu over every bounce
    # of a render of the same scene (profiles/k_extend_soup1M_720p_bounces.md),
    # scaled by the rays of one launch here
    traffic, l2_traffic = None, None
    tfile = os.path.join(ROOT, "profiles", "k_extend_soup1M_720p_traffic.json")
    if os.path.exists(tfile):
        try:
            tj = json.load(open(tfile))
            per_launch = cnt["closest_rays"] / max(1.0, n_launch)
            traffic = tj["bytes_per_ray"] * per_launch
            l2_traffic = tj["l2_bytes_per_ray"] * per_launch
        except Exception:
            traffic = None

    if rank == 0:
        res = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
               "warmup": a.warmup, "ms_per_step": step_ms / a.steps, "higher_is_better": True,
               "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded generator)",
               "config": config(a, sc, {"scene_setup_s": round(setup_s, 2), "wall_s_timed": round(wall, 3)}),
               "mrays_per_s": mrays,
               "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": h2d / n_e2e,
                       "d2h_bytes_per_step": d2h / n_e2e, "api": "pt_render (host image buffer)"},
               "gpu_launches": int(launches),
               "roofline": {"bound": "hbm", "kernel": "k_extend (closest-hit traversal)",
                            "achieved": achieved, "peak": peak,
                            "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback 6800",
                            "unit": "GB/s", "frac": achieved / peak,
                            "traffic": traffic,
                            "traffic_source": "ncu dram__bytes_read+write per extension ray, all bounces of the "
                                              "1280x720 render of this scene, x rays per launch",
                            "l2_traffic": l2_traffic,
                            "algorithmic_bytes_per_launch": alg_bytes / max(1.0, n_launch),
                            "avg_launch_ms": tim["trace_closest_ms"] / max(1.0, n_launch),
                            "per_ray": {"nodes": cnt["extend_nodes"] / cnt["closest_rays"],
                                        "tris": cnt["extend_tris"] / cnt["closest_rays"],
                                        "bytes": alg_bytes / cnt["closest_rays"]},
                            "extend_share_of_render": tim["trace_closest_ms"] / tim["render_ms"],
                            "shadow_share_of_render": tim["trace_shadow_ms"] / tim["render_ms"]},
               "clocks": clk.summary()}
        if world == 1 and not a.no_cpu_baseline:
            try:
                res["cpu_baseline"] = cpu_baseline(sc, a, repeats=3)
            except Exception as e:
                res["cpu_baseline"] = {"value": None, "unit": UNIT, "cores": os.cpu_count(), "kind": "unavailable",
                                       "sample": f"failed: {e}"}
        print(json.dumps(res))
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
