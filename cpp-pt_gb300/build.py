"""Builds the CUDA extension library in-tree: cpp-pt_gb300/lib/libcpppt_gb300.so.

    python cpp-pt_gb300/build.py            # incremental
    python cpp-pt_gb300/build.py --force

Translation units, compiled in parallel, CUDA for sm_103a only:
  csrc/render.cu  -- traversal and PT+NEE+MIS wavefront kernels (nvcc -gencode arch=compute_103a,code=sm_103a)
  csrc/guide.cu   -- SD-tree guided (PPG) wavefront kernels
  csrc/gpu_bvh.cu -- device build of the reference-topology BVH
  csrc/gpu_sah.cu -- device build of the 4-wide SAH traversal tree
  csrc/nn.cu      -- learned guide: MLP on the tensor cores, training, guided wavefront
  csrc/host.cpp   -- C ABI, render drivers, loader, image output
  csrc/bvh.cpp    -- BVH builders
  csrc/sdtree.cpp -- SD-tree structure and update
  csrc/image_io.cpp -- PNG / Radiance RGBE texture decoding
  csrc/loader.cpp -- the reference's scene file formats, mesh cache
Host files use -ffp-contract=off: the reference-topology BVH and the SD-tree
update must round like the reference.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "lib", "obj")
LIB = os.path.join(HERE, "lib", "libcpppt_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _deps(src: str) -> list[str]:
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))] + [
        os.path.join(HERE, "..", "include", "cpppt_gb300.h"), src]


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def _commands(extra_cuda: list[str] | None = None):
    nvcc = _nvcc()
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]
    jobs = []
    for name in ("render.cu", "guide.cu", "nn.cu", "batch.cu", "gpu_bvh.cu", "gpu_sah.cu", "host.cpp", "batch.cpp", "bvh.cpp", "sdtree.cpp",
                 "image_io.cpp", "loader.cpp"):
        src = os.path.join(CSRC, name)
        out = os.path.join(OBJ, name + ".o")
        cmd = [nvcc, "-c", src, "-o", out] + common
        if name.endswith(".cu"):
            cmd += ARCH + ["-lineinfo"] + (extra_cuda or [])
        else:  # compile-time knobs (-D...) reach the host files too
            cmd += ["-x", "c++"] + [f for f in (extra_cuda or []) if f.startswith("-D")]
        jobs.append((src, out, cmd))
    return nvcc, jobs


def build(force: bool = False, verbose: bool = False, extra_cuda: list[str] | None = None) -> str:
    os.makedirs(OBJ, exist_ok=True)
    nvcc, jobs = _commands(extra_cuda)
    todo = [(s, o, c) for s, o, c in jobs if force or _stale(o, _deps(s))]

    def run(job):
        s, o, c = job
        r = subprocess.run(c, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {' '.join(c)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, file=sys.stderr)
        return o

    with cf.ThreadPoolExecutor(max_workers=6) as ex:
        list(ex.map(run, todo))
    objs = [o for _, o, _ in jobs]
    if force or todo or _stale(LIB, objs):
        cmd = [nvcc, "-shared", "-o", LIB] + objs + ARCH
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    # command-line renderer with the reference's main() interface
    cli_src = os.path.join(CSRC, "cpppt_render.cpp")
    cli = os.path.join(HERE, "lib", "cpppt_render")
    if force or _stale(cli, [cli_src, LIB, os.path.join(CSRC, "gpu_pathtracer.h")]):
        cxx = os.environ.get("CXX", "g++")
        cmd = [cxx, "-O2", "-std=c++17", cli_src, "-o", cli, "-L" + os.path.dirname(LIB), "-lcpppt_gb300",
               "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CLI build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--ptxas-v", action="store_true", help="print register / spill usage")
    a = ap.parse_args()
    print(build(a.force, verbose=True, extra_cuda=["-Xptxas", "-v"] if a.ptxas_v else None))
