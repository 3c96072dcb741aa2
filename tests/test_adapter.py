"""The drop-in boundary bound to the reference for real: the
PathtracerGB300 : cpppt::Renderer adapter (include/pathtracer_gb300.h),
compiled against the reference's own headers with the flags of
oracle/build_ref.sh and driven through Renderer::render(Scene&, filename)
by the reference's main() flow (tests/adapter_main.cpp).  The files it
writes must be byte-identical to pt_render + pt_image_save on the same
settings file (the render is deterministic for a seed)."""
import os
import subprocess

import numpy as np
import pytest

from tests.golden.make_golden import SMALL_SCENES

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_SRC = os.path.join(ROOT, "oracle", "_ref", "src")
LIBDIR = os.path.join(ROOT, "cpp-pt_gb300", "lib")


def _build_adapter(out_dir: str) -> str:
    if not os.path.isdir(REF_SRC):
        pytest.fail("the reference copy oracle/_ref/src is missing (oracle/build_ref.sh)")
    exe = os.path.join(out_dir, "adapter_main")
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O1", "-fopenmp", "-ffp-contract=off", "-fpermissive", "-w",
           "-include", "memory", "-include", "cmath", "-include", "math.h", "-include", "fstream",
           "-I" + REF_SRC, "-I" + os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "adapter_main.cpp"),
           "-o", exe, "-L" + LIBDIR, "-lcpppt_gb300", "-Wl,-rpath," + LIBDIR]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-4000:]
    return exe


@pytest.mark.gpu
def test_adapter_renders_through_the_reference_renderer_interface(gpu_lib, tmp_path):
    from cpppt import ptfiles
    from cpppt.lib import GpuScene, save_image
    exe = _build_adapter(str(tmp_path))
    settings = ptfiles.write(SMALL_SCENES["cornell"](), str(tmp_path / "cornell"), spp_axis=2)
    r = subprocess.run([exe, settings], capture_output=True, text=True, timeout=300, cwd=str(tmp_path))
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("s")
    out = [l.split(None, 1)[1].strip() for l in open(settings) if l.startswith("output")][0]
    out = out if os.path.isabs(out) else os.path.join(os.path.dirname(settings), out)
    # the same files through the C ABI directly
    gs = GpuScene(settings_file=settings)
    d = gs.render_settings
    img = gs.render(d.spp, max_depth=d.max_depth, rr_start=d.rr_start, seed=d.seed)
    assert img.mean() > 0
    ref_prefix = str(tmp_path / "direct")
    save_image(ref_prefix, img)
    for ext in (".hdr", ".png"):
        got = open(out + ext, "rb").read()
        want = open(ref_prefix + ext, "rb").read()
        assert got == want, ext


@pytest.mark.gpu
def test_adapter_reports_errors_as_runtime_error(gpu_lib, tmp_path):
    """With no CUDA device visible the reference's own loader still reads the
    files, the library refuses (PT_ERR_NO_DEVICE), and the adapter turns that
    into std::runtime_error with pt_last_error's message, which main()
    catches and prints (main.cpp:143-145)."""
    from cpppt import ptfiles
    exe = _build_adapter(str(tmp_path))
    settings = ptfiles.write(SMALL_SCENES["cornell"](), str(tmp_path / "cornell"), spp_axis=1)
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run([exe, settings], capture_output=True, text=True, timeout=300, cwd=str(tmp_path), env=env)
    assert r.returncode == 1, r.stdout + r.stderr
    assert "device" in r.stdout.strip().splitlines()[-1].lower(), r.stdout
