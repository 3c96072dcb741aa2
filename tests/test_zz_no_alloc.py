"""pt_render_device_noalloc: the render entry point for callers that cannot
allocate device memory while they render (memory reserved up front by
another allocator or an engine's budget, frame loops that must stay off the
driver's allocation path).  Its scratch is a fixed array inside
the library, so it must give the same image as pt_render_device and leave
the device's free memory unchanged.

This file is collected last on purpose; it also runs alone in a fresh
process (python -m pytest tests/test_zz_no_alloc.py -m gpu)."""
import ctypes as C

import numpy as np
import pytest

from cpppt import scenes

pytestmark = pytest.mark.gpu


def _render(lib_mod, L, gs, fn, seed, out, spp=64, depth=8):
    import torch
    out.zero_()
    d = lib_mod.PtRenderDesc()
    d.spp, d.max_depth, d.rr_start, d.seed, d.mode, d.flags = spp, depth, 3, seed, 0, 0
    if fn == "noalloc":
        st = L.pt_render_device_noalloc(gs.h, C.byref(d), out.data_ptr(), None)
    else:
        st = L.pt_render_device(gs.h, C.byref(d), out.data_ptr())
    assert st == 0, L.pt_last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(gs.height, gs.width, 3)


def test_noalloc_render_matches_allocating_render_twice(gpu_lib):
    import torch
    from cpppt import lib as lib_mod
    from cpppt.lib import GpuScene
    torch.cuda.set_device(0)
    L = lib_mod.load()
    gs = GpuScene(scenes.cornell(64, 48))
    out = torch.zeros(gs.height * gs.width * 3, dtype=torch.float32, device="cuda")
    ref_a = _render(lib_mod, L, gs, "alloc", 11, out)
    ref_b = _render(lib_mod, L, gs, "alloc", 12, out)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    got_a = _render(lib_mod, L, gs, "noalloc", 11, out)  # first call on this device: address lookup
    got_b = _render(lib_mod, L, gs, "noalloc", 12, out)  # second call reuses the same scratch
    free1, _ = torch.cuda.mem_get_info()
    st = gs.stats()  # the allocation-free call fills the scene's counters like pt_render
    assert st["paths"] == gs.width * gs.height * 64 and st["closest_rays"] >= st["paths"]
    # Same paths, same counter-based random numbers, order-independent
    # fixed-point film: the images are equal to the last bit (tolerance 0).
    np.testing.assert_array_equal(got_a, ref_a)
    np.testing.assert_array_equal(got_b, ref_b)
    assert not np.array_equal(got_a, got_b)
    assert free1 == free0, f"device free memory changed by {free0 - free1} bytes"


def test_noalloc_rejects_images_beyond_its_maximum(gpu_lib):
    import torch
    from cpppt import lib as lib_mod
    from cpppt.lib import GpuScene
    L = lib_mod.load()
    gs = GpuScene(scenes.cornell(1024, 512))
    out = torch.zeros(1024 * 512 * 3, dtype=torch.float32, device="cuda")
    d = lib_mod.PtRenderDesc()
    d.spp, d.max_depth, d.rr_start, d.seed, d.mode, d.flags = 1, 4, 3, 0, 0, 0
    st = L.pt_render_device_noalloc(gs.h, C.byref(d), out.data_ptr(), None)
    assert st == 4
    assert b"exceeds the allocation-free render's maximum" in L.pt_last_error()
