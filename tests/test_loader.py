"""The reference's file formats: settings, .ptscene, .ptobj, .ptmat.

Files written by cpppt.ptfiles are read (a) by the reference's own Loader
(through the oracle harness, CPU) and (b) by this library's loader
(pt_scene_load, GPU); both must describe the same scene: the same hits,
bit for bit, on the fixture rays."""
import os

import numpy as np
import pytest

from tests.golden.make_golden import SMALL_SCENES


def _write(tmp_path, name):
    from cpppt import ptfiles
    return ptfiles.write(SMALL_SCENES[name](), str(tmp_path / name), spp_axis=2)


@pytest.mark.parametrize("name", ["cornell", "slitroom"])
def test_reference_loader_reads_written_files(tmp_path, golden, name):
    from oracle import oracle as orc
    if not orc.reference_available():
        pytest.skip("reference harness not built in this environment")
    g = golden(f"{name}_ref.npz")
    s = orc.Oracle("reference").load_files(_write(tmp_path, name))
    assert s.spp_axis == 2
    idx, t = s.trace_closest(g["rays"])
    assert np.array_equal(idx, g["hit_index"])
    assert np.array_equal(t.view(np.uint32), g["hit_t"].view(np.uint32))


def test_settings_errors_are_reported(tmp_path):
    from cpppt import lib
    bad = tmp_path / "bad.txt"
    bad.write_text("renderer nonsense\n")
    L = lib.load()
    import ctypes as C
    h = C.c_void_p()
    rs = lib.PtRenderDesc()
    st = L.pt_scene_load(str(bad).encode(), C.byref(h), C.byref(rs), None, 0)
    assert st == 5 and b"Unknown renderer type" in L.pt_last_error()
    st = L.pt_scene_load(str(tmp_path / "missing.txt").encode(), C.byref(h), C.byref(rs), None, 0)
    assert st == 5


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["cornell", "slitroom"])
def test_library_loader_matches_reference(gpu_lib, tmp_path, golden, name):
    from cpppt.lib import GpuScene
    g = golden(f"{name}_ref.npz")
    gs = GpuScene(settings_file=_write(tmp_path, name))
    assert gs.render_settings.spp == 4 and gs.render_settings.max_depth == 32
    sc = SMALL_SCENES[name]()
    assert (gs.width, gs.height, gs.n_triangles) == (sc.width, sc.height, sc.n_triangles)
    idx, t, _, _ = gs.trace_closest(g["rays"])
    assert np.array_equal(idx, g["hit_index"])
    assert np.array_equal(t.view(np.uint32), g["hit_t"].view(np.uint32))


@pytest.mark.gpu
def test_cli_renders_files(gpu_lib, tmp_path):
    import subprocess
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cli = os.path.join(root, "cpp-pt_gb300", "lib", "cpppt_render")
    settings = _write(tmp_path, "cornell")
    r = subprocess.run([cli, settings, "8"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("s")
    png = tmp_path / "cornell" / "out.png"
    hdr = tmp_path / "cornell" / "out.hdr"
    assert png.exists() and hdr.exists()
    assert png.read_bytes()[:8] == b"\x89PNG\r\n\x1a\n"
    assert hdr.read_bytes().startswith(b"#?RADIANCE")


def _read_cache(path):
    raw = open(path, "rb").read()
    assert raw[:8] == b"GBPTOBJ2"
    nv, nf = np.frombuffer(raw[24:32], np.int32)
    f32 = np.frombuffer(raw[32:32 + 36 * nv], np.float32).reshape(3, nv, 3)
    uv = np.frombuffer(raw[32 + 36 * nv:32 + 44 * nv], np.float32).reshape(nv, 2)
    faces = np.frombuffer(raw[32 + 44 * nv:], np.int32).reshape(nf, 3)
    return f32[0], f32[1], f32[2], uv, faces


def test_mesh_cache_holds_the_parsed_mesh(tmp_path):
    """pt_scene_load writes <mesh>.ptobj.gbbin with the parsed arrays (the
    scene is parsed before any device is touched, so this runs anywhere),
    reads it back while current, and rewrites it when the mesh changes."""
    import ctypes as C
    import glob
    from cpppt import lib
    L = lib.load()
    L.pt_set_mesh_cache(1)
    settings = _write(tmp_path, "cornell")
    objs = sorted(glob.glob(str(tmp_path / "cornell*" / "*.ptobj")) + glob.glob(str(tmp_path / "*.ptobj")))
    assert objs

    def load():
        h = C.c_void_p()
        rs = lib.PtRenderDesc()
        st = L.pt_scene_load(settings.encode(), C.byref(h), C.byref(rs), None, 0)
        assert st in (0, 2, 6), L.pt_last_error()  # 2 or 6: no usable sm_103 device; the files were read
        if st == 0:
            L.pt_scene_destroy(h)

    load()
    for o in objs:
        assert os.path.exists(o + ".gbbin")
        head = open(o).readline().split()
        nv, nf = int(head[0]), int(head[1])
        rows = [list(map(float, l.split())) for l in open(o).read().splitlines()[1:1 + nv]]
        faces = [list(map(int, l.split())) for l in open(o).read().splitlines()[1 + nv:1 + nv + nf]]
        v, n, t, uv, f = _read_cache(o + ".gbbin")
        assert np.array_equal(v, np.float32(np.array(rows)[:, 0:3]))
        assert np.array_equal(uv, np.float32(np.array(rows)[:, 3:5]))
        assert np.array_equal(n, np.float32(np.array(rows)[:, 5:8]))
        assert np.array_equal(t, np.float32(np.array(rows)[:, 8:11]))
        assert np.array_equal(f, np.array(faces, np.int32))
    # a changed mesh invalidates its cache
    o = objs[0]
    text = open(o).read().splitlines()
    vals = text[1].split()
    vals[0] = repr(float(vals[0]) + 0.25)
    text[1] = " ".join(vals)
    open(o, "w").write("\n".join(text) + "\n")
    os.utime(o, ns=(os.stat(o).st_atime_ns, os.stat(o).st_mtime_ns + 10 ** 9))
    load()
    v, _, _, _, _ = _read_cache(o + ".gbbin")
    assert v[0, 0] == np.float32(float(vals[0]))
