"""Texture decoding on the host: the library's own PNG / RGBE decoders
give the pixels the reference's Image<Vec3> / Image<float> load through
stb_image (rgb_image.h:160-205), bit for bit, on files covering the
formats' features."""
import itertools

import numpy as np
import pytest

from tests.imagefiles import write_png, write_rgbe


def _reference():
    from oracle import oracle as orc
    if not orc.reference_available():
        pytest.skip("reference harness not built here")
    return orc.Oracle("reference")


CASES = [  # (name, colour type, depth, channels, interlace, zlib level)
    ("grey8", 0, 8, 1, False, 9), ("grey1", 0, 1, 1, False, 6), ("grey2", 0, 2, 1, True, 9),
    ("grey4", 0, 4, 1, False, 0), ("grey16", 0, 16, 1, False, 9), ("greyalpha8", 4, 8, 2, False, 9),
    ("greyalpha16", 4, 16, 2, True, 1), ("rgb8", 2, 8, 3, False, 9), ("rgb8_stored", 2, 8, 3, False, 0),
    ("rgb16", 2, 16, 3, False, 9), ("rgb8_adam7", 2, 8, 3, True, 9), ("rgba8", 6, 8, 4, False, 9),
    ("rgba16_adam7", 6, 16, 4, True, 9), ("pal8", 3, 8, 1, False, 9), ("pal4_trns", 3, 4, 1, True, 9),
    ("pal1", 3, 1, 1, False, 9), ("pal2_trns", 3, 2, 1, False, 0),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_png_matches_reference_loader(tmp_path, case):
    from cpppt import lib
    ref = _reference()
    name, ct, depth, ch, interlace, level = case
    rng = np.random.default_rng(abs(hash(name)) % 2 ** 31)
    h, w = 13, 29  # odd sizes: partial Adam7 passes and partial bytes at low depths
    hi = (1 << depth) - 1
    palette = trns = None
    if ct == 3:
        n_pal = min(1 << depth, 200)
        palette = rng.integers(0, 256, (n_pal, 3))
        samples = rng.integers(0, n_pal, (h, w, 1))
        if name.endswith("trns"):
            trns = bytes(rng.integers(0, 256, max(1, n_pal - 1)).astype(np.uint8).tolist())
    else:
        samples = rng.integers(0, hi + 1, (h, w, ch))
        samples[:4] = samples[0:1]  # repeated rows: long matches in the deflate stream
    path = str(tmp_path / f"{name}.png")
    write_png(path, samples, ct, depth, interlace=interlace, palette=palette, trns=trns, level=level,
              first_filter=len(name) % 5)
    for rgb, srgb in itertools.product((True, False), (True, False)):
        got = lib.image_load(path, rgb=rgb, srgb=srgb)
        want = ref.image_load(path, rgb=rgb, srgb=srgb)
        assert got.shape == want.shape
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (name, rgb, srgb)


@pytest.mark.parametrize("rle", [True, False])
def test_rgbe_matches_reference_loader(tmp_path, rle):
    from cpppt import lib
    ref = _reference()
    rng = np.random.default_rng(5)
    h, w = 9, 40
    rgbe = rng.integers(0, 256, (h, w, 4)).astype(np.uint8)
    rgbe[:, 10:30, 3] = 130  # runs
    rgbe[2, :, 3] = 0  # zero exponent: black
    path = str(tmp_path / ("rle.hdr" if rle else "flat.hdr"))
    write_rgbe(path, rgbe, rle=rle)
    for rgb, srgb in itertools.product((True, False), (True, False)):
        got = lib.image_load(path, rgb=rgb, srgb=srgb)
        want = ref.image_load(path, rgb=rgb, srgb=srgb)
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), (rle, rgb, srgb)


def test_unreadable_images_are_errors(tmp_path):
    from cpppt import lib
    from cpppt.lib import PtError
    p = tmp_path / "x.jpg"
    p.write_bytes(b"\xff\xd8\xff\xe0 not decoded here")
    with pytest.raises(PtError):
        lib.image_load(str(p))
    q = tmp_path / "t.png"
    write_png(str(q), np.zeros((4, 4, 3), np.int64), 2, 8)
    q.write_bytes(q.read_bytes()[:40])  # truncated
    with pytest.raises(PtError):
        lib.image_load(str(q))
    with pytest.raises(PtError):
        lib.image_load(str(tmp_path / "missing.png"))


def test_loader_reads_image_textures(tmp_path):
    """pt_scene_load decodes a scene's image(...) textures while parsing
    (before any device work, so this runs anywhere); a missing or
    undecodable texture file is a PT_ERR_IO."""
    import ctypes as C
    from cpppt import lib
    from tests import texscene
    L = lib.load()

    def load(settings):
        h = C.c_void_p()
        rs = lib.PtRenderDesc()
        st = L.pt_scene_load(settings.encode(), C.byref(h), C.byref(rs), None, 0)
        if st == 0:
            L.pt_scene_destroy(h)
        return st

    settings = texscene.write(str(tmp_path / "ok"))
    assert load(settings) in (0, 2, 6), L.pt_last_error()  # 2 or 6: no usable sm_103 device here
    bad = texscene.write(str(tmp_path / "missing"))
    (tmp_path / "missing" / "checker.png").unlink()
    assert load(bad) == 5 and b"checker.png" in L.pt_last_error()
    broken = texscene.write(str(tmp_path / "broken"))
    (tmp_path / "broken" / "rough.png").write_bytes(b"\x89PNG\r\n\x1a\n broken")
    assert load(broken) == 5
