"""A small textured room in the reference's file formats, written from
scratch with its textures (PNG): a floor with a tiled sRGB checker albedo
(uv in [0, 1.75]^2, so the REPEAT border is exercised; the reference reads
outside the image where a pixel coordinate lands on a negative multiple of
the image size, rgb_image.h:236-244, which these uvs never reach), a back
wall whose metal
map switches between the diffuse and the GGX BxDF with a roughness map, a
side wall with a normal map, a plain wall, and a ceiling emitter with an
sRGB emission texture.  Used by the golden fixture (reference render) and
the GPU test (the library's loader on the same files)."""
from __future__ import annotations

import os

import numpy as np

from tests.imagefiles import write_png

W, H = 64, 48


def _f(x) -> str:
    return format(float(np.float32(x)), ".9g")


def _quad(path, corners, normal, tangent, uv_scale=1.0):
    """corners: a, b, c, d counter-clockwise seen from the normal side."""
    uvs = [(0.0, 0.0), (uv_scale, 0.0), (uv_scale, uv_scale), (0.0, uv_scale)]
    with open(path, "w") as f:
        f.write("4 2 TRIANGLE_MESH\n")
        for p, uv in zip(corners, uvs):
            f.write(" ".join(_f(x) for x in (*p, *uv, *normal, *tangent)) + "\n")
        f.write("0 1 2\n0 2 3\n")


def write(directory: str, spp_axis: int = 1) -> str:
    os.makedirs(directory, exist_ok=True)
    rng = np.random.default_rng(12)
    # textures
    yy, xx = np.mgrid[0:16, 0:16]
    checker = (((xx // 4) + (yy // 4)) % 2)[..., None] * np.array([200, 60, 40]) + \
        (1 - ((xx // 4) + (yy // 4)) % 2)[..., None] * np.array([40, 170, 220])
    write_png(os.path.join(directory, "checker.png"), checker, 2, 8)
    metal = np.zeros((8, 16, 1), np.int64)
    metal[:, 8:] = 255
    write_png(os.path.join(directory, "metal.png"), metal, 0, 8)
    rough = np.tile(np.linspace(0, 65535, 16).astype(np.int64)[None, :, None], (8, 1, 1))
    write_png(os.path.join(directory, "rough.png"), rough, 0, 16)
    nx = 128 + (40 * np.sin(np.arange(16) / 2.0)).astype(np.int64)
    nmap = np.stack([np.tile(nx[None, :], (16, 1)), np.full((16, 16), 128), np.full((16, 16), 230)], -1)
    write_png(os.path.join(directory, "normal.png"), nmap, 2, 8, interlace=True)
    emit = rng.integers(120, 256, (4, 4, 3))
    write_png(os.path.join(directory, "emit.png"), emit, 2, 8)
    # materials (DISNEY albedo spec roughness metal transparent ior normal alpha; EMISSION colour intensity)
    mats = {
        "floor.ptmat": "DISNEY image(checker.png) float(0.5) float(0.3) float(0) float(0) float(1.5) rgb(0.5,0.5,1) "
                       "float(1) -\n",
        "back.ptmat": "DISNEY rgb(0.7,0.7,0.7) float(0.5) image(rough.png) image(metal.png) float(0) float(1.5) "
                      "rgb(0.5,0.5,1) float(1) -\n",
        "side.ptmat": "DISNEY rgb(0.6,0.5,0.4) float(0.5) float(0.3) float(0) float(0) float(1.5) image(normal.png) "
                      "float(1) -\n",
        "plain.ptmat": "DISNEY rgb(0.5,0.6,0.5) float(0.5) float(0.3) float(0) float(0) float(1.5) rgb(0.5,0.5,1) "
                       "float(1) -\n",
        "light.ptmat": "EMISSION image(emit.png) float(6)\n",
    }
    for name, text in mats.items():
        with open(os.path.join(directory, name), "w") as f:
            f.write(text)
    # geometry: room [0,4] x [0,3] x [0,4], camera looking at the back wall (z = 0)
    quads = [
        ("floor.ptobj", [(0, 0, 4), (4, 0, 4), (4, 0, 0), (0, 0, 0)], (0, 1, 0), (1, 0, 0), 1.75, "floor.ptmat"),
        ("back.ptobj", [(0, 0, 0), (4, 0, 0), (4, 3, 0), (0, 3, 0)], (0, 0, 1), (1, 0, 0), 1.0, "back.ptmat"),
        ("left.ptobj", [(0, 0, 4), (0, 0, 0), (0, 3, 0), (0, 3, 4)], (1, 0, 0), (0, 0, -1), 1.0, "side.ptmat"),
        ("right.ptobj", [(4, 0, 0), (4, 0, 4), (4, 3, 4), (4, 3, 0)], (-1, 0, 0), (0, 0, 1), 1.0, "plain.ptmat"),
        ("ceil.ptobj", [(0, 3, 0), (4, 3, 0), (4, 3, 4), (0, 3, 4)], (0, -1, 0), (1, 0, 0), 1.0, "plain.ptmat"),
        ("light.ptobj", [(1.5, 2.99, 1.5), (2.5, 2.99, 1.5), (2.5, 2.99, 2.5), (1.5, 2.99, 2.5)], (0, -1, 0),
         (1, 0, 0), 1.0, "light.ptmat"),
    ]
    lines = ["camera 2 1.5 6.5 2 1.4 0 0 1 0 0.5"]
    for obj, corners, n, t, s, mat in quads:
        _quad(os.path.join(directory, obj), corners, n, t, s)
        lines.append(f"obj {obj} {mat}")
    scene = os.path.join(directory, "scene.ptscene")
    with open(scene, "w") as f:
        f.write("\n".join(lines) + "\n")
    settings = os.path.join(directory, "settings.txt")
    with open(settings, "w") as f:
        f.write(f"renderer pathtracer_mis\nspp {spp_axis}\nresolution {W} {H}\nscene {scene}\n"
                f"output {os.path.join(directory, 'out')}\n")
    return settings
