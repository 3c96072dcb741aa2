"""A small textured room in the reference's file formats, written from
scratch with its textures (PNG): a floor with a tiled sRGB checker albedo
(uv in [0, 1.75]^2, so the REPEAT border is exercised; the reference reads
outside the image where a pixel coordinate lands on a negative multiple of
the image size, rgb_image.h:236-244, which these uvs never reach), a back
wall whose metal map switches between the diffuse and the GGX BxDF with a
roughness map, a side wall with a normal map, a plain wall, and a ceiling
emitter with an sRGB emission texture.  Used by the golden fixture
(reference render), the GPU test (the library's loader on the same files)
and the oracle port's texture pin (`port_inputs`: the same room as arrays)."""
from __future__ import annotations

import os

import numpy as np

from tests.imagefiles import write_png

W, H = 64, 48
CAMERA = (2, 1.5, 6.5, 2, 1.4, 0, 0, 1, 0, 0.5)

# textures: file -> (bw or rgb use, written by _textures)
# materials: DISNEY slots (albedo, roughness, metal, normal) as ("rgb", ...),
# ("float", x) or ("image", file); EMISSION colour and intensity
MATERIALS = {
    "floor.ptmat": dict(albedo=("image", "checker.png"), rough=("float", 0.3), metal=("float", 0.0),
                        normal=("rgb", 0.5, 0.5, 1.0)),
    "back.ptmat": dict(albedo=("rgb", 0.7, 0.7, 0.7), rough=("image", "rough.png"), metal=("image", "metal.png"),
                       normal=("rgb", 0.5, 0.5, 1.0)),
    "side.ptmat": dict(albedo=("rgb", 0.6, 0.5, 0.4), rough=("float", 0.3), metal=("float", 0.0),
                       normal=("image", "normal.png")),
    "plain.ptmat": dict(albedo=("rgb", 0.5, 0.6, 0.5), rough=("float", 0.3), metal=("float", 0.0),
                        normal=("rgb", 0.5, 0.5, 1.0)),
    "light.ptmat": dict(emission=("image", "emit.png"), intensity=6.0),
}

# geometry: room [0,4] x [0,3] x [0,4], camera looking at the back wall (z = 0)
QUADS = [
    ("floor.ptobj", [(0, 0, 4), (4, 0, 4), (4, 0, 0), (0, 0, 0)], (0, 1, 0), (1, 0, 0), 1.75, "floor.ptmat"),
    ("back.ptobj", [(0, 0, 0), (4, 0, 0), (4, 3, 0), (0, 3, 0)], (0, 0, 1), (1, 0, 0), 1.0, "back.ptmat"),
    ("left.ptobj", [(0, 0, 4), (0, 0, 0), (0, 3, 0), (0, 3, 4)], (1, 0, 0), (0, 0, -1), 1.0, "side.ptmat"),
    ("right.ptobj", [(4, 0, 0), (4, 0, 4), (4, 3, 4), (4, 3, 0)], (-1, 0, 0), (0, 0, 1), 1.0, "plain.ptmat"),
    ("ceil.ptobj", [(0, 3, 0), (4, 3, 0), (4, 3, 4), (0, 3, 4)], (0, -1, 0), (1, 0, 0), 1.0, "plain.ptmat"),
    ("light.ptobj", [(1.5, 2.99, 1.5), (2.5, 2.99, 1.5), (2.5, 2.99, 2.5), (1.5, 2.99, 2.5)], (0, -1, 0),
     (1, 0, 0), 1.0, "light.ptmat"),
]


def _f(x) -> str:
    return format(float(np.float32(x)), ".9g")


def _uvs(scale):
    return [(0.0, 0.0), (scale, 0.0), (scale, scale), (0.0, scale)]


def _slot(t) -> str:
    if t[0] == "image":
        return f"image({t[1]})"
    if t[0] == "float":
        return f"float({_f(t[1])})"
    return "rgb(" + ",".join(_f(x) for x in t[1:]) + ")"


def _material_text(m: dict) -> str:
    if "emission" in m:
        return f"EMISSION {_slot(m['emission'])} float({_f(m['intensity'])})\n"
    # DISNEY albedo spec roughness metal transparent ior normal alpha
    return (f"DISNEY {_slot(m['albedo'])} float(0.5) {_slot(m['rough'])} {_slot(m['metal'])} float(0) float(1.5) "
            f"{_slot(m['normal'])} float(1) -\n")


def _textures(directory: str):
    rng = np.random.default_rng(12)
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


def _quad_file(path, corners, normal, tangent, uv_scale):
    with open(path, "w") as f:
        f.write("4 2 TRIANGLE_MESH\n")
        for p, uv in zip(corners, _uvs(uv_scale)):
            f.write(" ".join(_f(x) for x in (*p, *uv, *normal, *tangent)) + "\n")
        f.write("0 1 2\n0 2 3\n")


def write(directory: str, spp_axis: int = 1) -> str:
    """Writes the room's files; returns the settings path."""
    os.makedirs(directory, exist_ok=True)
    _textures(directory)
    for name, m in MATERIALS.items():
        with open(os.path.join(directory, name), "w") as f:
            f.write(_material_text(m))
    lines = ["camera " + " ".join(_f(x) for x in CAMERA)]
    for obj, corners, n, t, s, mat in QUADS:
        _quad_file(os.path.join(directory, obj), corners, n, t, s)
        lines.append(f"obj {obj} {mat}")
    scene = os.path.join(directory, "scene.ptscene")
    with open(scene, "w") as f:
        f.write("\n".join(lines) + "\n")
    settings = os.path.join(directory, "settings.txt")
    with open(settings, "w") as f:
        f.write(f"renderer pathtracer_mis\nspp {spp_axis}\nresolution {W} {H}\nscene {scene}\n"
                f"output {os.path.join(directory, 'out')}\n")
    return settings


def port_inputs(directory: str, image_load):
    """The room as flat arrays for the oracle port: a cpppt.scenes.Scene,
    per-vertex uv and the texture tables of or_scene_set_textures, with the
    texture pixels from image_load(path, rgb, srgb) (the reference's own
    Image loader through the harness) on the files `write` put in
    `directory`."""
    from cpppt.scenes import DIFFUSE, EMISSIVE, GGX, Scene
    names = list(MATERIALS)
    tex_keys, tex_info, tex_px = {}, [], []

    def tex(file, rgb, srgb):
        key = (file, rgb, srgb)
        if key not in tex_keys:
            px = image_load(os.path.join(directory, file), rgb=rgb, srgb=srgb).astype(np.float32)
            tex_keys[key] = len(tex_info)
            tex_info.append([sum(len(p) for p in tex_px), px.shape[1], px.shape[0], 3 if rgb else 1])
            tex_px.append(px.reshape(-1))
        return tex_keys[key]

    kinds, params, mat_tex, emit = [], [], [], []
    for name in names:
        m = MATERIALS[name]
        if "emission" in m:
            kinds.append(EMISSIVE)
            c = m["emission"]
            params.append([1, 1, 1, 0, 0, m["intensity"], 0, 0] if c[0] == "image" else [*c[1:], 0, 0,
                                                                                          m["intensity"], 0, 0])
            mat_tex.append([tex(c[1], True, True) if c[0] == "image" else -1, -1, -1, -1])
            emit.append(m["intensity"])
            continue
        a, r, me, nm = m["albedo"], m["rough"], m["metal"], m["normal"]
        kinds.append(GGX if me[0] == "float" and me[1] >= 0.1 else DIFFUSE)
        params.append([*(a[1:] if a[0] == "rgb" else (0, 0, 0)), r[1] if r[0] == "float" else 0, 1.5, 0, 0, 0])
        mat_tex.append([tex(a[1], True, True) if a[0] == "image" else -1,
                        tex(r[1], False, False) if r[0] == "image" else -1,
                        tex(me[1], False, False) if me[0] == "image" else -1,
                        tex(nm[1], True, False) if nm[0] == "image" else -1])
        emit.append(0.0)
    verts, nrms, tans, uvs, tris, vo, to, mm = [], [], [], [], [], [0], [0], []
    for obj, corners, n, t, s, mat in QUADS:
        base = len(verts)
        for p, uv in zip(corners, _uvs(s)):
            verts.append(p)
            nrms.append(n)
            tans.append(t)
            uvs.append(uv)
        tris += [(base, base + 1, base + 2), (base, base + 2, base + 3)]
        vo.append(len(verts))
        to.append(len(tris))
        mm.append(names.index(mat))
    f32 = lambda x: np.asarray(x, np.float32)  # noqa: E731
    i32 = lambda x: np.asarray(x, np.int32)  # noqa: E731
    sc = Scene(vertices=f32(verts), normals=f32(nrms), tangents=f32(tans), triangles=i32(tris),
               mesh_vert_offset=i32(vo), mesh_tri_offset=i32(to), mesh_material=i32(mm), mat_kind=i32(kinds),
               mat_params=f32(params), camera=f32(CAMERA), width=W, height=H, name="texroom")
    return (sc, f32(uvs).reshape(-1), i32(tex_info).reshape(-1), np.concatenate(tex_px).astype(np.float32),
            i32(mat_tex).reshape(-1), f32(emit))
