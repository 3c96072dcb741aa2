"""Writes a scene in the reference's text formats (src/loader/loader.h):

* settings file: `renderer pathtracer_mis`, `spp N` (N*N samples per pixel),
  `resolution W H`, `scene <file>`, `output <name>` (loader.h:256-311);
* .ptscene: `camera ox oy oz ax ay az ux uy uz tan_fovy` and
  `obj <mesh>.ptobj <material>.ptmat` lines (loader.h:314-351);
* .ptobj: `n_v n_f TRIANGLE_MESH`, then n_v lines `px py pz u v nx ny nz tx ty tz`
  and n_f lines `a b c` (loader.h:209-251);
* .ptmat: `DISNEY albedo spec roughness metal transparent ior normal alpha`
  or `EMISSION rgb(r,g,b) float(I)` (loader.h:146-207).  Dielectrics, which
  the reference format cannot express, are written as `DIELECTRIC float(ior)`
  (read by this library's loader only).

Floats are written with 9 significant digits, which round-trips float32.
"""
from __future__ import annotations

import os

import numpy as np

from .scenes import DIELECTRIC, EMISSIVE, GGX


def _f(x) -> str:
    return format(float(np.float32(x)), ".9g")


def material_text(kind: int, p) -> str:
    if kind == EMISSIVE:
        return f"EMISSION rgb({_f(p[0])},{_f(p[1])},{_f(p[2])}) float({_f(p[5])})\n"
    if kind == DIELECTRIC:
        return f"DIELECTRIC float({_f(p[4])})\n"
    metal = "float(1)" if kind == GGX else "float(0)"
    return (f"DISNEY rgb({_f(p[0])},{_f(p[1])},{_f(p[2])}) float(0.5) float({_f(p[3])}) {metal} float(0) "
            f"float({_f(p[4])}) rgb(0.5,0.5,1) float(1) -\n")


def write(sc, directory: str, spp_axis: int = 1, output: str = "out", renderer: str = "pathtracer_mis") -> str:
    """Writes the scene files into `directory`; returns the settings path."""
    os.makedirs(directory, exist_ok=True)
    lines = []
    c = sc.camera
    lines.append("camera " + " ".join(_f(x) for x in c[0:9]) + " " + _f(c[9]))
    for m in range(len(sc.mesh_material)):
        v0, v1 = sc.mesh_vert_offset[m], sc.mesh_vert_offset[m + 1]
        f0, f1 = sc.mesh_tri_offset[m], sc.mesh_tri_offset[m + 1]
        obj = f"mesh{m}.ptobj"
        with open(os.path.join(directory, obj), "w") as f:
            f.write(f"{v1 - v0} {f1 - f0} TRIANGLE_MESH\n")
            for v in range(v0, v1):
                p, n, t = sc.vertices[v], sc.normals[v], sc.tangents[v]
                f.write(" ".join(_f(x) for x in (*p, 0.0, 0.0, *n, *t)) + "\n")
            for tri in sc.triangles[f0:f1]:
                f.write(f"{tri[0] - v0} {tri[1] - v0} {tri[2] - v0}\n")
        mi = int(sc.mesh_material[m])
        mat = f"mat{mi}.ptmat"
        path = os.path.join(directory, mat)
        if not os.path.exists(path):
            with open(path, "w") as f:
                f.write(material_text(int(sc.mat_kind[mi]), sc.mat_params[mi]))
        lines.append(f"obj {obj} {mat}")
    scene_path = os.path.join(directory, "scene.ptscene")
    # No blank or comment-only lines: the reference's trim() (loader.h:99-106)
    # calls substr(npos) on them and throws.
    with open(scene_path, "w") as f:
        f.write("\n".join(lines) + "\n")
    settings = os.path.join(directory, "settings.txt")
    with open(settings, "w") as f:
        f.write(f"renderer {renderer}\nspp {spp_axis}\nresolution {sc.width} {sc.height}\n"
                f"scene {scene_path}\noutput {os.path.join(directory, output)}\n")
    return settings
