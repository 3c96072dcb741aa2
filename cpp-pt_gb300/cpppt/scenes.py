"""Seeded synthetic scenes in the reference's scene model.

A scene is flat arrays in the reference's insertion order
(src/loader/loader.h:353-367): meshes one after another, each with one
material, triangles of a mesh in file order.  The global primitive index of a
triangle is its position in ``triangles``.

Vertex data follow the .ptobj layout (loader.h:226-240): position, normal and
a tangent per vertex (the loader turns the tangent into a bitangent,
cross(normal, tangent)).  Winding matches the normals, as
BxDF::same_hemisphere (src/bxdf/bxdf.h:42-45) requires.

Material kinds: 0 Lambert (StandardMaterial with metal 0), 1 GGX conductor
(metal 1), 2 smooth dielectric, 3 emitter (EmissiveMaterial).  ``mat_params``
holds 8 floats per material: r, g, b, roughness, ior, intensity, 0, 0.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

DIFFUSE, GGX, DIELECTRIC, EMISSIVE = 0, 1, 2, 3


@dataclass
class Scene:
    vertices: np.ndarray  # (V,3) f32
    normals: np.ndarray  # (V,3) f32
    tangents: np.ndarray  # (V,3) f32
    triangles: np.ndarray  # (T,3) i32, global vertex indices
    mesh_vert_offset: np.ndarray  # (M+1,) i32
    mesh_tri_offset: np.ndarray  # (M+1,) i32
    mesh_material: np.ndarray  # (M,) i32
    mat_kind: np.ndarray  # (K,) i32
    mat_params: np.ndarray  # (K,8) f32
    camera: np.ndarray  # (10,) f32: origin, at, up, tan_fovy
    width: int
    height: int
    name: str = "scene"
    meta: dict = field(default_factory=dict)

    @property
    def n_triangles(self) -> int:
        return int(self.triangles.shape[0])

    @property
    def tri_material(self) -> np.ndarray:
        counts = np.diff(self.mesh_tri_offset)
        return np.repeat(self.mesh_material, counts).astype(np.int32)

    def with_resolution(self, width: int, height: int) -> "Scene":
        s = Scene(**{k: getattr(self, k) for k in self.__dataclass_fields__})
        s.width, s.height = int(width), int(height)
        return s


class _Builder:
    def __init__(self):
        self.v, self.n, self.t, self.f = [], [], [], []
        self.mesh_v, self.mesh_f, self.mesh_m = [0], [0], []
        self.kinds, self.params = [], []
        self.nv = 0

    def material(self, kind, rgb=(0.0, 0.0, 0.0), roughness=0.0, ior=1.5, intensity=0.0) -> int:
        self.kinds.append(kind)
        self.params.append([rgb[0], rgb[1], rgb[2], roughness, ior, intensity, 0.0, 0.0])
        return len(self.kinds) - 1

    def mesh(self, pos, nrm, tan, faces, mat):
        pos = np.asarray(pos, np.float32).reshape(-1, 3)
        self.v.append(pos)
        self.n.append(np.asarray(nrm, np.float32).reshape(-1, 3))
        self.t.append(np.asarray(tan, np.float32).reshape(-1, 3))
        self.f.append(np.asarray(faces, np.int64).reshape(-1, 3) + self.nv)
        self.nv += pos.shape[0]
        self.mesh_v.append(self.nv)
        self.mesh_f.append(self.mesh_f[-1] + len(self.f[-1]))
        self.mesh_m.append(mat)

    def build(self, camera, width, height, name, **meta) -> Scene:
        return Scene(
            vertices=np.ascontiguousarray(np.concatenate(self.v), np.float32),
            normals=np.ascontiguousarray(np.concatenate(self.n), np.float32),
            tangents=np.ascontiguousarray(np.concatenate(self.t), np.float32),
            triangles=np.ascontiguousarray(np.concatenate(self.f), np.int32),
            mesh_vert_offset=np.asarray(self.mesh_v, np.int32),
            mesh_tri_offset=np.asarray(self.mesh_f, np.int32),
            mesh_material=np.asarray(self.mesh_m, np.int32),
            mat_kind=np.asarray(self.kinds, np.int32),
            mat_params=np.asarray(self.params, np.float32).reshape(-1, 8),
            camera=np.asarray(camera, np.float32),
            width=int(width),
            height=int(height),
            name=name,
            meta=meta,
        )


def _perp(n: np.ndarray) -> np.ndarray:
    """A unit tangent perpendicular to each normal."""
    n = np.asarray(n, np.float64).reshape(-1, 3)
    a = np.where(np.abs(n[:, 1:2]) < 0.9, np.array([[0.0, 1.0, 0.0]]), np.array([[1.0, 0.0, 0.0]]))
    t = np.cross(a, n)
    t /= np.linalg.norm(t, axis=1, keepdims=True)
    return t


def _quad(b: _Builder, p0, p1, p2, p3, normal, mat, subdiv: int = 1):
    """Planar quad p0,p1,p2,p3 (counter-clockwise seen from `normal`),
    split into subdiv x subdiv cells of two triangles."""
    p0, p1, p2, p3 = (np.asarray(p, np.float64) for p in (p0, p1, p2, p3))
    k = subdiv
    uu, vv = np.meshgrid(np.linspace(0, 1, k + 1), np.linspace(0, 1, k + 1), indexing="ij")
    uu, vv = uu.reshape(-1, 1), vv.reshape(-1, 1)
    pos = (1 - uu) * (1 - vv) * p0 + uu * (1 - vv) * p1 + uu * vv * p2 + (1 - uu) * vv * p3
    nrm = np.tile(np.asarray(normal, np.float64), (pos.shape[0], 1))
    faces = []
    for i in range(k):
        for j in range(k):
            a = i * (k + 1) + j
            bb = (i + 1) * (k + 1) + j
            c = (i + 1) * (k + 1) + j + 1
            d = i * (k + 1) + j + 1
            faces.append((a, bb, c))
            faces.append((a, c, d))
    faces = np.asarray(faces)
    # orient the winding so cross(b-a, c-a) agrees with the normal
    e = np.cross(pos[faces[0, 1]] - pos[faces[0, 0]], pos[faces[0, 2]] - pos[faces[0, 0]])
    if np.dot(e, normal) < 0:
        faces = faces[:, [0, 2, 1]]
    b.mesh(pos, nrm, _perp(nrm), faces, mat)


def _box(b: _Builder, center, size, angle_y, mat, subdiv: int = 1):
    """Axis-aligned box rotated about y, outward normals, as 6 quads."""
    c = np.asarray(center, np.float64)
    hx, hy, hz = (0.5 * np.asarray(size, np.float64)).tolist()
    ca, sa = math.cos(angle_y), math.sin(angle_y)
    R = np.array([[ca, 0, sa], [0, 1, 0], [-sa, 0, ca]])

    def P(x, y, z):
        return R @ np.array([x, y, z]) + c

    faces = [
        ((0, -1, 0), [P(-hx, -hy, -hz), P(hx, -hy, -hz), P(hx, -hy, hz), P(-hx, -hy, hz)]),
        ((0, 1, 0), [P(-hx, hy, -hz), P(-hx, hy, hz), P(hx, hy, hz), P(hx, hy, -hz)]),
        ((-1, 0, 0), [P(-hx, -hy, -hz), P(-hx, -hy, hz), P(-hx, hy, hz), P(-hx, hy, -hz)]),
        ((1, 0, 0), [P(hx, -hy, -hz), P(hx, hy, -hz), P(hx, hy, hz), P(hx, -hy, hz)]),
        ((0, 0, -1), [P(-hx, -hy, -hz), P(-hx, hy, -hz), P(hx, hy, -hz), P(hx, -hy, -hz)]),
        ((0, 0, 1), [P(-hx, -hy, hz), P(hx, -hy, hz), P(hx, hy, hz), P(-hx, hy, hz)]),
    ]
    for n, q in faces:
        _quad(b, *q, R @ np.asarray(n, np.float64), mat, subdiv)


def cornell(width: int = 256, height: int = 256) -> Scene:
    """Procedural Cornell box in [0,1]^3: 5 Lambert walls (10 triangles), two
    white boxes rotated +-17 degrees (24 triangles), and a 0.25 x 0.25 ceiling
    emitter with radiance (17,12,4), i.e. EMISSION rgb(1,0.70588,0.23529)
    float(17).  36 triangles.  Pinhole camera, 40 degree vertical field of
    view, looking at the back wall (z = 0) through the open side z = 1."""
    b = _Builder()
    white = b.material(DIFFUSE, (0.73, 0.73, 0.73))
    red = b.material(DIFFUSE, (0.65, 0.05, 0.05))
    green = b.material(DIFFUSE, (0.12, 0.45, 0.15))
    light = b.material(EMISSIVE, (1.0, 0.70588, 0.23529), intensity=17.0)
    _quad(b, (0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1), (0, 1, 0), white)  # floor
    _quad(b, (0, 1, 0), (0, 1, 1), (1, 1, 1), (1, 1, 0), (0, -1, 0), white)  # ceiling
    _quad(b, (0, 0, 0), (0, 1, 0), (1, 1, 0), (1, 0, 0), (0, 0, 1), white)  # back
    _quad(b, (0, 0, 0), (0, 0, 1), (0, 1, 1), (0, 1, 0), (1, 0, 0), red)  # left
    _quad(b, (1, 0, 0), (1, 1, 0), (1, 1, 1), (1, 0, 1), (-1, 0, 0), green)  # right
    _box(b, (0.66, 0.15, 0.62), (0.3, 0.3, 0.3), math.radians(-17.0), white)
    _box(b, (0.34, 0.30, 0.36), (0.3, 0.6, 0.3), math.radians(17.0), white)
    y = 0.998
    _quad(b, (0.375, y, 0.375), (0.375, y, 0.625), (0.625, y, 0.625), (0.625, y, 0.375), (0, -1, 0), light)
    tan_fovy = math.tan(math.radians(20.0))
    cam_z = 1.0 + 0.5 / tan_fovy
    camera = [0.5, 0.5, cam_z, 0.5, 0.5, 0.0, 0.0, 1.0, 0.0, tan_fovy]
    return b.build(camera, width, height, "cornell")


def _geodesic_sphere(freq: int):
    """Icosahedron with every face split into freq^2 triangles, vertices
    projected to the unit sphere (20 * freq^2 triangles)."""
    t = (1.0 + 5 ** 0.5) / 2.0
    V0 = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                   [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    F0 = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
          (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
          (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts, index = [], {}

    def vid(p):
        key = tuple(np.round(p / np.linalg.norm(p), 9))
        if key not in index:
            index[key] = len(verts)
            verts.append(p / np.linalg.norm(p))
        return index[key]

    faces = []
    for a, bb, c in F0:
        A, B, C = V0[a], V0[bb], V0[c]
        grid = {}
        for i in range(freq + 1):
            for j in range(freq + 1 - i):
                grid[(i, j)] = vid(A + (B - A) * (i / freq) + (C - A) * (j / freq))
        for i in range(freq):
            for j in range(freq - i):
                faces.append((grid[(i, j)], grid[(i + 1, j)], grid[(i, j + 1)]))
                if j + i + 1 < freq:
                    faces.append((grid[(i + 1, j)], grid[(i + 1, j + 1)], grid[(i, j + 1)]))
    V = np.asarray(verts)
    F = np.asarray(faces)
    e = np.cross(V[F[:, 1]] - V[F[:, 0]], V[F[:, 2]] - V[F[:, 0]])
    out = np.einsum("ij,ij->i", e, V[F[:, 0]]) < 0
    F[out] = F[out][:, [0, 2, 1]]
    return V, F


def soup(seed: int = 2, n_spheres: int = 2000, freq: int = 5, width: int = 1920, height: int = 1080,
         extent: float = 20.0, only: int | None = None, rough_range: tuple = (0.05, 0.5)) -> Scene:
    """Seeded triangle soup of geodesic spheres (20*freq^2 triangles each;
    freq 5 gives 500) with centres uniform in [0, extent]^3 and radii
    log-uniform in [0.05, 1], inside a closed box room.  One material per
    sphere, uniform among Lambert (albedo U[0.1,0.9]), GGX conductor
    (roughness U[0.05,0.5]) and smooth dielectric (IOR 1.5).  Four emissive
    unit quads with radiance 20 under the ceiling.  2000 spheres x 500 gives
    the 1M-triangle configuration.  `only` (DIFFUSE, GGX or DIELECTRIC)
    gives every sphere that material kind, with the same random draws
    otherwise; `rough_range` is the GGX roughness interval."""
    rng = np.random.default_rng(seed)
    b = _Builder()
    lo, hi = -2.0, extent + 2.0
    wall = b.material(DIFFUSE, (0.7, 0.7, 0.7))
    light = b.material(EMISSIVE, (1.0, 1.0, 1.0), intensity=20.0)
    _quad(b, (lo, lo, lo), (hi, lo, lo), (hi, lo, hi), (lo, lo, hi), (0, 1, 0), wall)  # floor
    _quad(b, (lo, hi, lo), (lo, hi, hi), (hi, hi, hi), (hi, hi, lo), (0, -1, 0), wall)  # ceiling
    _quad(b, (lo, lo, hi), (lo, hi, hi), (hi, hi, hi), (hi, lo, hi), (0, 0, -1), wall)  # far
    _quad(b, (lo, lo, lo), (hi, lo, lo), (hi, hi, lo), (lo, hi, lo), (0, 0, 1), wall)  # near
    _quad(b, (lo, lo, lo), (lo, hi, lo), (lo, hi, hi), (lo, lo, hi), (1, 0, 0), wall)  # left
    _quad(b, (hi, lo, lo), (hi, lo, hi), (hi, hi, hi), (hi, hi, lo), (-1, 0, 0), wall)  # right
    yl = hi - 0.01
    for cx, cz in ((0.25, 0.25), (0.75, 0.25), (0.25, 0.75), (0.75, 0.75)):
        x = lo + (hi - lo) * cx
        z = lo + (hi - lo) * cz
        _quad(b, (x - 0.5, yl, z - 0.5), (x - 0.5, yl, z + 0.5), (x + 0.5, yl, z + 0.5), (x + 0.5, yl, z - 0.5),
              (0, -1, 0), light)
    V, F = _geodesic_sphere(freq)
    centres = rng.uniform(0.0, extent, size=(n_spheres, 3))
    radii = np.exp(rng.uniform(math.log(0.05), math.log(1.0), size=n_spheres))
    kinds = rng.integers(0, 3, size=n_spheres)
    albedo = rng.uniform(0.1, 0.9, size=(n_spheres, 3))
    rough = rng.uniform(rough_range[0], rough_range[1], size=n_spheres)
    tang = _perp(V)
    for i in range(n_spheres):
        k = int(kinds[i]) if only is None else int(only)
        if k == 0:
            m = b.material(DIFFUSE, tuple(albedo[i]))
        elif k == 1:
            m = b.material(GGX, (1.0, 1.0, 1.0), roughness=float(rough[i]))
        else:
            m = b.material(DIELECTRIC, (1.0, 1.0, 1.0), ior=1.5)
        b.mesh(V * radii[i] + centres[i], V, tang, F, m)
    tan_fovy = math.tan(math.radians(30.0))
    camera = [extent / 2, extent / 2, lo + 0.5, extent / 2, extent / 2, extent / 2, 0.0, 1.0, 0.0, tan_fovy]
    return b.build(camera, width, height, f"soup{n_spheres}x{20 * freq * freq}", seed=seed)


def slit_room(seed: int = 4, n_boxes: int = 1000, box_subdiv: int = 4, width: int = 1280, height: int = 720) -> Scene:
    """Occluded-light room: 10 x 4 x 10 (x, y, z), seeded clutter of boxes
    (each face split box_subdiv^2 cells; 1000 boxes x 192 = 192k triangles),
    Lambert albedo U[0.2,0.8].  The only emitter (1 x 1, radiance 50) sits in
    a 0.6-deep closet behind a wall at z = 9.4 that has a 0.05-high slit at
    y in [2.0, 2.05], so indirect light dominates."""
    rng = np.random.default_rng(seed)
    b = _Builder()
    wall = b.material(DIFFUSE, (0.75, 0.75, 0.75))
    light = b.material(EMISSIVE, (1.0, 1.0, 1.0), intensity=50.0)
    X, Y, Z = 10.0, 4.0, 10.0
    zw = 9.4
    _quad(b, (0, 0, 0), (X, 0, 0), (X, 0, Z), (0, 0, Z), (0, 1, 0), wall)
    _quad(b, (0, Y, 0), (0, Y, Z), (X, Y, Z), (X, Y, 0), (0, -1, 0), wall)
    _quad(b, (0, 0, 0), (0, Y, 0), (X, Y, 0), (X, 0, 0), (0, 0, 1), wall)
    _quad(b, (0, 0, Z), (X, 0, Z), (X, Y, Z), (0, Y, Z), (0, 0, -1), wall)
    _quad(b, (0, 0, 0), (0, 0, Z), (0, Y, Z), (0, Y, 0), (1, 0, 0), wall)
    _quad(b, (X, 0, 0), (X, Y, 0), (X, Y, Z), (X, 0, Z), (-1, 0, 0), wall)
    # the dividing wall: a thin box below and one above the slit
    ys0, ys1 = 2.0, 2.05
    _box(b, (X / 2, ys0 / 2, zw), (X, ys0, 0.04), 0.0, wall)
    _box(b, (X / 2, (ys1 + Y) / 2, zw), (X, Y - ys1, 0.04), 0.0, wall)
    _quad(b, (4.5, 1.5, Z - 0.01), (5.5, 1.5, Z - 0.01), (5.5, 2.5, Z - 0.01), (4.5, 2.5, Z - 0.01), (0, 0, -1), light)
    for _ in range(n_boxes):
        sx, sy, sz = rng.uniform(0.1, 0.8), rng.uniform(0.1, 1.2), rng.uniform(0.1, 0.8)
        cx, cz = rng.uniform(0.5, X - 0.5), rng.uniform(0.5, zw - 0.6)
        alb = rng.uniform(0.2, 0.8, size=3)
        m = b.material(DIFFUSE, tuple(alb))
        _box(b, (cx, sy / 2 + rng.uniform(0.0, 0.02), cz), (sx, sy, sz), rng.uniform(0, math.pi), m, box_subdiv)
    tan_fovy = math.tan(math.radians(30.0))
    camera = [X / 2, 2.6, 0.3, X / 2, 1.6, zw, 0.0, 1.0, 0.0, tan_fovy]
    return b.build(camera, width, height, f"slitroom{n_boxes}", seed=seed)


def hit_ray_batch(scene: Scene, n: int, seed: int = 6, hit_points: np.ndarray | None = None) -> np.ndarray:
    """Ray batch for closest-hit parity, 7 floats per ray
    {ox,oy,oz,dx,dy,dz,max_t}.  Mix: 50% camera rays, 30% cosine-ish rays
    from `hit_points` (or random interior points), 10% rays aimed at triangle
    edges and vertices (tie cases), 10% axis-parallel directions.  Rays never
    start on an axis-aligned plane of the scene with a direction inside that
    plane (measure-zero case where the reference's triangle test yields NaN
    distances)."""
    rng = np.random.default_rng(seed)
    V = scene.vertices.astype(np.float64)
    F = scene.triangles
    lo, hi = V.min(0), V.max(0)
    cam = scene.camera.astype(np.float64)
    o_cam, at, up = cam[0:3], cam[3:6], cam[6:9]
    fwd = (at - o_cam) / np.linalg.norm(at - o_cam)
    xax = np.cross(up, -fwd); xax /= np.linalg.norm(xax)
    yax = np.cross(-fwd, xax)
    n_cam = n // 2
    n_sec = (3 * n) // 10
    n_edge = n // 10
    n_axis = n - n_cam - n_sec - n_edge
    rays = np.zeros((n, 7), np.float64)
    # camera rays
    u = rng.uniform(-1, 1, size=(n_cam, 2))
    aspect = scene.width / scene.height
    d = (u[:, :1] * cam[9] * aspect) * xax + (u[:, 1:2] * cam[9]) * yax + fwd
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays[:n_cam, 0:3] = o_cam
    rays[:n_cam, 3:6] = d
    # secondary rays from interior points
    if hit_points is None or len(hit_points) == 0:
        pts = lo + (hi - lo) * rng.uniform(0.02, 0.98, size=(n_sec, 3))
    else:
        pts = hit_points[rng.integers(0, len(hit_points), size=n_sec)]
    dd = rng.normal(size=(n_sec, 3))
    dd /= np.linalg.norm(dd, axis=1, keepdims=True)
    rays[n_cam:n_cam + n_sec, 0:3] = pts
    rays[n_cam:n_cam + n_sec, 3:6] = dd
    # rays through edges / vertices of random triangles
    k = n_cam + n_sec
    tri = rng.integers(0, len(F), size=n_edge)
    w = rng.uniform(0, 1, size=n_edge)
    a, bb, c = V[F[tri, 0]], V[F[tri, 1]], V[F[tri, 2]]
    which = rng.integers(0, 4, size=n_edge)
    target = np.where((which == 0)[:, None], a * w[:, None] + bb * (1 - w[:, None]),
                      np.where((which == 1)[:, None], bb * w[:, None] + c * (1 - w[:, None]),
                               np.where((which == 2)[:, None], c * w[:, None] + a * (1 - w[:, None]), a)))
    org = lo + (hi - lo) * rng.uniform(0.05, 0.95, size=(n_edge, 3))
    dd = target - org
    dd /= np.linalg.norm(dd, axis=1, keepdims=True)
    rays[k:k + n_edge, 0:3] = org
    rays[k:k + n_edge, 3:6] = dd
    k += n_edge
    # axis-parallel directions from interior points off every vertex plane
    org = lo + (hi - lo) * rng.uniform(0.03, 0.97, size=(n_axis, 3))
    axis = rng.integers(0, 3, size=n_axis)
    sign = rng.choice([-1.0, 1.0], size=n_axis)
    dd = np.zeros((n_axis, 3))
    dd[np.arange(n_axis), axis] = sign
    rays[k:, 0:3] = org
    rays[k:, 3:6] = dd
    rays[:, 6] = np.inf
    out = rays.astype(np.float32)
    # renormalise in float32 as the reference's normalized() would see it
    for j in range(3):
        bad = (out[:, 3 + j] == 0.0) & np.isin(out[:, j], np.unique(scene.vertices[:, j]))
        out[bad, j] = np.nextafter(out[bad, j], np.float32(np.inf))
    return out
