"""ctypes front end of the oracle.  TEST INFRASTRUCTURE ONLY.

Two CPU implementations of the reference's PathtracerMIS + BVH path sit
behind the same Python interface:

* ``Oracle("port")``: oracle/pt_oracle.c, the C restatement
  (liboracle built here by ``build()``);
* ``Oracle("reference")``: the reference's own code compiled by
  oracle/build_ref.sh into oracle/_ref/libref_harness.so.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module, and only as a checker or as the timed CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libpt_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref_harness.so")
# Root of the reference checkout (drcd1/cpp-pt); only the harness build reads it.
REFERENCE_ROOT = os.environ.get("CPPPT_REFERENCE_ROOT", "/root/reference")


def build(force: bool = False) -> str:
    """Compiles pt_oracle.c (-O2 -fopenmp -ffp-contract=off)."""
    src = os.path.join(HERE, "pt_oracle.c")
    if not force and os.path.exists(PORT_SO) and os.path.getmtime(PORT_SO) >= os.path.getmtime(src):
        return PORT_SO
    os.makedirs(os.path.dirname(PORT_SO), exist_ok=True)
    cc = os.environ.get("CC", "gcc")
    subprocess.check_call([cc, "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11",
                           "-o", PORT_SO, src, "-lm"])
    return PORT_SO


def build_reference(force: bool = False) -> str | None:
    """Runs oracle/build_ref.sh when the reference sources (or a copy made
    earlier under oracle/_ref/src) are present.  Returns the library path or
    None when neither exists."""
    harness = os.path.join(HERE, "ref_harness.cpp")
    have_src = os.path.isdir(os.path.join(REFERENCE_ROOT, "src")) or os.path.isdir(os.path.join(HERE, "_ref", "src"))
    if not have_src:
        return None
    if not force and os.path.exists(REF_SO) and os.path.getmtime(REF_SO) >= os.path.getmtime(harness):
        return REF_SO
    subprocess.check_call(["bash", os.path.join(HERE, "build_ref.sh"), REFERENCE_ROOT],
                          stdout=subprocess.DEVNULL)
    return REF_SO


def reference_available() -> bool:
    return os.path.exists(REF_SO)


_P = C.c_void_p
_FP = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_IP = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_UP = np.ctypeslib.ndpointer(np.uint8, flags="C_CONTIGUOUS")


class Oracle:
    """One CPU implementation ("port" or "reference") of the path."""

    _libs: dict = {}

    def __init__(self, kind: str = "port"):
        self.kind = kind
        if kind not in Oracle._libs:
            path = build() if kind == "port" else REF_SO
            if kind == "reference" and not os.path.exists(path):
                raise FileNotFoundError("reference harness not built (oracle/build_ref.sh)")
            lib = C.CDLL(path)
            p = "or_" if kind == "port" else "ref_"
            create = getattr(lib, p + "scene_create")
            create.restype = _P
            create.argtypes = [C.c_int, _IP, _IP, _IP, _FP, _FP, _FP, _IP, C.c_int, _IP, _FP, _FP, C.c_int, C.c_int]
            getattr(lib, p + "scene_destroy").argtypes = [_P]
            getattr(lib, p + "trace_closest").argtypes = [_P, _FP, C.c_int, _IP, _FP]
            getattr(lib, p + "trace_any").argtypes = [_P, _FP, C.c_int, _UP]
            dump = getattr(lib, p + "bvh_dump")
            dump.restype = C.c_int
            dump.argtypes = [_P, _IP, _FP, _IP, _IP, C.c_int]
            if kind == "port":
                lib.or_render_mis.argtypes = [_P, C.c_int, C.c_int, C.c_int, _FP]
                lib.or_render_mis_cols.argtypes = [_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _FP]
                lib.or_render_variant.argtypes = [_P, C.c_int, C.c_int, C.c_int, C.c_int, _FP]
                lib.or_bsdf_eval.argtypes = [C.c_int, _FP, _FP, _FP, _FP, _FP, _FP, _FP, _IP]
                lib.or_bsdf_sample.argtypes = [C.c_int, _FP, _FP, _FP, _FP, _FP, _FP, _FP, _IP]
                lib.or_light_sample.argtypes = [_P, C.c_int, _FP, _FP]
                lib.or_scene_set_fast.argtypes = [_P, C.c_int]
                lib.or_scene_set_textures.argtypes = [_P, _FP, C.c_int, _IP, _FP, C.c_long, _IP, _FP]
            else:
                lib.ref_render_mis.restype = C.c_double
                lib.ref_render_mis.argtypes = [_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_char_p, _FP]
                lib.ref_render_variant.restype = C.c_double
                lib.ref_render_variant.argtypes = [_P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_char_p, _FP]
                lib.ref_render_ppg.restype = C.c_double
                lib.ref_render_ppg.argtypes = [_P, C.c_int, C.c_int, C.c_int, C.c_char_p, _FP]
                lib.ref_scene_error.restype = C.c_char_p
                lib.ref_scene_error.argtypes = [_P]
                lib.ref_max_threads.restype = C.c_int
                lib.ref_sdtree_run.restype = C.c_int
                lib.ref_sdtree_run.argtypes = [C.c_void_p] * 2 + [C.c_int] + [C.c_void_p] * 2 + [C.c_int] + \
                    [C.c_void_p] * 4 + [C.c_int] + [C.c_void_p] * 3
                lib.ref_image_load.restype = C.c_int
                lib.ref_image_load.argtypes = [C.c_char_p, C.c_int, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                               C.c_void_p, C.c_longlong]
                lib.ref_scene_load.restype = _P
                lib.ref_scene_load.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                               C.POINTER(C.c_int)]
            Oracle._libs[kind] = lib
        self.lib = Oracle._libs[kind]
        self.p = "or_" if kind == "port" else "ref_"

    def scene(self, sc) -> "OracleScene":
        return OracleScene(self, sc)

    def image_load(self, path: str, rgb: bool = True, srgb: bool = True) -> np.ndarray:
        """An image file as the reference's Image<Vec3> / Image<float> holds
        it (rgb_image.h:160-205)."""
        assert self.kind == "reference"
        w, h = C.c_int(), C.c_int()
        self.lib.ref_image_load(path.encode(), int(rgb), int(srgb), C.byref(w), C.byref(h), None, 0)
        out = np.zeros((h.value, w.value, 3) if rgb else (h.value, w.value), np.float32)
        rc = self.lib.ref_image_load(path.encode(), int(rgb), int(srgb), C.byref(w), C.byref(h), out.ctypes.data,
                                     out.size)
        assert rc == 0
        return out

    def load_files(self, settings_file: str) -> "OracleScene":
        """The reference's own Loader (loader.h:256-374) on scene files."""
        assert self.kind == "reference"
        w, h, spp = C.c_int(), C.c_int(), C.c_int()
        hnd = self.lib.ref_scene_load(settings_file.encode(), C.byref(w), C.byref(h), C.byref(spp))
        err = self.lib.ref_scene_error(hnd)
        s = OracleScene.__new__(OracleScene)
        s.o, s.sc, s.h, s._keep = self, None, hnd, []
        s.width, s.height, s.spp_axis = w.value, h.value, spp.value
        if err:
            raise RuntimeError("reference loader: " + err.decode())
        return s


class OracleScene:
    def __init__(self, oracle: Oracle, sc):
        self.o = oracle
        self.sc = sc
        lib, p = oracle.lib, oracle.p
        self._keep = [np.ascontiguousarray(a) for a in (
            sc.mesh_vert_offset, sc.mesh_tri_offset, sc.mesh_material, sc.vertices.reshape(-1),
            sc.normals.reshape(-1), sc.tangents.reshape(-1), sc.triangles.reshape(-1), sc.mat_kind,
            sc.mat_params.reshape(-1), sc.camera)]
        k = self._keep
        self.h = getattr(lib, p + "scene_create")(
            len(sc.mesh_material), k[0], k[1], k[2], k[3], k[4], k[5], k[6], len(sc.mat_kind), k[7], k[8], k[9],
            sc.width, sc.height)
        if oracle.kind == "reference":
            err = lib.ref_scene_error(self.h)
            if err:
                raise RuntimeError("reference scene: " + err.decode())

    def close(self):
        if self.h:
            getattr(self.o.lib, self.o.p + "scene_destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def trace_closest(self, rays: np.ndarray):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1)
        n = rays.size // 7
        idx = np.zeros(n, np.int32)
        t = np.zeros(n, np.float32)
        getattr(self.o.lib, self.o.p + "trace_closest")(self.h, rays, n, idx, t)
        return idx, t

    def trace_any(self, rays: np.ndarray):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1)
        n = rays.size // 7
        out = np.zeros(n, np.uint8)
        getattr(self.o.lib, self.o.p + "trace_any")(self.h, rays, n, out)
        return out

    def bvh_dump(self):
        n = self.sc.n_triangles
        cap = max(2 * n, 16)
        order = np.zeros(n, np.int32)
        boxes = np.zeros(6 * cap, np.float32)
        parent = np.zeros(cap, np.int32)
        pparent = np.zeros(n, np.int32)
        nn = getattr(self.o.lib, self.o.p + "bvh_dump")(self.h, order, boxes, parent, pparent, cap)
        return order, boxes[:6 * nn].reshape(nn, 6), parent[:nn], pparent

    def set_textures(self, uv, tex_info, tex_px, mat_tex, mat_emit):
        """Image textures (port only): uv per vertex, {first float, w, h,
        channels} per texture, the pixels, four texture indices per material
        (albedo or emission colour, roughness, metal, normal map; -1:
        constant) and the intensity of textured emitters."""
        assert self.o.kind == "port"
        k = [np.ascontiguousarray(a) for a in (uv, tex_info, tex_px, mat_tex, mat_emit)]
        self._keep += k
        self.o.lib.or_scene_set_textures(self.h, k[0], len(k[1]) // 4, k[1], k[2], len(k[2]), k[3], k[4])
        return self

    def _dims(self):
        """Image size: the scene's, or the settings file's for a loaded scene."""
        return (self.sc.width, self.sc.height) if self.sc is not None else (self.width, self.height)

    def render_mis(self, spp_axis: int, max_depth: int, seed_offset: int = 0, threads: int = 0):
        """Returns (image HxWx3 float32, seconds).  spp_axis^2 samples per pixel."""
        W, H = self._dims()
        out = np.zeros(W * H * 3, np.float32)
        if self.o.kind == "port":
            import time
            t0 = time.perf_counter()
            self.o.lib.or_render_mis(self.h, spp_axis, max_depth, seed_offset, out)
            sec = time.perf_counter() - t0
        else:
            with tempfile.TemporaryDirectory() as d:
                sec = self.o.lib.ref_render_mis(self.h, spp_axis, max_depth, seed_offset, threads,
                                                os.path.join(d, "img").encode(), out)
        return out.reshape(H, W, 3), sec

    def render_variant(self, integrator: int, spp_axis: int, max_depth: int, seed_offset: int = 0,
                       threads: int = 0):
        """integrator 1: Pathtracer (PT + NEE, no MIS); 2: PurePt (no NEE).
        Returns (image HxWx3 float32, seconds)."""
        W, H = self._dims()
        out = np.zeros(W * H * 3, np.float32)
        if self.o.kind == "port":
            import time
            t0 = time.perf_counter()
            self.o.lib.or_render_variant(self.h, integrator, spp_axis, max_depth, seed_offset, out)
            sec = time.perf_counter() - t0
        else:
            with tempfile.TemporaryDirectory() as d:
                sec = self.o.lib.ref_render_variant(self.h, integrator, spp_axis, max_depth, seed_offset, threads,
                                                    os.path.join(d, "img").encode(), out)
        return out.reshape(H, W, 3), sec

    def set_fast(self, fast: bool = True):
        """Port only: queries by the culling traversal, which gives the
        exhaustive recursion's answers (checked by test_oracle_pins.py) at a
        cost that scales with log(triangles) instead of with the tree."""
        assert self.o.kind == "port"
        self.o.lib.or_scene_set_fast(self.h, int(fast))
        return self

    def light_sample(self, cases):
        """LightGroup::connect_eye_path on given numbers (port only): cases =
        n x 6 (from xyz, u0, u1, u2) -> n x 10 (position, normal, Le |cos|,
        pdf)."""
        assert self.o.kind == "port"
        c = np.ascontiguousarray(np.asarray(cases, np.float32).reshape(-1))
        n = c.size // 6
        out = np.zeros(10 * n, np.float32)
        self.o.lib.or_light_sample(self.h, n, c, out)
        return out.reshape(n, 10)

    def render_ppg(self, spp_axis: int, seed_offset: int = 0, threads: int = 0):
        W, H = self._dims()
        out = np.zeros(W * H * 3, np.float32)
        with tempfile.TemporaryDirectory() as d:
            sec = self.o.lib.ref_render_ppg(self.h, spp_axis, seed_offset, threads, os.path.join(d, "img").encode(), out)
        return out.reshape(H, W, 3), sec


def bsdf_eval(params, normal, tangent, wo, wi):
    """Oracle BSDF eval/pdf/non_zero on a flat shading frame (first hit)."""
    lib = Oracle("port").lib
    n = len(params)
    f = lambda a: np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1))
    ev = np.zeros(3 * n, np.float32)
    pdf = np.zeros(n, np.float32)
    nz = np.zeros(n, np.int32)
    lib.or_bsdf_eval(n, f(params), f(normal), f(tangent), f(wo), f(wi), ev, pdf, nz)
    return ev.reshape(n, 3), pdf, nz


def bsdf_sample(params, normal, tangent, wo, u):
    """Oracle BxDF::sample on given uniform numbers u (n x 2): (wi, pdf, delta)."""
    lib = Oracle("port").lib
    n = len(params)
    f = lambda a: np.ascontiguousarray(np.asarray(a, np.float32).reshape(-1))
    wi = np.zeros(3 * n, np.float32)
    pdf = np.zeros(n, np.float32)
    delta = np.zeros(n, np.int32)
    lib.or_bsdf_sample(n, f(params), f(normal), f(tangent), f(wo), f(u), wi, pdf, delta)
    return wi.reshape(n, 3), pdf, delta
