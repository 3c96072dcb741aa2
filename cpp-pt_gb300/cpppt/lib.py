"""ctypes binding of the C ABI in include/cpppt_gb300.h.

The shared library is built in-tree by cpp-pt_gb300/build.py.  Loading fails
loudly when it is missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(os.path.dirname(HERE), "lib", "libcpppt_gb300.so")

PT_OK = 0
STATUS_NAMES = {0: "PT_OK", 1: "PT_ERR_INVALID", 2: "PT_ERR_CUDA", 3: "PT_ERR_MEMORY", 4: "PT_ERR_LIMIT",
                5: "PT_ERR_IO", 6: "PT_ERR_NO_DEVICE"}
MODE_MIS, MODE_SDTREE, MODE_NN, MODE_NEE, MODE_PT = 0, 1, 2, 3, 4
FLAG_TIME_KERNELS, FLAG_COUNT, FLAG_UNBIASED_MIS, FLAG_NN_FREEZE, FLAG_THROUGHPUT_RR = 1, 2, 4, 8, 16
NN_WEIGHTS = 15360
NN_KL, NN_CHI2 = 0, 1
NN_ENC_FREQ, NN_ENC_ONEBLOB = 0, 1

# every function the header declares
EXPORTS = ["pt_scene_create", "pt_scene_load", "pt_scene_destroy", "pt_scene_info", "pt_trace_closest", "pt_trace_any",
           "pt_trace_closest_device", "pt_trace_any_device", "pt_render", "pt_render_device",
           "pt_render_device_noalloc",
           "pt_render_stats_get", "pt_image_save", "pt_last_error", "pt_debug_ref_topology",
           "pt_debug_sdtree_run", "pt_nn_get_weights", "pt_nn_set_weights", "pt_nn_reset", "pt_nn_stats",
           "pt_debug_nn_forward", "pt_debug_nn_forward_ex", "pt_debug_nn_grad", "pt_debug_nn_grad_ex", "pt_nn_configure", "pt_nn_config_get",
           "pt_batch_create", "pt_batch_destroy", "pt_batch_render", "pt_batch_render_device", "pt_batch_set_tuning",
           "pt_batch_get_tuning", "pt_batch_stats", "pt_batch_autotune", "pt_set_mesh_cache",
           "pt_batch_render_ex", "pt_batch_render_ex_device", "pt_debug_image_load", "pt_debug_ref_topology_device", "pt_debug_wide_bvh", "pt_debug_bsdf",
           "pt_debug_light_sample", "pt_debug_traversal_limits", "pt_debug_tensor_wait_timeout"]


class PtMaterial(C.Structure):
    _fields_ = [("kind", C.c_int32), ("rgb", C.c_float * 3), ("roughness", C.c_float), ("ior", C.c_float),
                ("intensity", C.c_float), ("reserved", C.c_float)]


class PtCamera(C.Structure):
    _fields_ = [("origin", C.c_float * 3), ("at", C.c_float * 3), ("up", C.c_float * 3), ("tan_fovy", C.c_float),
                ("width", C.c_int32), ("height", C.c_int32)]


class PtSceneDesc(C.Structure):
    _fields_ = [("n_vertices", C.c_int32), ("vertices", C.c_void_p), ("normals", C.c_void_p),
                ("tangents", C.c_void_p), ("n_triangles", C.c_int32), ("triangles", C.c_void_p),
                ("tri_material", C.c_void_p), ("n_materials", C.c_int32), ("materials", C.c_void_p),
                ("camera", PtCamera)]


class PtRenderDesc(C.Structure):
    _fields_ = [("spp", C.c_int32), ("max_depth", C.c_int32), ("rr_start", C.c_int32), ("seed", C.c_uint32),
                ("mode", C.c_int32), ("flags", C.c_int32)]


class PtRenderStats(C.Structure):
    _fields_ = [(n, C.c_double) for n in ("paths", "closest_rays", "shadow_rays", "render_ms", "trace_closest_ms",
                                           "trace_shadow_ms", "iterations", "kernel_launches", "extend_nodes",
                                           "extend_tris", "h2d_bytes", "d2h_bytes", "nonfinite",
                                           "film_overflow")]


class PtNNConfig(C.Structure):
    _fields_ = [("learning_rate", C.c_float), ("bsdf_frac_min", C.c_float), ("bsdf_frac_max", C.c_float),
                ("batch", C.c_int32), ("divergence", C.c_int32), ("steps_per_round", C.c_int32),
                ("encoding", C.c_int32), ("passes", C.c_int32)]


class PtBatchJob(C.Structure):
    _fields_ = [("scene", C.c_int32), ("spp", C.c_int32), ("max_depth", C.c_int32), ("rr_start", C.c_int32),
                ("seed", C.c_uint32)]


class PtBatchTuning(C.Structure):
    _fields_ = [("capacity", C.c_int32), ("iters_per_graph", C.c_int32), ("tile_w", C.c_int32),
                ("tile_h", C.c_int32)]


class PtError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


_lib = None


def load(path: str = LIB_PATH):
    """Loads the library (no CUDA call is made)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} is missing: build it with cpp-pt_gb300/build.py")
    lib = C.CDLL(path)
    P = C.c_void_p
    lib.pt_scene_create.argtypes = [C.POINTER(PtSceneDesc), C.POINTER(P)]
    lib.pt_scene_load.argtypes = [C.c_char_p, C.POINTER(P), C.POINTER(PtRenderDesc), C.c_char_p, C.c_int32]
    lib.pt_scene_destroy.argtypes = [P]
    lib.pt_scene_destroy.restype = None
    lib.pt_scene_info.argtypes = [P, P, P, P, P]
    lib.pt_trace_closest.argtypes = [P, P, C.c_int32, P]
    lib.pt_trace_any.argtypes = [P, P, C.c_int32, P]
    lib.pt_trace_closest_device.argtypes = [P, P, C.c_int32, P, P]
    lib.pt_trace_any_device.argtypes = [P, P, C.c_int32, P, P]
    lib.pt_render.argtypes = [P, C.POINTER(PtRenderDesc), P]
    lib.pt_render_device.argtypes = [P, C.POINTER(PtRenderDesc), P]
    lib.pt_render_device_noalloc.argtypes = [P, C.POINTER(PtRenderDesc), P, P]
    lib.pt_render_stats_get.argtypes = [P, C.POINTER(PtRenderStats)]
    lib.pt_image_save.argtypes = [C.c_char_p, P, C.c_int32, C.c_int32]
    lib.pt_last_error.restype = C.c_char_p
    lib.pt_last_error.argtypes = []
    lib.pt_debug_ref_topology.argtypes = [P, C.c_int32, P, P, P, C.c_int32, P]
    lib.pt_debug_ref_topology_device.argtypes = [P, C.c_int32, P, P, P, C.c_int32, P, P]
    lib.pt_debug_wide_bvh.argtypes = [P, C.c_int32, C.c_int32, C.c_int32, C.c_int32, P, C.c_int32, P, P, P, P]
    lib.pt_debug_image_load.argtypes = [C.c_char_p, C.c_int32, C.c_int32, P, P, P, C.c_int64]
    lib.pt_nn_get_weights.argtypes = [P, P]
    lib.pt_nn_set_weights.argtypes = [P, P]
    lib.pt_nn_reset.argtypes = [P, C.c_uint32]
    lib.pt_nn_stats.argtypes = [P, P, P, P]
    lib.pt_debug_nn_forward.argtypes = [P, P, P, P, C.c_int32, P]
    lib.pt_debug_bsdf.argtypes = [C.c_int32, P, P]
    lib.pt_debug_traversal_limits.argtypes = [P, C.c_int32, C.c_int32]
    lib.pt_debug_tensor_wait_timeout.argtypes = []
    lib.pt_debug_light_sample.argtypes = [P, C.c_int32, P, P]
    lib.pt_debug_nn_grad.argtypes = [P, P, P, P, C.c_int32, P, P]
    lib.pt_debug_nn_grad_ex.argtypes = [P, P, P, P, C.c_int32, C.c_int32, C.c_float, C.c_float, C.c_int32, P, P]
    lib.pt_debug_nn_forward_ex.argtypes = [P, P, P, P, C.c_int32, C.c_int32, P]
    lib.pt_nn_configure.argtypes = [P, P]
    lib.pt_nn_config_get.argtypes = [P, P]
    lib.pt_set_mesh_cache.argtypes = [C.c_int32]
    lib.pt_set_mesh_cache.restype = None
    lib.pt_batch_create.argtypes = [P, C.c_int32, C.POINTER(P)]
    lib.pt_batch_destroy.argtypes = [P]
    lib.pt_batch_destroy.restype = None
    lib.pt_batch_render.argtypes = [P, P, C.c_int32, P]
    lib.pt_batch_render_device.argtypes = [P, P, C.c_int32, P]
    lib.pt_batch_render_ex.argtypes = [P, P, C.c_int32, C.c_int32, C.c_uint32, P]
    lib.pt_batch_render_ex_device.argtypes = [P, P, C.c_int32, C.c_int32, C.c_uint32, P]
    lib.pt_batch_set_tuning.argtypes = [P, P]
    lib.pt_batch_get_tuning.argtypes = [P, P]
    lib.pt_batch_stats.argtypes = [P, C.POINTER(PtRenderStats)]
    lib.pt_batch_autotune.argtypes = [P, P, C.c_int32, C.c_int32, P, P]
    lib.pt_debug_sdtree_run.argtypes = [P, P, C.c_int32, P, P, C.c_int32, P, P, P, P, C.c_int32, P, P, P]
    for name in EXPORTS:
        getattr(lib, name).restype = C.c_int32 if name not in ("pt_scene_destroy", "pt_last_error",
                                                               "pt_batch_destroy", "pt_set_mesh_cache") else \
            getattr(lib, name).restype
    _lib = lib
    return lib


def _check(status: int):
    if status != PT_OK:
        raise PtError(status, _lib.pt_last_error().decode())


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class GpuScene:
    """A scene on the GPU (pt_scene)."""

    def __init__(self, sc=None, settings_file: str | None = None):
        lib = load()
        self.h = C.c_void_p()
        self.render_settings = None
        self.output_name = None
        if settings_file is not None:
            rs = PtRenderDesc()
            out = C.create_string_buffer(4096)
            _check(lib.pt_scene_load(settings_file.encode(), C.byref(self.h), C.byref(rs), out, 4096))
            self.render_settings = rs
            self.output_name = out.value.decode()
            self.width, self.height, self.n_triangles, self.n_lights = self.info()
            return
        self.sc = sc
        self._keep = [np.ascontiguousarray(sc.vertices, np.float32), np.ascontiguousarray(sc.normals, np.float32),
                      np.ascontiguousarray(sc.tangents, np.float32), np.ascontiguousarray(sc.triangles, np.int32),
                      np.ascontiguousarray(sc.tri_material, np.int32)]
        mats = (PtMaterial * max(1, len(sc.mat_kind)))()
        for i, (k, p) in enumerate(zip(sc.mat_kind, sc.mat_params)):
            mats[i].kind = int(k)
            mats[i].rgb[:] = [float(p[0]), float(p[1]), float(p[2])]
            mats[i].roughness, mats[i].ior, mats[i].intensity = float(p[3]), float(p[4]), float(p[5])
        self._mats = mats
        d = PtSceneDesc()
        d.n_vertices = len(sc.vertices)
        d.vertices, d.normals, d.tangents = _ptr(self._keep[0]), _ptr(self._keep[1]), _ptr(self._keep[2])
        d.n_triangles = sc.n_triangles
        d.triangles, d.tri_material = _ptr(self._keep[3]), _ptr(self._keep[4])
        d.n_materials = len(sc.mat_kind)
        d.materials = C.cast(mats, C.c_void_p)
        cam = sc.camera
        d.camera.origin[:] = [float(x) for x in cam[0:3]]
        d.camera.at[:] = [float(x) for x in cam[3:6]]
        d.camera.up[:] = [float(x) for x in cam[6:9]]
        d.camera.tan_fovy = float(cam[9])
        d.camera.width, d.camera.height = sc.width, sc.height
        _check(lib.pt_scene_create(C.byref(d), C.byref(self.h)))
        self._keep = None  # the library has its own copies
        self.width, self.height = sc.width, sc.height
        self.n_triangles, self.n_lights = sc.n_triangles, None

    def close(self):
        if self.h:
            _lib.pt_scene_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def info(self):
        v = [C.c_int32() for _ in range(4)]
        _check(_lib.pt_scene_info(self.h, *[C.byref(x) for x in v]))
        return tuple(x.value for x in v)

    # --- ray batches (host buffers) ---
    def trace_closest(self, rays: np.ndarray):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 7)
        hits = np.zeros((len(rays), 4), np.float32)
        _check(_lib.pt_trace_closest(self.h, _ptr(rays), len(rays), _ptr(hits)))
        return hits[:, 1].view(np.int32).copy(), hits[:, 0].copy(), hits[:, 2].copy(), hits[:, 3].copy()

    def trace_any(self, rays: np.ndarray):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 7)
        occ = np.zeros(len(rays), np.uint8)
        _check(_lib.pt_trace_any(self.h, _ptr(rays), len(rays), _ptr(occ)))
        return occ

    # --- ray batches (device pointers, e.g. torch tensors) ---
    def trace_closest_device(self, d_rays: int, n: int, d_hits: int, stream: int = 0):
        _check(_lib.pt_trace_closest_device(self.h, d_rays, n, d_hits, stream or None))

    def trace_any_device(self, d_rays: int, n: int, d_occ: int, stream: int = 0):
        _check(_lib.pt_trace_any_device(self.h, d_rays, n, d_occ, stream or None))

    # --- rendering ---
    @staticmethod
    def desc(spp: int, max_depth: int = 32, rr_start: int = 3, seed: int = 0, mode: int = MODE_MIS,
             flags: int = 0) -> PtRenderDesc:
        d = PtRenderDesc()
        d.spp, d.max_depth, d.rr_start, d.seed, d.mode, d.flags = spp, max_depth, rr_start, seed, mode, flags
        return d

    def render(self, spp: int, max_depth: int = 32, rr_start: int = 3, seed: int = 0, mode: int = MODE_MIS,
               flags: int = 0, out: np.ndarray | None = None) -> np.ndarray:
        d = self.desc(spp, max_depth, rr_start, seed, mode, flags)
        if out is None:
            out = np.zeros((self.height, self.width, 3), np.float32)
        _check(_lib.pt_render(self.h, C.byref(d), _ptr(out)))
        return out

    def render_device(self, d_out: int, spp: int, max_depth: int = 32, rr_start: int = 3, seed: int = 0,
                      mode: int = MODE_MIS, flags: int = 0):
        d = self.desc(spp, max_depth, rr_start, seed, mode, flags)
        _check(_lib.pt_render_device(self.h, C.byref(d), d_out))

    # --- learned guide ---
    def nn_weights(self) -> np.ndarray:
        w = np.zeros(NN_WEIGHTS, np.float32)
        _check(_lib.pt_nn_get_weights(self.h, _ptr(w)))
        return w

    def nn_set_weights(self, w: np.ndarray):
        w = np.ascontiguousarray(w, np.float32)
        _check(_lib.pt_nn_set_weights(self.h, _ptr(w)))

    def nn_reset(self, seed: int = 12345):
        _check(_lib.pt_nn_reset(self.h, seed))

    def nn_configure(self, **kw):
        """Updates the learned guide's settings (learning_rate, bsdf_frac_min,
        bsdf_frac_max, batch, divergence: NN_KL / NN_CHI2, steps_per_round
        (batches per round), encoding: NN_ENC_FREQ / NN_ENC_ONEBLOB, passes:
        Adam steps per batch);
        returns the new settings."""
        c = PtNNConfig()
        _check(_lib.pt_nn_config_get(self.h, C.byref(c)))
        for k, v in kw.items():
            if k not in dict(PtNNConfig._fields_):
                raise KeyError(k)
            setattr(c, k, v)
        _check(_lib.pt_nn_configure(self.h, C.byref(c)))
        return self.nn_config()

    def nn_config(self) -> dict:
        c = PtNNConfig()
        _check(_lib.pt_nn_config_get(self.h, C.byref(c)))
        return {k: getattr(c, k) for k, _ in PtNNConfig._fields_}

    def nn_stats(self) -> dict:
        v = [C.c_double() for _ in range(3)]
        _check(_lib.pt_nn_stats(self.h, *[C.byref(x) for x in v]))
        return {"steps": v[0].value, "last_loss": v[1].value, "records": v[2].value}

    def stats(self) -> dict:
        s = PtRenderStats()
        _check(_lib.pt_render_stats_get(self.h, C.byref(s)))
        return {n: getattr(s, n) for n, _ in PtRenderStats._fields_}


class GpuBatch:
    """Several GpuScenes merged for batched rendering (pt_batch).  jobs:
    sequence of dicts with scene, spp, and optionally max_depth (32),
    rr_start (3), seed (0)."""

    def __init__(self, scenes):
        lib = load()
        self.scenes = list(scenes)  # keeps the members alive
        arr = (C.c_void_p * len(self.scenes))(*[s.h.value for s in self.scenes])
        self.h = C.c_void_p()
        _check(lib.pt_batch_create(arr, len(self.scenes), C.byref(self.h)))

    def close(self):
        if getattr(self, "h", None) and self.h.value:
            _lib.pt_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _jobs(jobs):
        arr = (PtBatchJob * len(jobs))()
        for a, j in zip(arr, jobs):
            a.scene, a.spp = j["scene"], j["spp"]
            a.max_depth, a.rr_start, a.seed = j.get("max_depth", 32), j.get("rr_start", 3), j.get("seed", 0)
        return arr

    def render(self, jobs, outputs=True, mode=MODE_MIS, flags=0):
        """Renders the jobs; returns one (H, W, 3) image per job (or None).
        mode / flags as GpuScene.render (not MODE_SDTREE); MODE_NN guides
        each job with its scene's own learned guide."""
        arr = self._jobs(jobs)
        if not all(0 <= j["scene"] < len(self.scenes) for j in jobs):
            outputs = False  # the library reports the bad job
        if not outputs:
            _check(_lib.pt_batch_render_ex(self.h, arr, len(jobs), mode, flags, None))
            return None
        imgs = [np.zeros((self.scenes[j["scene"]].height, self.scenes[j["scene"]].width, 3), np.float32)
                for j in jobs]
        ptrs = (C.c_void_p * len(jobs))(*[_ptr(x) for x in imgs])
        _check(_lib.pt_batch_render_ex(self.h, arr, len(jobs), mode, flags, ptrs))
        return imgs

    def render_device(self, jobs, d_outs, mode=MODE_MIS, flags=0):
        arr = self._jobs(jobs)
        ptrs = (C.c_void_p * len(jobs))(*d_outs)
        _check(_lib.pt_batch_render_ex_device(self.h, arr, len(jobs), mode, flags, ptrs))

    def tuning(self) -> dict:
        t = PtBatchTuning()
        _check(_lib.pt_batch_get_tuning(self.h, C.byref(t)))
        return {k: getattr(t, k) for k, _ in PtBatchTuning._fields_}

    def set_tuning(self, **kw):
        t = PtBatchTuning()
        _check(_lib.pt_batch_get_tuning(self.h, C.byref(t)))
        for k, v in kw.items():
            if k not in dict(PtBatchTuning._fields_):
                raise KeyError(k)
            setattr(t, k, v)
        _check(_lib.pt_batch_set_tuning(self.h, C.byref(t)))
        return self.tuning()

    def autotune(self, jobs, spp_divisor: int = 16):
        arr = self._jobs(jobs)
        t = PtBatchTuning()
        rate = C.c_double()
        _check(_lib.pt_batch_autotune(self.h, arr, len(jobs), spp_divisor, C.byref(t), C.byref(rate)))
        return {k: getattr(t, k) for k, _ in PtBatchTuning._fields_}, rate.value

    def stats(self) -> dict:
        s = PtRenderStats()
        _check(_lib.pt_batch_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in PtRenderStats._fields_}


def save_image(prefix: str, rgb: np.ndarray):
    load()
    rgb = np.ascontiguousarray(rgb, np.float32)
    _check(_lib.pt_image_save(prefix.encode(), _ptr(rgb), rgb.shape[1], rgb.shape[0]))


def image_load(path: str, rgb: bool = True, srgb: bool = True) -> np.ndarray:
    """A texture file's pixels as the library decodes them (host only):
    (H, W, 3) for rgb, (H, W) otherwise."""
    lib = load()
    w, h = C.c_int32(), C.c_int32()
    _check(lib.pt_debug_image_load(path.encode(), int(rgb), int(srgb), C.byref(w), C.byref(h), None, 0))
    out = np.zeros((h.value, w.value, 3) if rgb else (h.value, w.value), np.float32)
    _check(lib.pt_debug_image_load(path.encode(), int(rgb), int(srgb), C.byref(w), C.byref(h), _ptr(out), out.size))
    return out


def ref_topology(sc):
    """The reference BVH topology derived by the library (host only)."""
    lib = load()
    tv = np.ascontiguousarray(sc.vertices[sc.triangles].reshape(-1), np.float32)
    n = sc.n_triangles
    cap = max(2 * n, 16)
    order = np.zeros(n, np.int32)
    pparent = np.zeros(n, np.int32)
    boxes = np.zeros(6 * cap, np.float32)
    nn = C.c_int32()
    _check(lib.pt_debug_ref_topology(_ptr(tv), n, _ptr(order), _ptr(pparent), _ptr(boxes), cap, C.byref(nn)))
    return order, boxes[:6 * nn.value].reshape(-1, 6), pparent


def ref_topology_device(sc):
    """The same topology built on the GPU: (leaf order, node boxes, prim parents, levels)."""
    lib = load()
    tv = np.ascontiguousarray(sc.vertices[sc.triangles].reshape(-1), np.float32)
    n = sc.n_triangles
    cap = max(2 * n, 16)
    order = np.zeros(n, np.int32)
    pparent = np.zeros(n, np.int32)
    boxes = np.zeros(6 * cap, np.float32)
    nn, lv = C.c_int32(), C.c_int32()
    _check(lib.pt_debug_ref_topology_device(_ptr(tv), n, _ptr(order), _ptr(pparent), _ptr(boxes), cap, C.byref(nn),
                                            C.byref(lv)))
    return order, boxes[:6 * nn.value].reshape(-1, 6), pparent, lv.value


def wide_bvh(sc, on_device=True, host_threads=0, max_leaf=4):
    """The 4-wide traversal tree the library builds for a scene's triangles:
    (nodes (m, 16) uint32, leaf order, depth, inflation), built on the GPU
    (as scenes are) or on the host with host_threads threads."""
    lib = load()
    tv = np.ascontiguousarray(sc.vertices[sc.triangles].reshape(-1), np.float32)
    n = sc.n_triangles
    cap = max(n, 16)
    nodes = np.zeros((cap, 16), np.uint32)
    order = np.zeros(max(n, 1), np.int32)
    nn, depth, infl = C.c_int32(), C.c_int32(), C.c_float()
    _check(lib.pt_debug_wide_bvh(_ptr(tv), n, int(max_leaf), int(bool(on_device)), int(host_threads), _ptr(nodes),
                                 cap, C.byref(nn), _ptr(order), C.byref(depth), C.byref(infl)))
    return nodes[:nn.value], order[:n], depth.value, infl.value


def sdtree_run(lo, hi, rounds, queries, max_leaves=1 << 20, fn=None, lib=None):
    """Runs an SD-tree through rounds of splats + update (host only).
    rounds: list of (n,7) arrays {radiance, pos, dir}.  Returns dict with the
    sampling leaves, per-spatial-leaf leaf counts, splat counts, flux and the
    pdf of each query (n,6).  `fn` selects another implementation with the
    same signature (e.g. the reference harness)."""
    L = lib or load()
    f = fn or L.pt_debug_sdtree_run
    lo = np.ascontiguousarray(lo, np.float32)
    hi = np.ascontiguousarray(hi, np.float32)
    ns = np.array([len(r) for r in rounds], np.int32)
    sp = np.ascontiguousarray(np.concatenate(rounds) if rounds else np.zeros((0, 7)), np.float32)
    q = np.ascontiguousarray(queries, np.float32)
    leaves = np.zeros(4 * max_leaves, np.float32)
    cap = 1 << 16
    lc = np.zeros(cap, np.int32)
    cnt = np.zeros(cap, np.int32)
    flux = np.zeros(cap, np.float32)
    pdf = np.zeros(len(q), np.float32)
    nsp = C.c_int32()
    r = f(_ptr(lo), _ptr(hi), len(rounds), _ptr(ns), _ptr(sp), max_leaves, _ptr(leaves), _ptr(lc), _ptr(cnt),
          _ptr(flux), len(q), _ptr(q), _ptr(pdf), C.byref(nsp))
    if fn is None:
        _check(r)
        n = nsp.value
    else:
        n = r
    total = int(lc[:n].sum())
    return {"leaves": leaves[:4 * total].reshape(-1, 4), "leaf_counts": lc[:n], "counts": cnt[:n],
            "flux": flux[:n], "pdf": pdf}


def debug_bsdf(cases: np.ndarray) -> np.ndarray:
    """The integrator's BxDF eval / pdf / sample on the device (pt_debug_bsdf):
    cases n x 20 -> n x 10 (see the header)."""
    L = load()
    c = np.ascontiguousarray(cases, np.float32).reshape(-1, 20)
    out = np.zeros((len(c), 10), np.float32)
    _check(L.pt_debug_bsdf(len(c), _ptr(c), _ptr(out)))
    return out


def debug_light_sample(scene: "GpuScene", cases: np.ndarray) -> np.ndarray:
    """The integrator's light sampling on the device (pt_debug_light_sample):
    cases n x 6 (point, u0, u1, u2) -> n x 10 (position, normal, Le |cos|, pdf)."""
    L = load()
    c = np.ascontiguousarray(cases, np.float32).reshape(-1, 6)
    out = np.zeros((len(c), 10), np.float32)
    _check(L.pt_debug_light_sample(scene.h, len(c), _ptr(c), _ptr(out)))
    return out


def nn_forward(weights, lo, hi, inputs, encoding=NN_ENC_FREQ):
    """Debug forward pass of the learned guide on the GPU: (n,9) -> (n,41)."""
    L = load()
    w = np.ascontiguousarray(weights, np.float32)
    x = np.ascontiguousarray(inputs, np.float32)
    out = np.zeros((len(x), 41), np.float32)
    lo = np.ascontiguousarray(lo, np.float32)
    hi = np.ascontiguousarray(hi, np.float32)
    _check(L.pt_debug_nn_forward_ex(_ptr(w), _ptr(lo), _ptr(hi), _ptr(x), len(x), int(encoding), _ptr(out)))
    return out


def nn_grad(weights, lo, hi, records):
    """Debug gradient of the training loss on the GPU: returns (loss, dL/dW)."""
    L = load()
    w = np.ascontiguousarray(weights, np.float32)
    r = np.ascontiguousarray(records, np.float32)
    g = np.zeros(NN_WEIGHTS, np.float32)
    loss = C.c_float()
    lo = np.ascontiguousarray(lo, np.float32)
    hi = np.ascontiguousarray(hi, np.float32)
    _check(L.pt_debug_nn_grad(_ptr(w), _ptr(lo), _ptr(hi), _ptr(r), len(r), _ptr(g), C.byref(loss)))
    return loss.value, g


def nn_grad_step(weights, lo, hi, records, divergence=NN_CHI2, c_lo=0.3, c_hi=0.9, encoding=NN_ENC_FREQ):
    """The renderer's training-step gradient on the GPU (device T sum, KL or
    chi-square weights, BSDF fraction in [c_lo, c_hi]): (loss, dL/dW)."""
    L = load()
    w = np.ascontiguousarray(weights, np.float32)
    r = np.ascontiguousarray(records, np.float32)
    g = np.zeros(NN_WEIGHTS, np.float32)
    loss = C.c_float()
    lo = np.ascontiguousarray(lo, np.float32)
    hi = np.ascontiguousarray(hi, np.float32)
    _check(L.pt_debug_nn_grad_ex(_ptr(w), _ptr(lo), _ptr(hi), _ptr(r), len(r), int(divergence), float(c_lo),
                                 float(c_hi), int(encoding), _ptr(g), C.byref(loss)))
    return loss.value, g
