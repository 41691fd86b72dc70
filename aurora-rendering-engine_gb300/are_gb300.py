"""Python binding of the GB300 path-tracing core (ctypes over include/aurora_gb300.h).

The core itself is C++/CUDA in ``libaurora_gb300.so``; this module only
mirrors the C structs, marshals numpy arrays and turns status codes into
exceptions.  There is no Python or CPU fallback: if the shared library is
missing, ``load()`` raises.

Reference interface mirrored: the scene is what rt.cpp's ``Scene`` holds
(experiments/rt.cpp:146-186) or an ``are::ObjectSet`` of primitives with
material and texture objects (include/object/object_set.h:10-12), and
``Renderer.render`` is rt.cpp's ``render(scene, camPos, camTarget, camUp,
fov, vp)`` (rt.cpp:337-374) with spp, depth and seed made explicit.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "libaurora_gb300.so"

MAT_LAMBERTIAN, MAT_METAL, MAT_DIELECTRIC, MAT_DIFFUSE_LIGHT = 0, 1, 2, 3
TEX_SOLID, TEX_CHECKER, TEX_IMAGE = 0, 1, 2
FILTER_NEAREST, FILTER_BILINEAR = 0, 1
MAP_SURFACE_UV, MAP_SPHERICAL = 0, 1
BG_CONSTANT, BG_SKY_GRADIENT = 0, 1
TRI_REFERENCE_MT, TRI_WATERTIGHT = 0, 1
BVH_HOST_SAH, BVH_DEVICE = 0, 1
ACCEL_AUTO, ACCEL_BVH = 0, 1
EST_PATH, EST_LEGACY_RT, EST_GUIDED = 0, 1, 2
FLAG_DEVICE_OUTPUT, FLAG_NO_JITTER, FLAG_CLAMP_OUTPUT, FLAG_LEGACY_MT19937 = 1, 2, 4, 8
CONFIG_RANDOM_SPHERES, CONFIG_CORNELL, CONFIG_MESH, CONFIG_CORNELL_OCCLUDED, CONFIG_LEGACY_RT = 0, 1, 2, 4, 5
CONFIG_SPHERE_FIELD = 6
SCHEDULE_AUTO, SCHEDULE_WAVEFRONT, SCHEDULE_MEGAKERNEL = 0, 1, 2
TONEMAP_GAMMA, TONEMAP_LINEAR = 0, 1

MATERIAL_DTYPE = np.dtype([("type", "<i4"), ("texture", "<i4"), ("fuzz", "<f4"), ("ior", "<f4"),
                           ("emit", "<f4", 3), ("reflect_ratio", "<f4"), ("tint", "<f4", 3), ("pad_", "<f4")])
TEXTURE_DTYPE = np.dtype([("type", "<i4"), ("mapping", "<i4"), ("scale", "<f4"), ("width", "<i4"),
                          ("height", "<i4"), ("texel_offset", "<i4"), ("a", "<f4", 3), ("b", "<f4", 3),
                          ("center", "<f4", 3), ("filter", "<i4")])
assert MATERIAL_DTYPE.itemsize == 48 and TEXTURE_DTYPE.itemsize == 64

STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "out of memory", 4: "no device",
          5: "kernel timeout", 6: "internal error", 7: "file error"}


class AreError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


# ---------------------------------------------------------------------------
# scene container (numpy), shared by the core and the oracle tests


@dataclass
class SceneArrays:
    spheres: np.ndarray = field(default_factory=lambda: np.zeros((0, 4), np.float32))
    sphere_mat: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    quads: np.ndarray = field(default_factory=lambda: np.zeros((0, 9), np.float32))
    quad_mat: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    triangles: np.ndarray = field(default_factory=lambda: np.zeros((0, 9), np.float32))
    triangle_uv: np.ndarray | None = None
    triangle_mat: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    materials: np.ndarray = field(default_factory=lambda: np.zeros(0, MATERIAL_DTYPE))
    textures: np.ndarray = field(default_factory=lambda: np.zeros(0, TEXTURE_DTYPE))
    texels: np.ndarray | None = None
    background: int = BG_CONSTANT
    bg_a: tuple = (0.0, 0.0, 0.0)
    bg_b: tuple = (0.0, 0.0, 0.0)
    triangle_test: int = TRI_WATERTIGHT
    bvh_leaf_size: int = 0
    bvh_build: int = 0
    bvh_width: int = 0
    accel: int = 0

    @property
    def n_prims(self) -> int:
        return len(self.sphere_mat) + len(self.quad_mat) + len(self.triangle_mat)

    # builders -------------------------------------------------------------
    def texture(self, type=TEX_SOLID, a=(0, 0, 0), b=(0, 0, 0), scale=1.0, mapping=MAP_SURFACE_UV,
                center=(0, 0, 0), width=0, height=0, texel_offset=0, filter=FILTER_NEAREST) -> int:
        t = np.zeros(1, TEXTURE_DTYPE)
        t["type"], t["mapping"], t["scale"], t["filter"] = type, mapping, scale, filter
        t["width"], t["height"], t["texel_offset"] = width, height, texel_offset
        t["a"], t["b"], t["center"] = a, b, center
        self.textures = np.concatenate([self.textures, t])
        return len(self.textures) - 1

    def material(self, type=MAT_LAMBERTIAN, texture=-1, fuzz=0.0, ior=1.5, emit=(0, 0, 0), reflect_ratio=0.0,
                 tint=(0, 0, 0), albedo=None) -> int:
        if albedo is not None:
            texture = self.texture(TEX_SOLID, a=albedo)
        m = np.zeros(1, MATERIAL_DTYPE)
        m["type"], m["texture"], m["fuzz"], m["ior"] = type, texture, fuzz, ior
        m["emit"], m["reflect_ratio"], m["tint"] = emit, reflect_ratio, tint
        self.materials = np.concatenate([self.materials, m])
        return len(self.materials) - 1

    def add_spheres(self, s, mat) -> None:
        s = np.asarray(s, np.float32).reshape(-1, 4)
        self.spheres = np.concatenate([self.spheres, s])
        self.sphere_mat = np.concatenate([self.sphere_mat, np.broadcast_to(np.asarray(mat, np.int32), len(s))])

    def add_quads(self, q, mat) -> None:
        q = np.asarray(q, np.float32).reshape(-1, 9)
        self.quads = np.concatenate([self.quads, q])
        self.quad_mat = np.concatenate([self.quad_mat, np.broadcast_to(np.asarray(mat, np.int32), len(q))])

    def add_triangles(self, t, mat, uv=None) -> None:
        t = np.asarray(t, np.float32).reshape(-1, 9)
        n0 = len(self.triangle_mat)
        self.triangles = np.concatenate([self.triangles, t])
        self.triangle_mat = np.concatenate([self.triangle_mat, np.broadcast_to(np.asarray(mat, np.int32), len(t))])
        if uv is not None or self.triangle_uv is not None:
            old = self.triangle_uv if self.triangle_uv is not None else np.zeros((n0, 6), np.float32)
            new = np.zeros((len(t), 6), np.float32) if uv is None else np.asarray(uv, np.float32).reshape(-1, 6)
            self.triangle_uv = np.concatenate([old, new])


# ---------------------------------------------------------------------------
# C structs

_f = C.POINTER(C.c_float)
_i32 = C.POINTER(C.c_int32)


class SceneDesc(C.Structure):
    _fields_ = [
        ("n_spheres", C.c_int32), ("spheres", _f), ("sphere_mat", _i32),
        ("n_quads", C.c_int32), ("quads", _f), ("quad_mat", _i32),
        ("n_triangles", C.c_int32), ("triangles", _f), ("triangle_uv", _f), ("triangle_mat", _i32),
        ("n_materials", C.c_int32), ("materials", C.c_void_p),
        ("n_textures", C.c_int32), ("textures", C.c_void_p),
        ("n_texels", C.c_int64), ("texels", _f),
        ("background", C.c_int32), ("bg_a", C.c_float * 3), ("bg_b", C.c_float * 3),
        ("triangle_test", C.c_int32), ("bvh_leaf_size", C.c_int32), ("bvh_build", C.c_int32),
        ("bvh_width", C.c_int32), ("accel", C.c_int32)]


class Camera(C.Structure):
    _fields_ = [("lookfrom", C.c_float * 3), ("lookat", C.c_float * 3), ("vup", C.c_float * 3),
                ("vfov_deg", C.c_float), ("aperture", C.c_float), ("focus_dist", C.c_float)]

    def to_dict(self) -> dict:
        return {"lookfrom": list(self.lookfrom), "lookat": list(self.lookat), "vup": list(self.vup),
                "vfov_deg": self.vfov_deg, "aperture": self.aperture, "focus_dist": self.focus_dist}

    @staticmethod
    def from_dict(d: dict) -> "Camera":
        c = Camera()
        c.lookfrom = (C.c_float * 3)(*d["lookfrom"])
        c.lookat = (C.c_float * 3)(*d["lookat"])
        c.vup = (C.c_float * 3)(*d["vup"])
        c.vfov_deg = d["vfov_deg"]
        c.aperture = d.get("aperture", 0.0)
        c.focus_dist = d.get("focus_dist", 1.0)
        return c


class RenderParams(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32), ("max_depth", C.c_int32),
                ("seed", C.c_uint64), ("rr_depth", C.c_int32), ("t_min", C.c_float), ("estimator", C.c_int32),
                ("flags", C.c_int32), ("pool_size", C.c_int32), ("chunk", C.c_int32), ("block_size", C.c_int32),
                ("schedule", C.c_int32)]

    def to_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}

    @staticmethod
    def from_dict(d: dict) -> "RenderParams":
        p = RenderParams()
        for k, _ in RenderParams._fields_:
            if k in d:
                setattr(p, k, d[k])
        return p


KERNELS = ("intersect", "shade", "generate", "other")


class BatchOptions(C.Structure):
    _fields_ = [("block_size", C.c_int32), ("fetch", C.c_int32), ("leaf_size", C.c_int32), ("bvh_width", C.c_int32)]

    def to_dict(self) -> dict:
        return {"block_size": self.block_size, "fetch": self.fetch, "leaf_size": self.leaf_size,
                "bvh_width": self.bvh_width}


class TonemapParams(C.Structure):
    _fields_ = [("mode", C.c_int32), ("gamma", C.c_float), ("flags", C.c_uint32), ("reserved_", C.c_int32)]


class GuideParams(C.Structure):
    _fields_ = [("mix", C.c_float), ("guide_depth", C.c_int32), ("train", C.c_int32), ("batch", C.c_int32),
                ("lr", C.c_float), ("weight_clip", C.c_float), ("cache_res", C.c_int32), ("max_steps", C.c_int32)]

    @staticmethod
    def make(mix=0.5, guide_depth=2, train=1, batch=1 << 18, lr=1e-2, weight_clip=100.0, cache_res=0,
             max_steps=0) -> "GuideParams":
        g = GuideParams()
        g.mix, g.guide_depth, g.train, g.batch, g.lr, g.weight_clip = mix, guide_depth, train, batch, lr, weight_clip
        g.cache_res, g.max_steps = cache_res, max_steps
        return g


class RenderStats(C.Structure):
    _fields_ = [("samples", C.c_int64), ("segments", C.c_int64), ("iterations", C.c_int64),
                ("device_ms", C.c_double), ("kernel_ms", C.c_double * 4), ("kernel_launches", C.c_int64 * 4),
                ("error_word", C.c_int32), ("reserved_", C.c_int32), ("aux", C.c_double * 4)]

    def to_dict(self) -> dict:
        d = {k: getattr(self, k) for k in ("samples", "segments", "iterations", "device_ms", "error_word")}
        d["kernel_ms"] = dict(zip(KERNELS, list(self.kernel_ms)))
        d["kernel_launches"] = dict(zip(KERNELS, list(self.kernel_launches)))
        d["aux"] = list(self.aux)
        return d


def _np_ptr(a, t):
    if a is None or a.size == 0:
        return C.cast(None, t)
    return a.ctypes.data_as(t)


def desc_struct(s: SceneArrays) -> tuple[SceneDesc, list]:
    keep = []

    def arr(x, dt):
        if x is None:
            return None
        y = np.ascontiguousarray(x, dtype=dt)
        keep.append(y)
        return y

    d = SceneDesc()
    sp, spm = arr(s.spheres, np.float32), arr(s.sphere_mat, np.int32)
    qd, qdm = arr(s.quads, np.float32), arr(s.quad_mat, np.int32)
    tr, trm = arr(s.triangles, np.float32), arr(s.triangle_mat, np.int32)
    tru = arr(s.triangle_uv, np.float32)
    mats, texs = arr(s.materials, MATERIAL_DTYPE), arr(s.textures, TEXTURE_DTYPE)
    tx = arr(s.texels, np.float32)
    d.n_spheres, d.spheres, d.sphere_mat = len(spm), _np_ptr(sp, _f), _np_ptr(spm, _i32)
    d.n_quads, d.quads, d.quad_mat = len(qdm), _np_ptr(qd, _f), _np_ptr(qdm, _i32)
    d.n_triangles, d.triangles, d.triangle_mat = len(trm), _np_ptr(tr, _f), _np_ptr(trm, _i32)
    d.triangle_uv = _np_ptr(tru, _f)
    d.n_materials, d.materials = len(mats), (mats.ctypes.data if len(mats) else None)
    d.n_textures, d.textures = len(texs), (texs.ctypes.data if len(texs) else None)
    d.n_texels = 0 if tx is None else tx.size // 3
    d.texels = _np_ptr(tx, _f)
    d.background = int(s.background)
    d.bg_a = (C.c_float * 3)(*[float(v) for v in s.bg_a])
    d.bg_b = (C.c_float * 3)(*[float(v) for v in s.bg_b])
    d.triangle_test = int(s.triangle_test)
    d.bvh_leaf_size = int(s.bvh_leaf_size)
    d.bvh_build = int(s.bvh_build)
    d.bvh_width = int(s.bvh_width)
    d.accel = int(s.accel)
    return d, keep


def _copy(ptr, n, cols, dtype=np.float32):
    if n == 0 or not ptr:
        return np.zeros((0, cols) if cols > 1 else 0, dtype)
    ctype = {np.float32: C.c_float, np.int32: C.c_int32}[dtype]
    a = np.ctypeslib.as_array(C.cast(ptr, C.POINTER(ctype)), shape=(n * cols,)).copy()
    return a.reshape(n, cols) if cols > 1 else a


def arrays_from_desc(d: SceneDesc) -> SceneArrays:
    s = SceneArrays()
    s.spheres, s.sphere_mat = _copy(d.spheres, d.n_spheres, 4), _copy(d.sphere_mat, d.n_spheres, 1, np.int32)
    s.quads, s.quad_mat = _copy(d.quads, d.n_quads, 9), _copy(d.quad_mat, d.n_quads, 1, np.int32)
    s.triangles, s.triangle_mat = _copy(d.triangles, d.n_triangles, 9), _copy(d.triangle_mat, d.n_triangles, 1,
                                                                               np.int32)
    s.triangle_uv = _copy(d.triangle_uv, d.n_triangles, 6) if d.triangle_uv else None
    if d.n_materials:
        buf = (C.c_char * (48 * d.n_materials)).from_address(d.materials)
        s.materials = np.frombuffer(bytes(buf), MATERIAL_DTYPE).copy()
    if d.n_textures:
        buf = (C.c_char * (64 * d.n_textures)).from_address(d.textures)
        s.textures = np.frombuffer(bytes(buf), TEXTURE_DTYPE).copy()
    s.texels = _copy(d.texels, d.n_texels, 3) if d.n_texels else None
    s.background, s.bg_a, s.bg_b = d.background, tuple(d.bg_a), tuple(d.bg_b)
    s.triangle_test, s.bvh_leaf_size, s.bvh_build = d.triangle_test, d.bvh_leaf_size, d.bvh_build
    s.bvh_width = d.bvh_width
    s.accel = d.accel
    return s


# ---------------------------------------------------------------------------
# library

_LIB = None


def exported_symbols() -> list[str]:
    """Entry points declared in include/aurora_gb300.h (ARE_API functions)."""
    import re  # noqa: PLC0415
    hdr = (HERE.parent / "include" / "aurora_gb300.h").read_text()
    return re.findall(r"ARE_API\s+[\w\s\*]+?\b(are_\w+)\s*\(", hdr)


def load(path: str | os.PathLike | None = None):
    """Load libaurora_gb300.so.  Raises if it has not been built: there is no
    fallback implementation."""
    global _LIB
    if _LIB is not None and path is None:
        return _LIB
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(f"{p} is missing: run __graft_entry__.build() to compile the CUDA core")
    L = C.CDLL(str(p))
    L.are_status_string.restype = C.c_char_p
    L.are_status_string.argtypes = [C.c_int]
    L.are_last_error.restype = C.c_char_p
    L.are_version.restype = C.c_int32
    L.are_device_count.restype = C.c_int32
    L.are_trim_memory.argtypes = [C.c_int32]
    L.are_scene_create.argtypes = [C.POINTER(SceneDesc), C.POINTER(C.c_void_p)]
    L.are_scene_destroy.argtypes = [C.c_void_p]
    L.are_scene_info.argtypes = [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                                 C.POINTER(C.c_int32)]
    L.are_render.argtypes = [C.c_void_p, C.POINTER(Camera), C.POINTER(RenderParams), C.c_void_p, C.c_void_p,
                             C.POINTER(RenderStats)]
    L.are_render_noalloc.argtypes = [C.c_void_p, C.POINTER(Camera), C.POINTER(RenderParams), C.c_void_p, C.c_void_p,
                                     C.POINTER(RenderStats)]
    L.are_intersect.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int32, C.POINTER(C.c_float)]
    L.are_config_build.argtypes = [C.c_int32, C.c_uint64, C.c_int32, C.POINTER(C.c_void_p)]
    L.are_config_desc.restype = C.POINTER(SceneDesc)
    L.are_config_desc.argtypes = [C.c_void_p]
    L.are_config_defaults.argtypes = [C.c_void_p, C.POINTER(Camera), C.POINTER(RenderParams)]
    L.are_config_free.argtypes = [C.c_void_p]
    L.are_render_guided.argtypes = [C.c_void_p, C.c_void_p, C.POINTER(Camera), C.POINTER(RenderParams),
                                    C.POINTER(GuideParams), C.c_void_p, C.c_void_p, C.POINTER(RenderStats)]
    L.are_render_batch.argtypes = [C.POINTER(C.c_void_p), C.POINTER(Camera), C.POINTER(RenderParams), C.c_int32,
                                   C.POINTER(BatchOptions), C.POINTER(C.c_void_p), C.POINTER(C.c_double),
                                   C.POINTER(RenderStats)]
    L.are_batch_autotune.argtypes = [C.POINTER(C.POINTER(SceneDesc)), C.POINTER(Camera), C.POINTER(RenderParams),
                                     C.c_int32, C.c_int32, C.POINTER(BatchOptions), C.POINTER(C.c_double)]
    L.are_tonemap.argtypes = [C.c_void_p, C.c_int64, C.POINTER(TonemapParams), C.c_void_p]
    L.are_write_ppm.argtypes = [C.c_char_p, C.c_void_p, C.c_int32, C.c_int32]
    L.are_write_pfm.argtypes = [C.c_char_p, C.c_void_p, C.c_int32, C.c_int32]
    L.are_read_ppm.argtypes = [C.c_char_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_void_p]
    L.are_guide_loss_history.restype = C.c_int32
    L.are_guide_loss_history.argtypes = [C.c_void_p, C.c_void_p, C.c_int32]
    L.are_guide_param_count.restype = C.c_int32
    L.are_guide_create.argtypes = [C.c_uint64, C.POINTER(C.c_void_p)]
    L.are_guide_destroy.argtypes = [C.c_void_p]
    L.are_guide_get_params.argtypes = [C.c_void_p, C.c_void_p]
    L.are_guide_set_params.argtypes = [C.c_void_p, C.c_void_p]
    L.are_guide_forward.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
    L.are_guide_mixture.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]
    L.are_guide_gradient.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(C.c_float), C.c_void_p]
    L.are_guide_train.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_float, C.POINTER(C.c_float)]
    L.are_guide_set_wait_limit.argtypes = [C.c_void_p, C.c_int32]
    for name in exported_symbols():
        fn = getattr(L, name)
        if fn.restype is C.c_int:  # are_status returns
            fn.restype = C.c_int
    if path is None:
        _LIB = L
    return L


def check(status: int) -> None:
    if status != 0:
        L = load()
        raise AreError(status, L.are_last_error().decode(errors="replace"))


# ---------------------------------------------------------------------------
# high-level wrappers


def trim_memory(device: int = -1) -> None:
    """are_trim_memory: return the device memory pool's cached blocks to the driver."""
    check(load().are_trim_memory(device))


def build_config(config: int, seed: int = 42, mesh_frequency: int = 0):
    """Seeded synthetic scene -> (SceneArrays, camera dict, params dict)."""
    L = load()
    h = C.c_void_p()
    check(L.are_config_build(config, seed, mesh_frequency, C.byref(h)))
    try:
        d = L.are_config_desc(h).contents
        arrays = arrays_from_desc(d)
        cam, par = Camera(), RenderParams()
        check(L.are_config_defaults(h, C.byref(cam), C.byref(par)))
        return arrays, cam.to_dict(), par.to_dict()
    finally:
        L.are_config_free(h)


class Scene:
    """A device-resident scene (are_scene_create / are_scene_destroy)."""

    def __init__(self, arrays: SceneArrays):
        self.lib = load()
        d, keep = desc_struct(arrays)
        h = C.c_void_p()
        check(self.lib.are_scene_create(C.byref(d), C.byref(h)))
        self.h = h
        self.arrays = arrays

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.are_scene_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

    def info(self) -> dict:
        n_prims, n_nodes = C.c_int64(), C.c_int64()
        max_leaf, depth = C.c_int32(), C.c_int32()
        check(self.lib.are_scene_info(self.h, C.byref(n_prims), C.byref(n_nodes), C.byref(max_leaf), C.byref(depth)))
        return {"prims": n_prims.value, "nodes": n_nodes.value, "max_leaf": max_leaf.value, "depth": depth.value}

    def intersect(self, rays: np.ndarray) -> tuple[np.ndarray, float]:
        """Closest hit of host rays (n x 8) -> (hits n x 4, kernel ms)."""
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        hits = np.empty((len(rays), 4), np.float32)
        ms = C.c_float()
        check(self.lib.are_intersect(self.h, rays.ctypes.data, len(rays), hits.ctypes.data, 0, C.byref(ms)))
        return hits, ms.value

    def intersect_device(self, rays_ptr: int, n: int, hits_ptr: int) -> float:
        ms = C.c_float()
        check(self.lib.are_intersect(self.h, rays_ptr, n, hits_ptr, 1, C.byref(ms)))
        return ms.value

    def render(self, cam: dict, params: dict, with_var: bool = True) -> tuple[np.ndarray, np.ndarray | None, dict]:
        p = RenderParams.from_dict(params)
        p.flags = int(p.flags) & ~FLAG_DEVICE_OUTPUT
        c = Camera.from_dict(cam)
        n = p.width * p.height * 3
        rgb = np.empty(n, np.float32)
        var = np.empty(n, np.float32) if with_var else None
        st = RenderStats()
        check(self.lib.are_render(self.h, C.byref(c), C.byref(p), rgb.ctypes.data,
                                  var.ctypes.data if var is not None else None, C.byref(st)))
        shape = (p.height, p.width, 3)
        return rgb.reshape(shape), (var.reshape(shape) if var is not None else None), st.to_dict()

    def render_guided(self, guide: "Guide", cam: dict, params: dict, gparams: "GuideParams | None" = None,
                      with_var: bool = True):
        """are_render_guided with host buffers -> (rgb, var, stats incl. 'train_steps')."""
        p = RenderParams.from_dict(params)
        p.flags = int(p.flags) & ~FLAG_DEVICE_OUTPUT
        c = Camera.from_dict(cam)
        g = gparams or GuideParams.make()
        n = p.width * p.height * 3
        rgb = np.empty(n, np.float32)
        var = np.empty(n, np.float32) if with_var else None
        st = RenderStats()
        check(self.lib.are_render_guided(self.h, guide.h, C.byref(c), C.byref(p), C.byref(g), rgb.ctypes.data,
                                         var.ctypes.data if var is not None else None, C.byref(st)))
        d = st.to_dict()
        d["train_steps"] = int(st.aux[1])
        d["train_samples"] = int(st.aux[0])
        d["guided_vertices"] = int(st.aux[2])
        d["last_loss"] = st.aux[3]
        shape = (p.height, p.width, 3)
        return rgb.reshape(shape), (var.reshape(shape) if var is not None else None), d

    def render_device(self, cam: dict, params: dict, rgb_ptr: int, var_ptr: int | None = None) -> dict:
        p = RenderParams.from_dict(params)
        p.flags = int(p.flags) | FLAG_DEVICE_OUTPUT
        c = Camera.from_dict(cam)
        st = RenderStats()
        check(self.lib.are_render(self.h, C.byref(c), C.byref(p), rgb_ptr, var_ptr, C.byref(st)))
        return st.to_dict()


class Guide:
    """The path-guiding network (are_guide_*): FP16 tensor-core MLP, FP32 master weights."""

    def __init__(self, seed: int = 1):
        self.lib = load()
        h = C.c_void_p()
        check(self.lib.are_guide_create(seed, C.byref(h)))
        self.h = h
        self.n_params = self.lib.are_guide_param_count()

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            self.lib.are_guide_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

    @property
    def params(self) -> np.ndarray:
        p = np.empty(self.n_params, np.float32)
        check(self.lib.are_guide_get_params(self.h, p.ctypes.data))
        return p

    @params.setter
    def params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.n_params
        check(self.lib.are_guide_set_params(self.h, p.ctypes.data))

    def forward(self, feat: np.ndarray) -> np.ndarray:
        feat = np.ascontiguousarray(feat, np.float32).reshape(-1, 9)
        out = np.empty((len(feat), 48), np.float32)
        check(self.lib.are_guide_forward(self.h, feat.ctypes.data, len(feat), out.ctypes.data))
        return out

    def mixture(self, feat: np.ndarray) -> np.ndarray:
        """are_guide_mixture: the packed vMF mixture per row (n x 48)."""
        feat = np.ascontiguousarray(feat, np.float32).reshape(-1, 9)
        out = np.empty((len(feat), 48), np.float32)
        check(self.lib.are_guide_mixture(self.h, feat.ctypes.data, len(feat), out.ctypes.data))
        return out

    def gradient(self, samples: np.ndarray):
        samples = np.ascontiguousarray(samples, np.float32).reshape(-1, 13)
        g = np.empty(self.n_params, np.float32)
        loss = C.c_float()
        check(self.lib.are_guide_gradient(self.h, samples.ctypes.data, len(samples), C.byref(loss), g.ctypes.data))
        return loss.value, g

    def loss_history(self) -> list:
        out = np.zeros(4096, np.float32)
        n = self.lib.are_guide_loss_history(self.h, out.ctypes.data, len(out))
        return list(out[:n])

    def set_wait_limit(self, polls: int) -> None:
        """are_guide_set_wait_limit: polls for the first tensor-core wait of each warpgroup (-1 = default)."""
        check(self.lib.are_guide_set_wait_limit(self.h, int(polls)))

    def train(self, samples: np.ndarray, lr: float = 1e-2) -> float:
        samples = np.ascontiguousarray(samples, np.float32).reshape(-1, 13)
        loss = C.c_float()
        check(self.lib.are_guide_train(self.h, samples.ctypes.data, len(samples), lr, C.byref(loss)))
        return loss.value


def render_batch(scenes: list, cams: list, params: list, options: "BatchOptions | None" = None, want_images=True):
    """are_render_batch: many scenes in one persistent launch.
    Returns (images or None, per-scene completion ms, stats)."""
    L = load()
    n = len(scenes)
    hs = (C.c_void_p * n)(*[sc.h.value for sc in scenes])
    cs = (Camera * n)(*[Camera.from_dict(c) for c in cams])
    ps = (RenderParams * n)(*[RenderParams.from_dict(p) for p in params])
    imgs = [np.empty(p["width"] * p["height"] * 3, np.float32) for p in params] if want_images else None
    outs = (C.c_void_p * n)(*[im.ctypes.data for im in imgs]) if want_images else None
    ms = (C.c_double * n)()
    st = RenderStats()
    check(L.are_render_batch(hs, cs, ps, n, C.byref(options) if options else None, outs, ms, C.byref(st)))
    if imgs is not None:
        imgs = [im.reshape(p["height"], p["width"], 3) for im, p in zip(imgs, params)]
    return imgs, list(ms), st.to_dict()


def batch_autotune(arrays: list, cams: list, params: list, calib_spp: int = 2):
    """are_batch_autotune over leaf size x block size x fetch -> (BatchOptions, ms)."""
    L = load()
    n = len(arrays)
    descs = [desc_struct(a) for a in arrays]
    dp = (C.POINTER(SceneDesc) * n)(*[C.pointer(d) for d, _ in descs])
    cs = (Camera * n)(*[Camera.from_dict(c) for c in cams])
    ps = (RenderParams * n)(*[RenderParams.from_dict(p) for p in params])
    best = BatchOptions()
    ms = C.c_double()
    check(L.are_batch_autotune(dp, cs, ps, n, calib_spp, C.byref(best), C.byref(ms)))
    return best, ms.value


def batch_workload(n_scenes: int = 64, seed: int = 2026, min_count: int = 50, max_count: int = 200_000):
    """The uneven batch: sphere counts log-uniform in [min_count, max_count],
    resolution and spp drawn per scene by the scene generator."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for i in range(n_scenes):
        cnt = int(np.exp(rng.uniform(np.log(min_count), np.log(max_count))))
        out.append(build_config(CONFIG_SPHERE_FIELD, seed=seed * 1000 + i, mesh_frequency=cnt))
    return out


# ---------------------------------------------------------------------------
# output formats


def tonemap(rgb: np.ndarray, mode: int = TONEMAP_GAMMA, gamma: float = 2.2) -> np.ndarray:
    """are_tonemap of a host float32 image (any shape) -> uint8 of the same shape."""
    L = load()
    a = np.ascontiguousarray(rgb, np.float32)
    out = np.empty(a.shape, np.uint8)
    check(L.are_tonemap(a.ctypes.data, a.size, C.byref(TonemapParams(mode, gamma, 0, 0)), out.ctypes.data))
    return out


def tonemap_device(rgb_ptr: int, n_values: int, out_ptr: int, mode: int = TONEMAP_GAMMA, gamma: float = 2.2) -> None:
    """are_tonemap on device pointers of the current device."""
    L = load()
    check(L.are_tonemap(rgb_ptr, n_values, C.byref(TonemapParams(mode, gamma, FLAG_DEVICE_OUTPUT, 0)), out_ptr))


def write_ppm(path, rgb8: np.ndarray) -> None:
    """are_write_ppm of an (h, w, 3) uint8 image."""
    a = np.ascontiguousarray(rgb8, np.uint8)
    h, w = a.shape[:2]
    check(load().are_write_ppm(os.fsencode(path), a.ctypes.data, w, h))


def write_pfm(path, rgb: np.ndarray) -> None:
    """are_write_pfm of an (h, w, 3) float32 image."""
    a = np.ascontiguousarray(rgb, np.float32)
    h, w = a.shape[:2]
    check(load().are_write_pfm(os.fsencode(path), a.ctypes.data, w, h))


def read_ppm(path) -> np.ndarray:
    """are_read_ppm -> (h, w, 3) float32 texels, byte / 255."""
    L = load()
    w, h = C.c_int32(), C.c_int32()
    check(L.are_read_ppm(os.fsencode(path), C.byref(w), C.byref(h), None))
    out = np.empty((h.value, w.value, 3), np.float32)
    check(L.are_read_ppm(os.fsencode(path), C.byref(w), C.byref(h), out.ctypes.data))
    return out
