"""ctypes access to the oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of bench.py use this module, as the checker.

``Oracle`` wraps oracle/_build/liborc.so (the C restatement).  ``RefRT`` and
``RefLib`` wrap oracle/_ref/*.so, built from the reference's own sources, when
they exist (they cannot be rebuilt where the reference tree is absent).

Scenes are passed as any object with the numpy attributes of
``are_gb300.SceneArrays`` (spheres, sphere_mat, quads, quad_mat, triangles,
triangle_uv, triangle_mat, materials, textures, texels, background, bg_a,
bg_b, triangle_test); materials/textures are numpy structured arrays with the
48-byte layouts of the C structs.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_f = C.POINTER(C.c_float)
_d = C.POINTER(C.c_double)
_i32 = C.POINTER(C.c_int32)


class OrcScene(C.Structure):
    _fields_ = [
        ("n_spheres", C.c_int32), ("spheres", _f), ("sphere_mat", _i32),
        ("n_quads", C.c_int32), ("quads", _f), ("quad_mat", _i32),
        ("n_triangles", C.c_int32), ("triangles", _f), ("triangle_uv", _f), ("triangle_mat", _i32),
        ("n_materials", C.c_int32), ("materials", C.c_void_p),
        ("n_textures", C.c_int32), ("textures", C.c_void_p),
        ("n_texels", C.c_int64), ("texels", _f),
        ("background", C.c_int32), ("bg_a", C.c_float * 3), ("bg_b", C.c_float * 3),
        ("triangle_test", C.c_int32), ("bvh_leaf_size", C.c_int32),
    ]


class OrcCamera(C.Structure):
    _fields_ = [("lookfrom", C.c_float * 3), ("lookat", C.c_float * 3), ("vup", C.c_float * 3),
                ("vfov_deg", C.c_float), ("aperture", C.c_float), ("focus_dist", C.c_float)]


class OrcParams(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("spp", C.c_int32), ("max_depth", C.c_int32),
                ("seed", C.c_uint64), ("rr_depth", C.c_int32), ("t_min", C.c_float), ("estimator", C.c_int32),
                ("flags", C.c_int32), ("pool_size", C.c_int32), ("chunk", C.c_int32), ("block_size", C.c_int32),
                ("reserved_", C.c_int32)]


class OrcStats(C.Structure):
    _fields_ = [("samples", C.c_int64), ("segments", C.c_int64)]


def _ptr(a, t):
    if a is None or len(a) == 0:
        return C.cast(None, t)
    return a.ctypes.data_as(t)


def _scene_struct(s) -> tuple[OrcScene, list]:
    keep = []

    def arr(x, dt):
        if x is None:
            return None
        y = np.ascontiguousarray(x, dtype=dt)
        keep.append(y)
        return y

    sp, spm = arr(s.spheres, np.float32), arr(s.sphere_mat, np.int32)
    qd, qdm = arr(s.quads, np.float32), arr(s.quad_mat, np.int32)
    tr, tru, trm = arr(s.triangles, np.float32), arr(s.triangle_uv, np.float32), arr(s.triangle_mat, np.int32)
    mats = np.ascontiguousarray(s.materials)
    texs = np.ascontiguousarray(s.textures)
    tx = arr(s.texels, np.float32)
    keep += [mats, texs]
    st = OrcScene()
    st.n_spheres = len(spm)
    st.spheres = _ptr(sp, _f)
    st.sphere_mat = _ptr(spm, _i32)
    st.n_quads = len(qdm)
    st.quads = _ptr(qd, _f)
    st.quad_mat = _ptr(qdm, _i32)
    st.n_triangles = len(trm)
    st.triangles = _ptr(tr, _f)
    st.triangle_uv = _ptr(tru, _f) if tru is not None and len(tru) else C.cast(None, _f)
    st.triangle_mat = _ptr(trm, _i32)
    st.n_materials = len(mats)
    st.materials = mats.ctypes.data if len(mats) else None
    st.n_textures = len(texs)
    st.textures = texs.ctypes.data if len(texs) else None
    st.n_texels = 0 if tx is None else tx.size // 3
    st.texels = _ptr(tx, _f) if tx is not None else C.cast(None, _f)
    st.background = int(s.background)
    st.bg_a = (C.c_float * 3)(*[float(v) for v in s.bg_a])
    st.bg_b = (C.c_float * 3)(*[float(v) for v in s.bg_b])
    st.triangle_test = int(s.triangle_test)
    st.bvh_leaf_size = 0
    return st, keep


def camera_struct(cam) -> OrcCamera:
    c = OrcCamera()
    c.lookfrom = (C.c_float * 3)(*cam["lookfrom"])
    c.lookat = (C.c_float * 3)(*cam["lookat"])
    c.vup = (C.c_float * 3)(*cam["vup"])
    c.vfov_deg = cam["vfov_deg"]
    c.aperture = cam.get("aperture", 0.0)
    c.focus_dist = cam.get("focus_dist", 1.0)
    return c


def params_struct(p) -> OrcParams:
    q = OrcParams()
    for k, _ in OrcParams._fields_:
        if k in p:
            setattr(q, k, p[k])
    return q


class Oracle:
    """The C restatement: closest hit and the path estimator in FP32/FP64."""

    def __init__(self, path: str | Path | None = None):
        if path is None:
            # rebuilds only when a source is newer than the library
            from oracle import build as _b  # noqa: PLC0415
            path = _b.build_oracle()
        path = Path(path)
        L = C.CDLL(str(path))
        L.orc_prepare.restype = C.c_void_p
        L.orc_prepare.argtypes = [C.POINTER(OrcScene), C.c_int32]
        L.orc_release.argtypes = [C.c_void_p]
        L.orc_intersect_f32.argtypes = [C.c_void_p, _f, C.c_int64, _f, C.c_int32]
        L.orc_render_f32.argtypes = [C.c_void_p, C.POINTER(OrcCamera), C.POINTER(OrcParams), _f, _f,
                                     C.c_int32, C.c_int32, C.c_int32, C.POINTER(OrcStats)]
        L.orc_render_f64.argtypes = [C.c_void_p, C.POINTER(OrcCamera), C.POINTER(OrcParams), _d, _d,
                                     C.c_int32, C.c_int32, C.c_int32, C.POINTER(OrcStats)]
        L.orc_rng_u32.restype = C.c_uint32
        L.orc_rng_u32.argtypes = [C.c_uint64, C.c_uint32]
        L.orc_path_key.restype = C.c_uint64
        L.orc_path_key.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32]
        L.orc_texture_eval_f32.argtypes = [C.c_void_p, C.c_int32, C.c_float, C.c_float, _f, _f]
        L.orc_hemisphere_f32.argtypes = [_f, C.c_float, C.c_float, _f]
        L.orc_reflect_f64.argtypes = [_d, _d, _d]
        L.orc_refract_f64.argtypes = [_d, _d, C.c_double, _d]
        L.orc_ppm_quantize.argtypes = [_f, C.c_int64, C.c_float, C.POINTER(C.c_uint8)]
        L.orc_texture_quantize.argtypes = [_f, C.c_int64, C.POINTER(C.c_uint8)]
        L.orc_render_legacy.argtypes = [C.c_void_p, C.POINTER(OrcCamera), C.POINTER(OrcParams), _f, C.c_int32,
                                        C.c_uint32, C.c_int32]
        L.orc_mt19937.argtypes = [C.c_uint32, C.c_int64, C.POINTER(C.c_uint32), _f]
        L.orc_guide_num_params.restype = C.c_int32
        L.orc_guide_forward.argtypes = [_f, _f, C.c_int64, _d]
        L.orc_guide_pdf.restype = C.c_double
        L.orc_guide_pdf.argtypes = [_d, _d]
        L.orc_guide_loss_grad.restype = C.c_double
        L.orc_guide_loss_grad.argtypes = [_f, _f, C.c_int64, _d]
        L.orc_guide_encode.argtypes = [_d, _d]
        self.lib = L

    # path-guiding network (FP64) -------------------------------------------------
    def quantize(self, rgb: np.ndarray, mode: int = 0, gamma: float = 2.2) -> np.ndarray:
        """8-bit quantisation: mode 0 rt.cpp:384-386 (gamma), 1 texture.cpp:378-383 (linear)."""
        a = np.ascontiguousarray(rgb, np.float32).reshape(-1)
        out = np.empty(a.size, np.uint8)
        u8 = out.ctypes.data_as(C.POINTER(C.c_uint8))
        if mode == 0:
            self.lib.orc_ppm_quantize(a.ctypes.data_as(_f), a.size, gamma, u8)
        else:
            self.lib.orc_texture_quantize(a.ctypes.data_as(_f), a.size, u8)
        return out.reshape(np.shape(rgb))

    def guide_forward(self, params: np.ndarray, feat: np.ndarray) -> np.ndarray:
        params = np.ascontiguousarray(params, np.float32)
        feat = np.ascontiguousarray(feat, np.float32).reshape(-1, 9)
        out = np.zeros((len(feat), 48))
        self.lib.orc_guide_forward(_ptr(params, _f), _ptr(feat.reshape(-1), _f), len(feat), _ptr(out.reshape(-1), _d))
        return out

    def guide_loss_grad(self, params: np.ndarray, samples: np.ndarray):
        params = np.ascontiguousarray(params, np.float32)
        samples = np.ascontiguousarray(samples, np.float32).reshape(-1, 13)
        grad = np.zeros(self.lib.orc_guide_num_params())
        loss = self.lib.orc_guide_loss_grad(_ptr(params, _f), _ptr(samples.reshape(-1), _f), len(samples),
                                            _ptr(grad, _d))
        return loss, grad

    def guide_pdf(self, out48: np.ndarray, w: np.ndarray) -> float:
        o = np.ascontiguousarray(out48, np.float64)
        w = np.ascontiguousarray(w, np.float64)
        return self.lib.orc_guide_pdf(_ptr(o, _d), _ptr(w, _d))

    class Ctx:
        def __init__(self, orc, scene, accel):
            self.orc = orc
            self.struct, self.keep = _scene_struct(scene)
            self.h = orc.lib.orc_prepare(C.byref(self.struct), accel)
            if not self.h:
                raise MemoryError("orc_prepare failed")

        def __del__(self):
            if getattr(self, "h", None):
                self.orc.lib.orc_release(self.h)
                self.h = None

    def prepare(self, scene, accel: int = -1) -> "Oracle.Ctx":
        return Oracle.Ctx(self, scene, accel)

    def intersect(self, ctx, rays: np.ndarray, nthreads: int = 8) -> np.ndarray:
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
        hits = np.empty((len(rays), 4), np.float32)
        rc = self.lib.orc_intersect_f32(ctx.h, _ptr(rays.reshape(-1), _f), len(rays), _ptr(hits.reshape(-1), _f),
                                        nthreads)
        assert rc == 0
        return hits

    def render(self, ctx, cam: dict, params: dict, fp64: bool = False, nthreads: int = 8, rows=(0, 0)):
        p = params_struct(params)
        c = camera_struct(cam)
        n = params["width"] * params["height"] * 3
        dt, pt, fn = ((np.float64, _d, self.lib.orc_render_f64) if fp64 else
                      (np.float32, _f, self.lib.orc_render_f32))
        mean = np.zeros(n, dt)
        var = np.zeros(n, dt)
        st = OrcStats()
        rc = fn(ctx.h, C.byref(c), C.byref(p), _ptr(mean, pt), _ptr(var, pt), rows[0], rows[1], nthreads,
                C.byref(st))
        assert rc == 0
        shape = (params["height"], params["width"], 3)
        return mean.reshape(shape), var.reshape(shape), {"samples": st.samples, "segments": st.segments}


def render_legacy(orc: "Oracle", ctx, cam: dict, params: dict, rng_mode: int, mt_seed: int = 0,
                  nthreads: int = 8) -> np.ndarray:
    """rt.cpp's estimator (AO + depth-0 mirror + diffuse paths) on the oracle."""
    p = params_struct(params)
    c = camera_struct(cam)
    out = np.zeros(params["width"] * params["height"] * 3, np.float32)
    assert orc.lib.orc_render_legacy(ctx.h, C.byref(c), C.byref(p), _ptr(out, _f), rng_mode, mt_seed, nthreads) == 0
    return out.reshape(params["height"], params["width"], 3)


class RefRT:
    """experiments/rt.cpp compiled from the reference tree (oracle/_ref)."""

    PATH = HERE / "_ref" / "libref_rt.so"

    def __init__(self):
        L = C.CDLL(str(self.PATH))
        L.ref_scene_export.argtypes = [_f, C.c_int]
        L.ref_intersect.argtypes = [_f, C.c_int64, _f]
        L.ref_intersect_soup.argtypes = [_f, C.c_int, _f, C.c_int64, _f]
        L.ref_checker_at.argtypes = [_f, _f, C.c_float, C.c_float, C.c_float, _f]
        L.ref_rotate_to_hemisphere.argtypes = [_f, C.c_float, C.c_float, _f]
        L.ref_render.argtypes = [C.c_uint, C.c_int, C.c_int, _f]
        L.ref_write_ppm.argtypes = [_f, C.c_int, C.c_int, C.c_char_p]
        self.lib = L

    @classmethod
    def available(cls) -> bool:
        return cls.PATH.exists()

    def scene(self) -> np.ndarray:
        n = self.lib.ref_scene_size()
        out = np.zeros((n, 28), np.float32)
        assert self.lib.ref_scene_export(_ptr(out.reshape(-1), _f), n) == n
        return out

    def intersect(self, rays6: np.ndarray) -> np.ndarray:
        rays6 = np.ascontiguousarray(rays6, np.float32)
        hits = np.empty((len(rays6), 4), np.float32)
        self.lib.ref_intersect(_ptr(rays6.reshape(-1), _f), len(rays6), _ptr(hits.reshape(-1), _f))
        return hits

    def intersect_soup(self, tris9: np.ndarray, rays6: np.ndarray) -> np.ndarray:
        tris9 = np.ascontiguousarray(tris9, np.float32)
        rays6 = np.ascontiguousarray(rays6, np.float32)
        hits = np.empty((len(rays6), 4), np.float32)
        self.lib.ref_intersect_soup(_ptr(tris9.reshape(-1), _f), len(tris9), _ptr(rays6.reshape(-1), _f),
                                    len(rays6), _ptr(hits.reshape(-1), _f))
        return hits

    def render(self, seed: int, w: int, h: int) -> np.ndarray:
        out = np.zeros(w * h * 3, np.float32)
        self.lib.ref_render(seed, w, h, _ptr(out, _f))
        return out.reshape(h, w, 3)


class RefLib:
    """The reference library's src/*.cpp compiled from the reference tree."""

    PATH = HERE / "_ref" / "libref_lib.so"

    def __init__(self):
        L = C.CDLL(str(self.PATH))
        L.ref_lib_triangle_check.argtypes = [_d, _d, _d]
        L.ref_lib_triangles_intersect.argtypes = [_d, C.c_int, _d, C.c_int64, _d]
        L.ref_lib_reflect.argtypes = [_d, _d, _d]
        L.ref_lib_refract.argtypes = [_d, _d, C.c_double, _d]
        L.ref_lib_plane_intersect.argtypes = [_d, _d, _d, _d, _d]
        L.ref_lib_texture_load.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int), _d, C.c_int64]
        self.lib = L

    @classmethod
    def available(cls) -> bool:
        return cls.PATH.exists()
