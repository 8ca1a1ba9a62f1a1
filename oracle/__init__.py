"""TEST INFRASTRUCTURE ONLY -- ctypes front of the CPU oracle (liboracle.so).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this package; it is the
checker, never the measured or shipped path.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from sparkle_gb300.abi import (HIT_DTYPE, MarshalledScene, Scene, spk_camera, spk_config, spk_material)

from . import build as _build

FAITHFUL, PRUNED = 0, 1
_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        L = C.CDLL(path)
        vp = C.c_void_p
        L.or_scene_create.restype = vp
        L.or_scene_create.argtypes = [vp, C.c_uint32, vp, C.c_uint32, vp, C.c_uint32, vp]
        L.or_scene_destroy.argtypes = [vp]
        L.or_trace.restype = C.c_uint64
        L.or_trace.argtypes = [vp, vp, C.c_uint64, vp, C.c_int32, C.c_int32, C.c_int32]
        L.or_trace_brute.argtypes = [vp, vp, C.c_uint64, vp, C.c_int32]
        L.or_renderer_create.restype = vp
        L.or_renderer_create.argtypes = [vp, vp, vp]
        L.or_renderer_destroy.argtypes = [vp]
        L.or_render.argtypes = [vp, C.c_uint32, C.c_int32, C.c_int32, C.c_uint32, C.c_uint32]
        L.or_render_rows.argtypes = [vp, C.c_uint32, C.c_int32, C.c_int32, C.c_uint32, C.c_uint32, C.c_uint32]
        L.or_read_framebuffer.argtypes = [vp, vp, vp]
        L.or_read_gbuffer.argtypes = [vp, vp, vp]
        L.or_guides.argtypes = [vp, vp, vp]
        L.or_scene_set_textures.argtypes = [vp, vp, C.c_uint32, vp]
        L.or_counts.argtypes = [vp, vp, vp, vp]
        L.or_sample_counts.argtypes = [vp, vp, vp]
        L.or_rng_fill.argtypes = [C.c_int32, C.c_uint64, C.c_uint32, vp, vp]
        L.or_float_to_half.restype = C.c_uint32
        L.or_float_to_half.argtypes = [C.c_float]
        L.or_rgba16f_to_rgba8.argtypes = [vp, C.c_uint64, vp]
        L.or_sky_from_equirect.argtypes = [vp, C.c_uint32, C.c_uint32, C.c_int32, C.c_uint32, vp]
        L.or_sample_surface.argtypes = [vp, vp, vp, vp, C.c_uint32, vp]
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class OracleScene:
    def __init__(self, scene: Scene):
        self.m = MarshalledScene(scene)
        a = self.m.args()
        self.h = lib().or_scene_create(C.cast(a[0], C.c_void_p), a[1], C.cast(a[2], C.c_void_p), a[3],
                                       C.cast(a[4], C.c_void_p), a[5], C.cast(a[6], C.c_void_p))
        if not self.h:
            raise RuntimeError("or_scene_create failed")
        if scene.textures or self.m.has_maps:
            lib().or_scene_set_textures(self.h, C.cast(self.m.textures, C.c_void_p), len(scene.textures),
                                        C.cast(self.m.maps, C.c_void_p) if self.m.has_maps else None)

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_scene_destroy(self.h)
            self.h = None

    def trace(self, rays: np.ndarray, any_hit: bool = False, traversal: int = FAITHFUL, threads: int = 0):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        hits = np.zeros(rays.shape[0], HIT_DTYPE)
        ovf = lib().or_trace(self.h, _p(rays), rays.shape[0], _p(hits), int(any_hit), traversal, threads)
        return hits, int(ovf)

    def trace_brute(self, rays: np.ndarray, threads: int = 0):
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        hits = np.zeros(rays.shape[0], HIT_DTYPE)
        lib().or_trace_brute(self.h, _p(rays), rays.shape[0], _p(hits), threads)
        return hits


class OracleRenderer:
    """The reference cpu pipeline (CPURenderer) restated on the host."""

    def __init__(self, scene: OracleScene, config: spk_config, camera: spk_camera):
        self.scene = scene
        self.config = config
        self.camera = camera
        self.h = lib().or_renderer_create(scene.h, C.byref(config), C.byref(camera))

    def __del__(self):
        if getattr(self, "h", None):
            lib().or_renderer_destroy(self.h)
            self.h = None

    def render(self, frames: int = 1, traversal: int = FAITHFUL, threads: int = 0, rows=None, row_step: int = 1):
        """Renders `frames` frames; only rows range(*rows)[::row_step] when `rows` is given (timing samples)."""
        r0, r1 = (0, 0) if rows is None else rows
        lib().or_render_rows(self.h, frames, traversal, threads, r0, r1, row_step)

    def framebuffer(self):
        w, h = self.config.width, self.config.height
        hdr = np.zeros((h, w, 4), np.float32)
        out = np.zeros((h, w, 4), np.uint16)
        lib().or_read_framebuffer(self.h, _p(hdr), _p(out))
        return hdr, out

    def gbuffer(self):
        w, h = self.config.width, self.config.height
        col = np.zeros((h, w, 4), np.float32)
        nrm = np.zeros((h, w, 3), np.float32)
        lib().or_read_gbuffer(self.h, _p(col), _p(nrm))
        return col, nrm

    def guides(self):
        """Primary-hit guides: (normal xyz + linear depth, albedo rgb + hit flag), rows bottom-up."""
        w, h = self.config.width, self.config.height
        nd = np.zeros((h, w, 4), np.float32)
        al = np.zeros((h, w, 4), np.float32)
        lib().or_guides(self.h, _p(nd), _p(al))
        return nd, al

    def counts(self):
        a, b, c = C.c_uint64(), C.c_uint64(), C.c_uint64()
        lib().or_counts(self.h, C.byref(a), C.byref(b), C.byref(c))
        return a.value, b.value, c.value

    def sample_counts(self):
        a, b = C.c_uint32(), C.c_uint32()
        lib().or_sample_counts(self.h, C.byref(a), C.byref(b))
        return a.value, b.value


def rng_fill(kind: int, seed: int, n: int):
    u = np.zeros(n, np.uint32)
    f = np.zeros(n, np.float32)
    lib().or_rng_fill(kind, seed, n, _p(u), _p(f))
    return u, f


def float_to_half(x: float) -> int:
    return int(lib().or_float_to_half(x))


def sky_from_equirect(rgba, srgb: bool, n: int) -> np.ndarray:
    """The reference's sky cube cook (SkyLightCookJob::Execute, SkyLight.cpp:83-113) of an (H, W, 4) map."""
    src = np.ascontiguousarray(rgba, np.float32)
    out = np.zeros((6, n, n, 4), np.float32)
    lib().or_sky_from_equirect(_p(src), src.shape[1], src.shape[0], int(srgb), n, _p(out))
    return out


def rgba16f_to_rgba8(rgba16f) -> np.ndarray:
    """The reference's screenshot conversion (ConvertPixelsToRGBA8, Image.cpp:54-67) of half bits."""
    src = np.ascontiguousarray(rgba16f, np.uint16)
    out = np.zeros(src.shape, np.uint8)
    lib().or_rgba16f_to_rgba8(_p(src), src.size // 4, _p(out))
    return out


def sample_surface(mat: spk_material, ray_dir, normal, tangent, seed: int):
    rd = np.asarray(ray_dir, np.float32)
    n = np.asarray(normal, np.float32)
    t = np.asarray(tangent, np.float32)
    out = np.zeros(7, np.float32)
    lib().or_sample_surface(C.byref(mat), _p(rd), _p(n), _p(t), seed, _p(out))
    return out
