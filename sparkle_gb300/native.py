"""ctypes binding of the in-tree CUDA library (sparkle_gb300/_build/libspk.so) and a thin Python front.

There is no fallback: if the library is missing, or the process has no CUDA device, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build
from .abi import (HIT_DTYPE, MarshalledScene, Scene, spk_camera, spk_config, spk_stats, spk_tuning)

_lib = None

SPK_ERRORS = {0: "ok", 1: "invalid argument", 2: "cuda error", 3: "out of memory", 4: "not ready",
              5: "device limit", 6: "internal"}

# Every symbol include/spk.h declares.
EXPORTED = ["spk_abi_version", "spk_create", "spk_destroy", "spk_last_error", "spk_set_scene", "spk_set_camera",
            "spk_camera_from_look", "spk_set_config", "spk_render", "spk_read_framebuffer",
            "spk_framebuffer_device", "spk_sample_counts", "spk_is_converged", "spk_trace", "spk_trace_device",
            "spk_synchronize", "spk_get_stats", "spk_set_instrumentation", "spk_render_noalloc",
            "spk_tuning_defaults", "spk_set_tuning", "spk_get_tuning"]


class SpkError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"spk error {status} ({SPK_ERRORS.get(status, '?')}): {message}")
        self.status = status


def library_path(build: bool = True) -> str:
    if build:
        return _build.build()
    return _build.LIB


def lib(build: bool = True):
    """Loads libspk.so (building it first when `build` and it is stale)."""
    global _lib
    if _lib is None:
        path = library_path(build)
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: run sparkle_gb300.build.build() (the CUDA path has no fallback)")
        L = C.CDLL(path)
        vp, u32, i32, u64 = C.c_void_p, C.c_uint32, C.c_int32, C.c_uint64
        L.spk_abi_version.restype = u32
        L.spk_create.argtypes = [i32, C.POINTER(vp)]
        L.spk_destroy.argtypes = [vp]
        L.spk_last_error.restype = C.c_char_p
        L.spk_last_error.argtypes = [vp]
        L.spk_set_scene.argtypes = [vp, vp, u32, vp, u32, vp, u32, vp]
        L.spk_set_camera.argtypes = [vp, vp]
        L.spk_camera_from_look.argtypes = [vp, vp, vp, C.c_float, C.c_float, C.c_float, C.c_float, u32, u32, vp]
        L.spk_set_config.argtypes = [vp, vp]
        L.spk_render.argtypes = [vp, u32]
        L.spk_read_framebuffer.argtypes = [vp, vp, vp]
        L.spk_framebuffer_device.argtypes = [vp, C.POINTER(vp), C.POINTER(vp)]
        L.spk_sample_counts.argtypes = [vp, C.POINTER(u32), C.POINTER(u32)]
        L.spk_is_converged.restype = i32
        L.spk_is_converged.argtypes = [vp]
        L.spk_trace.argtypes = [vp, vp, u64, vp, i32]
        L.spk_trace_device.argtypes = [vp, vp, u64, vp, i32]
        L.spk_synchronize.argtypes = [vp]
        L.spk_get_stats.argtypes = [vp, vp]
        L.spk_set_instrumentation.argtypes = [vp, u32]
        L.spk_render_noalloc.argtypes = [vp, u32, vp, vp]
        L.spk_tuning_defaults.argtypes = [vp]
        L.spk_tuning_defaults.restype = None
        L.spk_set_tuning.argtypes = [vp, vp]
        L.spk_get_tuning.argtypes = [vp, vp]
        for name in EXPORTED:
            if name != "spk_last_error" and getattr(L, name).restype is C.c_int:
                getattr(L, name).restype = i32
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


class Context:
    """One spk_ctx: resident scene + camera + config + frame buffers on one CUDA device."""

    def __init__(self, device: int = 0):
        self.L = lib()
        h = C.c_void_p()
        st = self.L.spk_create(device, C.byref(h))
        if st != 0:
            raise SpkError(st, "spk_create failed (no CUDA device?)")
        self.h = h
        self._scene = None
        self.config = None

    def close(self):
        if getattr(self, "h", None):
            self.L.spk_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _check(self, st: int):
        if st != 0:
            raise SpkError(st, self.L.spk_last_error(self.h).decode())

    def set_scene(self, scene: Scene):
        m = MarshalledScene(scene)
        a = m.args()
        self._check(self.L.spk_set_scene(self.h, C.cast(a[0], C.c_void_p), a[1], C.cast(a[2], C.c_void_p), a[3],
                                         C.cast(a[4], C.c_void_p), a[5], C.cast(a[6], C.c_void_p)))
        self._scene = m

    def set_camera(self, camera: spk_camera):
        self._check(self.L.spk_set_camera(self.h, C.byref(camera)))

    def set_config(self, config: spk_config):
        self._check(self.L.spk_set_config(self.h, C.byref(config)))
        self.config = config

    def render(self, frames: int = 1):
        self._check(self.L.spk_render(self.h, frames))

    def synchronize(self):
        self._check(self.L.spk_synchronize(self.h))

    def framebuffer(self):
        w, h = self.config.width, self.config.height
        hdr = np.zeros((h, w, 4), np.float32)
        out = np.zeros((h, w, 4), np.uint16)
        self._check(self.L.spk_read_framebuffer(self.h, _p(hdr), _p(out)))
        return hdr, out

    def read_framebuffer_into(self, hdr, out):
        """Reads into caller-owned host buffers (ctypes addresses or numpy arrays; either may be None)."""
        hp = None if hdr is None else (_p(hdr) if isinstance(hdr, np.ndarray) else C.c_void_p(hdr))
        op = None if out is None else (_p(out) if isinstance(out, np.ndarray) else C.c_void_p(out))
        self._check(self.L.spk_read_framebuffer(self.h, hp, op))

    def framebuffer_device(self):
        a, b = C.c_void_p(), C.c_void_p()
        self._check(self.L.spk_framebuffer_device(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def sample_counts(self):
        a, b = C.c_uint32(), C.c_uint32()
        self._check(self.L.spk_sample_counts(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def is_converged(self) -> bool:
        return bool(self.L.spk_is_converged(self.h))

    def trace(self, rays: np.ndarray, any_hit: bool = False) -> np.ndarray:
        rays = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        hits = np.zeros(rays.shape[0], HIT_DTYPE)
        self._check(self.L.spk_trace(self.h, _p(rays), rays.shape[0], _p(hits), int(any_hit)))
        return hits

    def trace_device(self, d_rays: int, n: int, d_hits: int, any_hit: bool = False):
        self._check(self.L.spk_trace_device(self.h, C.c_void_p(d_rays), n, C.c_void_p(d_hits), int(any_hit)))

    def render_noalloc(self, frames: int, d_hdr: int, d_rgba16f: int):
        """spk_render_noalloc: renders into caller-owned device buffers without allocating (see include/spk.h)."""
        self._check(self.L.spk_render_noalloc(self.h, frames, C.c_void_p(d_hdr), C.c_void_p(d_rgba16f)))

    def set_instrumentation(self, count_traffic: bool):
        self._check(self.L.spk_set_instrumentation(self.h, 1 if count_traffic else 0))

    def tuning(self) -> dict:
        t = spk_tuning()
        self._check(self.L.spk_get_tuning(self.h, C.byref(t)))
        return {k: getattr(t, k) for k, _ in spk_tuning._fields_ if k != "reserved"}

    def set_tuning(self, **knobs):
        """Updates the named knobs of spk_tuning (the others keep their current value)."""
        t = spk_tuning()
        self._check(self.L.spk_get_tuning(self.h, C.byref(t)))
        for k, v in knobs.items():
            if k not in dict(spk_tuning._fields_) or k == "reserved":
                raise KeyError(f"unknown tuning knob {k!r}")
            setattr(t, k, int(v))
        self._check(self.L.spk_set_tuning(self.h, C.byref(t)))

    def stats(self) -> dict:
        s = spk_stats()
        self._check(self.L.spk_get_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in spk_stats._fields_}


def camera_from_look(position, target, world_up, vfov_rad, focus_distance, aperture_radius, exposure, width, height):
    """spk_camera_from_look through the library."""
    cam = spk_camera()
    f3 = C.c_float * 3
    st = lib().spk_camera_from_look(C.byref(f3(*position)), C.byref(f3(*target)), C.byref(f3(*world_up)),
                                    vfov_rad, focus_distance, aperture_radius, exposure, width, height,
                                    C.byref(cam))
    if st != 0:
        raise SpkError(st, "spk_camera_from_look")
    return cam
