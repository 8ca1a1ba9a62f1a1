"""ctypes binding of the in-tree CUDA library (sparkle_gb300/_build/libspk.so) and a thin Python front.

There is no fallback: if the library is missing, or the process has no CUDA device, the calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build
from .abi import (HIT_DTYPE, MarshalledScene, Scene, affine_inverse, instance_array, spk_camera, spk_config,
                  spk_request, spk_scene_desc, spk_stats, spk_tuning)

_lib = None

SPK_ERRORS = {0: "ok", 1: "invalid argument", 2: "cuda error", 3: "out of memory", 4: "not ready",
              5: "device limit", 6: "internal", 7: "i/o"}

# Every symbol include/spk.h declares.
EXPORTED = ["spk_abi_version", "spk_create", "spk_destroy", "spk_last_error", "spk_set_scene", "spk_set_camera",
            "spk_camera_from_look", "spk_set_config", "spk_render", "spk_read_framebuffer",
            "spk_framebuffer_device", "spk_sample_counts", "spk_is_converged", "spk_trace", "spk_trace_device",
            "spk_synchronize", "spk_get_stats", "spk_set_instrumentation", "spk_render_noalloc",
            "spk_tuning_defaults", "spk_set_tuning", "spk_get_tuning", "spk_render_guides", "spk_guides_device",
            "spk_read_guides", "spk_set_scenes", "spk_render_batch", "spk_read_batch", "spk_set_instances",
            "spk_set_instance_transforms", "spk_update_mesh", "spk_read_bvh_nodes", "spk_read_rgba8",
            "spk_save_image", "spk_write_png", "spk_write_hdr", "spk_write_exr", "spk_convert_rgba8",
            "spk_flip", "spk_relmse", "spk_sky_from_equirect",
            # include/spk_denoise.h
            "spk_dn_create", "spk_dn_destroy", "spk_dn_last_error", "spk_dn_init", "spk_dn_num_params",
            "spk_dn_get_params", "spk_dn_set_params", "spk_dn_pack_features", "spk_dn_pack_halves", "spk_dn_train_step",
            "spk_dn_gradients", "spk_dn_infer", "spk_dn_fallback", "spk_dn_synchronize", "spk_dn_last_ms",
            "spk_dn_conv3x3", "spk_dn_state_size", "spk_dn_save_state", "spk_dn_load_state",
            "spk_dn_debug_wait_timeout", "spk_checkpoint_size", "spk_save_checkpoint", "spk_load_checkpoint",
            "spk_debug_fail_allocation", "spk_debug_walk_budget", "spk_bvh_blob_size", "spk_save_bvh", "spk_set_bvh",
            "spk_get_config", "spk_render_denoised"]


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
        L.spk_set_scenes.argtypes = [vp, vp, u32]
        L.spk_set_instances.argtypes = [vp, vp, u32]
        L.spk_set_instance_transforms.argtypes = [vp, u32, u32, vp, vp]
        L.spk_update_mesh.argtypes = [vp, u32, u32, vp, vp, vp]
        L.spk_read_bvh_nodes.argtypes = [vp, vp, u64, C.POINTER(u64)]
        L.spk_read_rgba8.argtypes = [vp, vp]
        L.spk_save_image.argtypes = [vp, C.c_char_p, u32]
        L.spk_write_png.argtypes = [C.c_char_p, vp, u32, u32]
        L.spk_write_hdr.argtypes = [C.c_char_p, vp, u32, u32]
        L.spk_write_exr.argtypes = [C.c_char_p, vp, u32, u32]
        L.spk_convert_rgba8.argtypes = [vp, u64, vp]
        L.spk_flip.argtypes = [i32, vp, vp, u32, u32, C.c_float, vp, C.POINTER(C.c_double)]
        L.spk_relmse.argtypes = [i32, vp, vp, u64, C.c_float, C.POINTER(C.c_double)]
        L.spk_sky_from_equirect.argtypes = [i32, vp, u32, u32, u32, u32, vp]
        L.spk_checkpoint_size.argtypes = [vp, C.POINTER(u64)]
        L.spk_save_checkpoint.argtypes = [vp, vp, u64]
        L.spk_load_checkpoint.argtypes = [vp, vp, u64]
        L.spk_debug_fail_allocation.argtypes = [u32]
        L.spk_debug_fail_allocation.restype = None
        L.spk_debug_walk_budget.argtypes = [vp, u32]
        L.spk_get_config.argtypes = [vp, vp]
        L.spk_render_denoised.argtypes = [vp, vp, u32, u32, C.c_float, vp, C.POINTER(u32)]
        L.spk_bvh_blob_size.argtypes = [vp, C.POINTER(u64)]
        L.spk_save_bvh.argtypes = [vp, vp, u64]
        L.spk_set_bvh.argtypes = [vp, vp, u64]
        L.spk_dn_state_size.argtypes = [vp, C.POINTER(u64)]
        L.spk_dn_save_state.argtypes = [vp, vp, u64]
        L.spk_dn_load_state.argtypes = [vp, vp, u64]
        L.spk_dn_debug_wait_timeout.argtypes = [vp]
        L.spk_render_batch.argtypes = [vp, vp, u32, u32, u32]
        L.spk_read_batch.argtypes = [vp, u32, vp, vp]
        L.spk_render_guides.argtypes = [vp]
        L.spk_guides_device.argtypes = [vp, C.POINTER(vp), C.POINTER(vp)]
        L.spk_read_guides.argtypes = [vp, vp, vp]
        f32, pf = C.c_float, C.POINTER(C.c_float)
        L.spk_dn_create.argtypes = [i32, u64, C.POINTER(vp)]
        L.spk_dn_destroy.argtypes = [vp]
        L.spk_dn_last_error.restype = C.c_char_p
        L.spk_dn_last_error.argtypes = [vp]
        L.spk_dn_init.argtypes = [vp, u64]
        L.spk_dn_num_params.argtypes = [vp, C.POINTER(u64)]
        L.spk_dn_get_params.argtypes = [vp, vp, u64]
        L.spk_dn_set_params.argtypes = [vp, vp, u64]
        L.spk_dn_pack_features.argtypes = [vp, vp, vp, vp, u32, u32, u32, vp]
        L.spk_dn_pack_halves.argtypes = [vp, vp, vp, vp, vp, u32, u32, u32, vp, vp]
        L.spk_dn_train_step.argtypes = [vp, vp, vp, u32, u32, u32, f32, pf]
        L.spk_dn_gradients.argtypes = [vp, vp, vp, u32, u32, u32, pf, vp, u64]
        L.spk_dn_infer.argtypes = [vp, vp, u32, u32, u32, vp]
        L.spk_dn_fallback.argtypes = [vp, vp, vp, vp, vp, u32, u32, u32, f32, vp, C.POINTER(u32)]
        L.spk_dn_synchronize.argtypes = [vp]
        L.spk_dn_last_ms.argtypes = [vp, pf]
        L.spk_dn_conv3x3.argtypes = [vp, i32, vp, u32, u32, vp, vp, vp, u32, u32, u32, u32, u32, i32, vp, u32, vp]
        for name in EXPORTED:
            if name not in ("spk_last_error", "spk_dn_last_error") and getattr(L, name).restype is C.c_int:
                getattr(L, name).restype = i32
        _lib = L
    return _lib


def _p(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def debug_fail_allocation(nth: int):
    """spk_debug_fail_allocation: the nth device allocation from now fails once (0 disarms)."""
    lib().spk_debug_fail_allocation(nth)


def _image_call(fn, path, img, dtype, channels=4):
    img = np.ascontiguousarray(img, dtype)
    if img.ndim != 3 or img.shape[2] != channels:
        raise ValueError(f"expected an (H, W, {channels}) image")
    st = fn(os.fsencode(path), _p(img), img.shape[1], img.shape[0])
    if st != 0:
        raise SpkError(st, f"cannot write {path}")


def write_png(path, rgba8):
    """spk_write_png: an (H, W, 4) uint8 image, rows top first."""
    _image_call(lib().spk_write_png, path, rgba8, np.uint8)


def write_hdr(path, rgba):
    """spk_write_hdr: an (H, W, 4) float32 image (alpha ignored), rows top first, as Radiance RGBE."""
    _image_call(lib().spk_write_hdr, path, rgba, np.float32)


def write_exr(path, rgba16f):
    """spk_write_exr: an (H, W, 4) uint16 (half bits) image, rows top first, as uncompressed OpenEXR."""
    _image_call(lib().spk_write_exr, path, rgba16f, np.uint16)


def convert_rgba8(rgba16f) -> np.ndarray:
    """spk_convert_rgba8: the screenshot conversion of an RGBA16F image (uint16 half bits) on the host."""
    src = np.ascontiguousarray(rgba16f, np.uint16)
    out = np.zeros(src.shape, np.uint8)
    st = lib().spk_convert_rgba8(_p(src), src.size // 4, _p(out))
    if st != 0:
        raise SpkError(st, "spk_convert_rgba8 failed")
    return out


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
        if scene.textures or m.has_maps:  # spk_set_scene has no texture arguments
            d = m.desc()
            self._check(self.L.spk_set_scenes(self.h, C.byref(d), 1))
        else:
            a = m.args()
            self._check(self.L.spk_set_scene(self.h, C.cast(a[0], C.c_void_p), a[1], C.cast(a[2], C.c_void_p), a[3],
                                             C.cast(a[4], C.c_void_p), a[5], C.cast(a[6], C.c_void_p)))
        self._scene = m

    def set_scenes(self, scenes):
        """Several resident scenes (spk_set_scenes) for render_batch; scene 0 is what render() sees."""
        ms = [MarshalledScene(sc) for sc in scenes]
        descs = (spk_scene_desc * len(ms))()
        for k, m in enumerate(ms):
            descs[k] = m.desc()
        self._check(self.L.spk_set_scenes(self.h, descs, len(ms)))
        self._scene = ms

    def set_instances(self, instances):
        """spk_set_instances: replaces the instance list (add / remove / reorder) over the resident meshes."""
        arr = instance_array(instances)
        self._check(self.L.spk_set_instances(self.h, arr, len(instances)))

    def set_instance_transforms(self, first: int, transforms):
        """spk_set_instance_transforms: new 3x4 transforms for instances first, first + 1, ..."""
        t = np.ascontiguousarray(np.asarray(transforms, np.float32).reshape(-1, 3, 4))
        inv = np.ascontiguousarray(np.stack([affine_inverse(m) for m in t]).astype(np.float32)) if len(t) else t
        self._check(self.L.spk_set_instance_transforms(self.h, first, len(t), _p(t), _p(inv)))

    def update_mesh(self, mesh_id: int, positions, normals=None, tangents=None):
        """spk_update_mesh: new vertex positions (and optionally normals / tangents) of a resident mesh."""
        pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
        nrm = None if normals is None else np.ascontiguousarray(normals, np.float32).reshape(-1, 3)
        tan = None if tangents is None else np.ascontiguousarray(tangents, np.float32).reshape(-1, 4)
        self._check(self.L.spk_update_mesh(self.h, mesh_id, pos.shape[0], _p(pos), None if nrm is None else _p(nrm),
                                           None if tan is None else _p(tan)))

    def read_rgba8(self) -> np.ndarray:
        """spk_read_rgba8: the screenshot image, (H, W, 4) uint8, rows top first."""
        out = np.zeros((self.config.height, self.config.width, 4), np.uint8)
        self._check(self.L.spk_read_rgba8(self.h, _p(out)))
        return out

    def save_image(self, path, fmt: int = 0):
        """spk_save_image: SPK_IMAGE_PNG (0), SPK_IMAGE_HDR (1) or SPK_IMAGE_EXR (2)."""
        self._check(self.L.spk_save_image(self.h, os.fsencode(path), fmt))

    def save_checkpoint(self) -> bytes:
        """spk_save_checkpoint: the accumulation state (frame buffer, output image, sample bookkeeping)."""
        n = C.c_uint64()
        self._check(self.L.spk_checkpoint_size(self.h, C.byref(n)))
        buf = np.zeros(n.value, np.uint8)
        self._check(self.L.spk_save_checkpoint(self.h, _p(buf), n.value))
        return buf.tobytes()

    def load_checkpoint(self, data: bytes):
        """spk_load_checkpoint: resume from save_checkpoint() bytes (same config; scene and camera set)."""
        buf = np.frombuffer(data, np.uint8)
        self._check(self.L.spk_load_checkpoint(self.h, _p(buf), buf.size))

    def save_bvh(self) -> bytes:
        """spk_save_bvh: the scene's BLASes as a blob for a later spk_set_bvh."""
        n = C.c_uint64()
        self._check(self.L.spk_bvh_blob_size(self.h, C.byref(n)))
        buf = np.zeros(n.value, np.uint8)
        self._check(self.L.spk_save_bvh(self.h, _p(buf), n.value))
        return buf.tobytes()

    def set_bvh(self, blob):
        """spk_set_bvh: reuse a saved blob's BLASes at the next set_scene (None drops it)."""
        if blob is None:
            self._check(self.L.spk_set_bvh(self.h, None, 0))
            return
        buf = np.frombuffer(blob, np.uint8)
        self._check(self.L.spk_set_bvh(self.h, _p(buf), buf.size))

    def debug_walk_budget(self, steps: int):
        """spk_debug_walk_budget: at most `steps` node steps per ray walk (0 = the default)."""
        self._check(self.L.spk_debug_walk_budget(self.h, steps))

    def bvh_nodes(self) -> np.ndarray:
        """The resident node array as (n, 80) bytes (spk_read_bvh_nodes)."""
        n = C.c_uint64()
        self._check(self.L.spk_read_bvh_nodes(self.h, None, 0, C.byref(n)))
        out = np.zeros((n.value, 80), np.uint8)
        self._check(self.L.spk_read_bvh_nodes(self.h, _p(out), n.value, C.byref(n)))
        return out

    def render_batch(self, requests, rng: int = 1, enable_nee: bool = False):
        """requests: list of dicts with scene, width, height, spp, bounce, seed, camera (spk_camera)."""
        arr = (spk_request * len(requests))()
        for k, r in enumerate(requests):
            arr[k] = spk_request(r["scene"], r["width"], r["height"], r["spp"], r["bounce"], r.get("seed", 0),
                                 r["camera"])
        self._check(self.L.spk_render_batch(self.h, arr, len(requests), rng, 1 if enable_nee else 0))
        self._batch = [(r["width"], r["height"]) for r in requests]

    def read_batch(self, index: int):
        """(hdr (H, W, 4) float32 bottom row first, rgba16f (H, W, 4) uint16 top row first) of request `index`."""
        w, h = self._batch[index]
        hdr = np.zeros((h, w, 4), np.float32)
        out = np.zeros((h, w, 4), np.uint16)
        self._check(self.L.spk_read_batch(self.h, index, _p(hdr), _p(out)))
        return hdr, out

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

    def render_guides(self):
        self._check(self.L.spk_render_guides(self.h))

    def guides(self):
        """Host copies of the primary-hit guides: (normal xyz + linear depth, albedo rgb + hit flag)."""
        w, h = self.config.width, self.config.height
        nd = np.zeros((h, w, 4), np.float32)
        al = np.zeros((h, w, 4), np.float32)
        self._check(self.L.spk_read_guides(self.h, _p(nd), _p(al)))
        return nd, al

    def guides_into(self, normal_depth_ptr: int, albedo_ptr: int):
        """Copies the guides to caller buffers (host or device pointers, H*W float4 each)."""
        self._check(self.L.spk_read_guides(self.h, C.c_void_p(normal_depth_ptr), C.c_void_p(albedo_ptr)))

    def guides_device(self):
        a, b = C.c_void_p(), C.c_void_p()
        self._check(self.L.spk_guides_device(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def tuning(self) -> dict:
        t = spk_tuning()
        self._check(self.L.spk_get_tuning(self.h, C.byref(t)))
        return {k: getattr(t, k) for k, _ in spk_tuning._fields_}

    def set_tuning(self, **knobs):
        """Updates the named knobs of spk_tuning (the others keep their current value)."""
        t = spk_tuning()
        self._check(self.L.spk_get_tuning(self.h, C.byref(t)))
        for k, v in knobs.items():
            if k not in dict(spk_tuning._fields_):
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


def _dptr(t) -> C.c_void_p:
    """Device pointer of a torch tensor (or None)."""
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p()


class Denoiser:
    """One spk_denoiser (the U-Net of include/spk_denoise.h) on one CUDA device. Tensors are torch CUDA
    tensors; each call waits for torch's current stream before it starts and for the denoiser's stream
    before it returns, so results can be read by torch right away."""

    FEATURES = 10
    ALIGN = 16

    def __init__(self, device: int = 0, seed: int = 0):
        self.L = lib()
        h = C.c_void_p()
        st = self.L.spk_dn_create(device, seed, C.byref(h))
        if st != 0:
            raise SpkError(st, "spk_dn_create failed (no CUDA device?)")
        self.h = h
        n = C.c_uint64()
        self._check(self.L.spk_dn_num_params(self.h, C.byref(n)))
        self.num_params = n.value

    def close(self):
        if getattr(self, "h", None):
            self.L.spk_dn_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def _check(self, st: int):
        if st != 0:
            raise SpkError(st, self.L.spk_dn_last_error(self.h).decode())

    @staticmethod
    def _torch_sync():
        import torch
        torch.cuda.current_stream().synchronize()

    def _done(self):
        self._check(self.L.spk_dn_synchronize(self.h))

    def init(self, seed: int):
        self._check(self.L.spk_dn_init(self.h, seed))

    def save_state(self) -> bytes:
        """spk_dn_save_state: parameters, Adam moments and step count (a training checkpoint)."""
        n = C.c_uint64()
        self._check(self.L.spk_dn_state_size(self.h, C.byref(n)))
        buf = np.zeros(n.value, np.uint8)
        self._check(self.L.spk_dn_save_state(self.h, _p(buf), n.value))
        return buf.tobytes()

    def load_state(self, data: bytes):
        """spk_dn_load_state: resume training from save_state() bytes."""
        buf = np.frombuffer(data, np.uint8)
        self._check(self.L.spk_dn_load_state(self.h, _p(buf), buf.size))

    def render_denoised(self, ctx, spp: int, tile: int = 16, threshold: float = 0.02):
        """spk_render_denoised: (denoised (H, W, 4) float32 bottom row first, fallback tile count)."""
        w, h = ctx.config.width, ctx.config.height
        out = np.zeros((h, w, 4), np.float32)
        tiles = C.c_uint32()
        self._check(self.L.spk_render_denoised(ctx.h, self.h, spp, tile, threshold, _p(out), C.byref(tiles)))
        return out, tiles.value

    def debug_wait_timeout(self):
        """spk_dn_debug_wait_timeout: a kernel whose bounded mbarrier wait runs out (raises SpkError 5)."""
        self._check(self.L.spk_dn_debug_wait_timeout(self.h))

    def get_params(self) -> np.ndarray:
        out = np.empty(self.num_params, np.float32)
        self._check(self.L.spk_dn_get_params(self.h, _p(out), self.num_params))
        return out

    def set_params(self, params: np.ndarray):
        params = np.ascontiguousarray(params, np.float32)
        assert params.size == self.num_params
        self._check(self.L.spk_dn_set_params(self.h, _p(params), self.num_params))

    def pack_features(self, hdr, normal_depth, albedo, out):
        """hdr, normal_depth, albedo: (n, h, w, 4) float32 CUDA tensors; out: (n, h, w, 10) float32."""
        n, h, w, _ = hdr.shape
        self._torch_sync()
        self._check(self.L.spk_dn_pack_features(self.h, _dptr(hdr), _dptr(normal_depth), _dptr(albedo), n, h, w,
                                                _dptr(out)))
        self._done()
        return out

    def pack_halves(self, full, half_a, normal_depth, albedo, out_a, out_b):
        """Features of sample half A (`half_a`) and half B (2 * full - half_a)."""
        n, h, w, _ = full.shape
        self._torch_sync()
        self._check(self.L.spk_dn_pack_halves(self.h, _dptr(full), _dptr(half_a), _dptr(normal_depth),
                                              _dptr(albedo), n, h, w, _dptr(out_a), _dptr(out_b)))
        self._done()

    def train_step(self, features, target, lr: float) -> float:
        n, h, w, _ = features.shape
        loss = C.c_float()
        self._torch_sync()
        self._check(self.L.spk_dn_train_step(self.h, _dptr(features), _dptr(target), n, h, w, lr, C.byref(loss)))
        self._done()
        return loss.value

    def gradients(self, features, target):
        n, h, w, _ = features.shape
        loss = C.c_float()
        grad = np.empty(self.num_params, np.float32)
        self._torch_sync()
        self._check(self.L.spk_dn_gradients(self.h, _dptr(features), _dptr(target), n, h, w, C.byref(loss),
                                            _p(grad), self.num_params))
        return loss.value, grad

    def infer(self, features, out=None):
        import torch
        n, h, w, _ = features.shape
        if out is None:
            out = torch.empty((n, h, w, 4), dtype=torch.float32, device=features.device)
        self._torch_sync()
        self._check(self.L.spk_dn_infer(self.h, _dptr(features), n, h, w, _dptr(out)))
        self._done()
        return out

    def last_ms(self) -> float:
        ms = C.c_float()
        self._check(self.L.spk_dn_last_ms(self.h, C.byref(ms)))
        return ms.value

    def fallback(self, denoised, den_a, den_b, plain, tile: int, threshold: float, out=None):
        import torch
        h, w = denoised.shape[-3], denoised.shape[-2]
        if out is None:
            out = torch.empty_like(denoised)
        count = C.c_uint32()
        self._torch_sync()
        self._check(self.L.spk_dn_fallback(self.h, _dptr(denoised), _dptr(den_a), _dptr(den_b), _dptr(plain), h, w,
                                           tile, threshold, _dptr(out), C.byref(count)))
        return out, count.value

    def conv3x3(self, op: int, x, x_channels: int, w, y, y_channels: int, n: int, h: int, width: int, bias=None,
                relu: bool = False, mask=None, mask_ld: int = 0, dw=None, x_ld: int = None, y_ld: int = None):
        """Low-level conv op on bf16 NHWC CUDA tensors (op 0 forward, 1 dgrad, 2 wgrad into dw)."""
        self._torch_sync()
        self._check(self.L.spk_dn_conv3x3(self.h, op, _dptr(x), x_channels, x_ld or x_channels, _dptr(w),
                                          _dptr(bias), _dptr(y), y_channels, y_ld or y_channels, n, h, width,
                                          1 if relu else 0, _dptr(mask), mask_ld, _dptr(dw)))
        self._done()
