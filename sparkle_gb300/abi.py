"""ctypes mirror of include/spk.h plus the Scene container that marshals numpy arrays into it.

The structs here are byte-for-byte the C structs of spk.h (checked by tests/test_abi.py), so a Python
caller and a C/C++ caller hand the library identical data.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

SPK_ABI_VERSION = 4
SPK_INVALID_ID = 0xFFFFFFFF

SPK_PRIM_MESH, SPK_PRIM_SPHERE = 0, 1
SPK_MAT_PBR, SPK_MAT_DIELECTRIC = 0, 1
SPK_SKY_NONE, SPK_SKY_GRADIENT, SPK_SKY_CUBE = 0, 1, 2
SPK_RNG_XOSHIRO128P, SPK_RNG_XOSHIRO256SS = 0, 1
SPK_KERNEL_AUTO, SPK_KERNEL_MEGAKERNEL, SPK_KERNEL_WAVEFRONT = 0, 1, 2
SPK_IMAGE_PNG, SPK_IMAGE_HDR, SPK_IMAGE_EXR = 0, 1, 2

_f = C.c_float
_u32 = C.c_uint32
_pf = C.POINTER(C.c_float)
_pu32 = C.POINTER(C.c_uint32)


class spk_mesh(C.Structure):
    _fields_ = [("positions", _pf), ("normals", _pf), ("tangents", _pf), ("uvs", _pf), ("indices", _pu32),
                ("num_vertices", _u32), ("num_faces", _u32)]


class spk_instance(C.Structure):
    _fields_ = [("type", _u32), ("mesh_id", _u32), ("material_id", _u32), ("radius", _f),
                ("transform", _f * 12), ("inv_transform", _f * 12)]


class spk_material(C.Structure):
    _fields_ = [("type", _u32), ("base_color", _f * 3), ("emissive", _f * 3), ("metallic", _f),
                ("roughness", _f), ("eta", _f)]


class spk_sky(C.Structure):
    _fields_ = [("mode", _u32), ("color", _f * 3), ("cube_size", _u32), ("cube_rgba", _pf)]


class spk_camera(C.Structure):
    _fields_ = [("position", _f * 3), ("right", _f * 3), ("up", _f * 3), ("front", _f * 3),
                ("lower_left", _f * 3), ("max_u", _f * 3), ("max_v", _f * 3), ("aperture_radius", _f),
                ("exposure", _f), ("far_plane", _f)]


class spk_config(C.Structure):
    _fields_ = [("width", _u32), ("height", _u32), ("spp", _u32), ("max_spp", _u32), ("bounce", _u32),
                ("spatial_denoise", _u32), ("enable_nee", _u32), ("rng", _u32), ("seed", _u32),
                ("debug_mode", _u32), ("kernel", _u32), ("sample_offset", _u32)]


class spk_ray(C.Structure):
    _fields_ = [("origin", _f * 3), ("direction", _f * 3)]


class spk_hit(C.Structure):
    _fields_ = [("t", _f), ("u", _f), ("v", _f), ("prim", _u32), ("face", _u32)]


class spk_stats(C.Structure):
    _fields_ = [("extension_rays", C.c_uint64), ("shadow_rays", C.c_uint64), ("paths", C.c_uint64),
                ("device_ms", _f), ("trace_kernel_ms", _f), ("trace_launches", _u32), ("kernel_launches", _u32),
                ("error_flags", _u32), ("bvh_nodes", _u32), ("bvh_bytes", C.c_uint64),
                ("node_visits", C.c_uint64), ("triangle_tests", C.c_uint64), ("graph_replays", _u32),
                ("blas_reused", _u32)]


class spk_tuning(C.Structure):
    _fields_ = [("cuda_graph", _u32), ("material_sort", _u32), ("bvh_width", _u32), ("bvh_leaf_size", _u32),
                ("extend_blocks_per_sm", _u32), ("shade_blocks_per_sm", _u32), ("batch_slots", _u32),
                ("ray_sort", _u32), ("bvh_collapse", _u32), ("bvh_builder", _u32), ("path_slots_per_pixel", _u32),
                ("shadow_stage", _u32), ("multi_frame", _u32), ("primary_packets", _u32)]


class spk_texture(C.Structure):
    _fields_ = [("width", _u32), ("height", _u32), ("srgb", _u32), ("rgba", C.POINTER(C.c_float))]


class spk_material_maps(C.Structure):
    _fields_ = [("base_color", C.c_int32), ("metallic_roughness", C.c_int32), ("emissive", C.c_int32),
                ("normal", C.c_int32)]


class spk_scene_desc(C.Structure):
    _fields_ = [("meshes", C.c_void_p), ("num_meshes", _u32), ("instances", C.c_void_p), ("num_instances", _u32),
                ("materials", C.c_void_p), ("num_materials", _u32), ("sky", C.c_void_p), ("textures", C.c_void_p),
                ("num_textures", _u32), ("maps", C.c_void_p)]


class spk_request(C.Structure):
    _fields_ = [("scene", _u32), ("width", _u32), ("height", _u32), ("spp", _u32), ("bounce", _u32),
                ("seed", _u32), ("camera", spk_camera)]


HIT_DTYPE = np.dtype([("t", "<f4"), ("u", "<f4"), ("v", "<f4"), ("prim", "<u4"), ("face", "<u4")])


def make_config(width: int, height: int, spp: int = 1, max_spp: int = 2048, bounce: int = 8,
                spatial_denoise: bool = False, enable_nee: bool = False, rng: int = SPK_RNG_XOSHIRO128P,
                seed: int = 0, kernel: int = SPK_KERNEL_AUTO, sample_offset: int = 0) -> spk_config:
    return spk_config(width, height, spp, max_spp, bounce, int(spatial_denoise), int(enable_nee), rng, seed, 0,
                      kernel, sample_offset)


def affine_inverse(m: np.ndarray) -> np.ndarray:
    """Inverse of a 3x4 affine matrix, rounded once to float32 (computed in float64)."""
    m = np.asarray(m, dtype=np.float64).reshape(3, 4)
    lin = np.linalg.inv(m[:, :3])
    t = -lin @ m[:, 3]
    return np.concatenate([lin, t[:, None]], axis=1).astype(np.float32)


@dataclass
class Mesh:
    positions: np.ndarray  # (V, 3) float32
    normals: np.ndarray    # (V, 3) float32
    indices: np.ndarray    # (F, 3) uint32
    tangents: Optional[np.ndarray] = None  # (V, 4) float32
    uvs: Optional[np.ndarray] = None       # (V, 2) float32

    def __post_init__(self):
        self.positions = np.ascontiguousarray(self.positions, dtype=np.float32).reshape(-1, 3)
        self.normals = np.ascontiguousarray(self.normals, dtype=np.float32).reshape(-1, 3)
        self.indices = np.ascontiguousarray(self.indices, dtype=np.uint32).reshape(-1, 3)
        if self.tangents is not None:
            self.tangents = np.ascontiguousarray(self.tangents, dtype=np.float32).reshape(-1, 4)
        if self.uvs is not None:
            self.uvs = np.ascontiguousarray(self.uvs, dtype=np.float32).reshape(-1, 2)

    @property
    def num_faces(self) -> int:
        return int(self.indices.shape[0])


@dataclass
class Instance:
    mesh_id: int
    material_id: int
    transform: np.ndarray = field(default_factory=lambda: np.eye(3, 4, dtype=np.float32))
    sphere: bool = False
    radius: float = 0.0

    def __post_init__(self):
        self.transform = np.asarray(self.transform, dtype=np.float32).reshape(3, 4)


@dataclass
class Material:
    base_color: tuple = (1.0, 1.0, 1.0)
    emissive: tuple = (0.0, 0.0, 0.0)
    metallic: float = 0.0
    roughness: float = 1.0
    eta: float = 0.0
    dielectric: bool = False
    # texture maps: indices into Scene.textures, -1 for none (MaterialResource's *_texture fields)
    base_color_tex: int = -1
    metallic_roughness_tex: int = -1
    emissive_tex: int = -1
    normal_tex: int = -1

    @staticmethod
    def lambertian(color):
        """LambertianMaterial: PBR with metallic 0, roughness 1 (LambertianMaterial.h:8-15)."""
        return Material(tuple(color), (0, 0, 0), 0.0, 1.0, 0.0, False)

    @staticmethod
    def metal(color, roughness):
        return Material(tuple(color), (0, 0, 0), 1.0, float(roughness), 0.0, False)

    @staticmethod
    def glass(color=(1, 1, 1), eta=1.5):
        """DieletricMaterial: roughness 0, metallic 0 (DieletricMaterial.h:10-17)."""
        return Material(tuple(color), (0, 0, 0), 0.0, 0.0, float(eta), True)

    @staticmethod
    def light(radiance):
        return Material((1, 1, 1), tuple(radiance), 0.0, 1.0, 0.0, False)


@dataclass
class Texture:
    """An Image2D's texels as float RGBA (8-bit data divided by 255), row y = v * height; `srgb` decodes
    after the bilinear filter."""
    rgba: np.ndarray  # (H, W, 4) float32
    srgb: bool = False

    def __post_init__(self):
        self.rgba = np.ascontiguousarray(self.rgba, dtype=np.float32)
        if self.rgba.ndim != 3 or self.rgba.shape[2] != 4:
            raise ValueError("texture texels must be (H, W, 4)")


@dataclass
class Sky:
    mode: int = SPK_SKY_NONE
    color: tuple = (0.0, 0.0, 0.0)
    cube: Optional[np.ndarray] = None  # (6, N, N, 4) float32


@dataclass
class Scene:
    meshes: List[Mesh]
    instances: List[Instance]
    materials: List[Material]
    sky: Sky = field(default_factory=Sky)
    name: str = "scene"
    textures: List[Texture] = field(default_factory=list)

    @property
    def num_triangles(self) -> int:
        return sum(self.meshes[i.mesh_id].num_faces for i in self.instances if not i.sphere)

    def world_bounds(self):
        lo = np.full(3, np.inf)
        hi = np.full(3, -np.inf)
        for inst in self.instances:
            m = inst.transform.astype(np.float64)
            if inst.sphere:
                c = m[:, 3]
                lo = np.minimum(lo, c - inst.radius)
                hi = np.maximum(hi, c + inst.radius)
            else:
                p = self.meshes[inst.mesh_id].positions.astype(np.float64)
                w = p @ m[:, :3].T + m[:, 3]
                lo = np.minimum(lo, w.min(0))
                hi = np.maximum(hi, w.max(0))
        return lo, hi


def _ptr(a: Optional[np.ndarray], ctype):
    if a is None:
        return C.cast(None, C.POINTER(ctype))
    return a.ctypes.data_as(C.POINTER(ctype))


def instance_array(instances):
    """spk_instance records of a list of Instance (at least one slot, so the pointer is never NULL)."""
    arr = (spk_instance * max(1, len(instances)))()
    for k, inst in enumerate(instances):
        rec = spk_instance()
        rec.type = SPK_PRIM_SPHERE if inst.sphere else SPK_PRIM_MESH
        rec.mesh_id = inst.mesh_id
        rec.material_id = inst.material_id
        rec.radius = inst.radius
        rec.transform[:] = inst.transform.reshape(-1).tolist()
        rec.inv_transform[:] = affine_inverse(inst.transform).reshape(-1).tolist()
        arr[k] = rec
    return arr


class MarshalledScene:
    """ctypes arrays for spk_set_scene / or_scene_create; keeps the numpy buffers alive."""

    def __init__(self, scene: Scene):
        self.scene = scene
        self.meshes = (spk_mesh * max(1, len(scene.meshes)))()
        for k, m in enumerate(scene.meshes):
            self.meshes[k] = spk_mesh(_ptr(m.positions, C.c_float), _ptr(m.normals, C.c_float),
                                      _ptr(m.tangents, C.c_float), _ptr(m.uvs, C.c_float),
                                      _ptr(m.indices, C.c_uint32), m.positions.shape[0], m.indices.shape[0])
        self.instances = instance_array(scene.instances)
        self.materials = (spk_material * max(1, len(scene.materials)))()
        for k, mat in enumerate(scene.materials):
            rec = spk_material()
            rec.type = SPK_MAT_DIELECTRIC if mat.dielectric else SPK_MAT_PBR
            rec.base_color[:] = list(mat.base_color)
            rec.emissive[:] = list(mat.emissive)
            rec.metallic, rec.roughness, rec.eta = mat.metallic, mat.roughness, mat.eta
            self.materials[k] = rec
        self._cube = None
        self.sky = spk_sky()
        self.sky.mode = scene.sky.mode
        self.sky.color[:] = list(scene.sky.color)
        if scene.sky.mode == SPK_SKY_CUBE:
            self._cube = np.ascontiguousarray(scene.sky.cube, dtype=np.float32)
            self.sky.cube_size = self._cube.shape[1]
            self.sky.cube_rgba = _ptr(self._cube, C.c_float)

        self.textures = (spk_texture * max(1, len(scene.textures)))()
        for k, t in enumerate(scene.textures):
            h, w, _ = t.rgba.shape
            self.textures[k] = spk_texture(w, h, 1 if t.srgb else 0, _ptr(t.rgba, C.c_float))
        self.has_maps = any(m.base_color_tex >= 0 or m.metallic_roughness_tex >= 0 or m.emissive_tex >= 0 or
                            m.normal_tex >= 0 for m in scene.materials)
        self.maps = (spk_material_maps * max(1, len(scene.materials)))()
        for k, m in enumerate(scene.materials):
            self.maps[k] = spk_material_maps(m.base_color_tex, m.metallic_roughness_tex, m.emissive_tex, m.normal_tex)

    def args(self):
        s = self.scene
        return (self.meshes, len(s.meshes), self.instances, len(s.instances), self.materials, len(s.materials),
                C.byref(self.sky))

    def desc(self) -> "spk_scene_desc":
        """spk_scene_desc of this scene (with its textures and maps)."""
        a = self.args()
        s = self.scene
        return spk_scene_desc(C.cast(a[0], C.c_void_p), a[1], C.cast(a[2], C.c_void_p), a[3], C.cast(a[4], C.c_void_p),
                              a[5], C.cast(a[6], C.c_void_p), C.cast(self.textures, C.c_void_p), len(s.textures),
                              C.cast(self.maps, C.c_void_p) if self.has_maps else None)


def rays_to_array(origins: np.ndarray, directions: np.ndarray) -> np.ndarray:
    """Packs (N,3) origins and (N,3) directions into the (N,6) float32 layout of spk_ray."""
    out = np.empty((origins.shape[0], 6), dtype=np.float32)
    out[:, :3] = origins
    out[:, 3:] = directions
    return out


def camera_from_look(position, target, world_up, vfov_rad, focus_distance, aperture_radius, exposure, width,
                     height) -> spk_camera:
    """Python copy of spk_camera_from_look (CameraRenderProxy.cpp:21-34, 113-136) for hosts without the
    library; the posture basis is rounded to float32 once, then every derived term is float32."""
    f32 = np.float32
    pos = np.asarray(position, np.float64)
    front = np.asarray(target, np.float64) - pos
    front /= np.linalg.norm(front)
    right = np.cross(front, np.asarray(world_up, np.float64))
    right /= np.linalg.norm(right)
    up = np.cross(right, front)
    pos, front, right, up = (v.astype(f32) for v in (pos, front, right, up))
    h = f32(np.tan(f32(vfov_rad) / f32(2)))
    height_fp = f32(2) * h * f32(focus_distance)
    aspect = f32(width) / f32(height)
    width_fp = aspect * height_fp
    max_u = right * width_fp
    max_v = up * height_fp
    lower_left = pos + front * f32(focus_distance) - max_u * f32(0.5) - max_v * f32(0.5)
    cam = spk_camera()
    cam.position[:] = pos.tolist()
    cam.right[:] = right.tolist()
    cam.up[:] = up.tolist()
    cam.front[:] = front.tolist()
    cam.lower_left[:] = lower_left.tolist()
    cam.max_u[:] = max_u.tolist()
    cam.max_v[:] = max_v.tolist()
    cam.aperture_radius = aperture_radius
    cam.exposure = exposure
    cam.far_plane = 1000.0
    return cam
