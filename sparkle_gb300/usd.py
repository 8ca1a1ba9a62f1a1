"""USD scene import and export in the text format (USDA), with the reference loader's conventions.

Restates Sparkle's USDLoader (libraries/source/io/scene/USDLoader.cpp) and USDExporter (USDExporter.cpp),
which go through tinyusdz (not in the reference tree). This module parses and writes USDA itself; the
binary crate format (USDC / USDZ) needs tinyusdz and is not read. What the reference does and this module
mirrors:

* Nodes (LoadNode, USDLoader.cpp:498-540): the default prim's subtree (defaultPrim, else the first root
  prim). Every Xform is a scene node whose local matrix is its xformOps (xformOp:transform / translate /
  scale / rotateX|Y|Z|XYZ|... / orient, in xformOpOrder), transposed from USD's row-vector matrices into
  column form (MatrixCast, :29-41); world = parent world x local. A Mesh prim is a component of its parent
  node: it takes the parent's world transform (its own xformOps are not read). No up-axis conversion.
* Meshes (LoadMesh, :280-350): points, faceVertexIndices (polygons fan-triangulated as tydra does),
  normals (required), primvars:st as uvs, primvars:tangents (float3 gets w = 1); without tangents each
  vertex gets cross(cross(n, a), n) with w = 1, a = GetPossibleMajorAxis(n) (Utilities.h:222-234),
  unnormalised as the reference leaves it. A mesh without a bound material is skipped.
* Materials (:352-428): a UsdPreviewSurface with opacity < 1 (not textured) is a dielectric with
  eta = ior; otherwise PBR. diffuseColor / emissiveColor / metallic / roughness are read as values when
  not connected; a connected diffuseColor becomes the base-colour texture (factor left at 1), a connected
  emissiveColor the emissive texture (emissive factor 1), connected metallic + roughness one
  metallic-roughness texture (G roughness, B metallic), a connected normal the normal map. Unauthored
  inputs take UsdPreviewSurface's defaults (diffuse 0.18, emissive 0, metallic 0, roughness 0.5,
  opacity 1, ior 1.5).
* Dome lights (LoadSkyLight, :474-496) become the sky: with a texture file (relative to the USD file) the
  cube SkyLight cooks from that map (sparkle_gb300.sky), else the gradient sky of its colour x intensity x
  2^exposure (GetLightColor, :455-458). Distant lights are not read: the CPU path ignores the
  directional light.
* Cameras (LoadCamera, :80-126; load_usda_camera): a perspective Camera prim is a component of its parent
  node, like a mesh; the last one loaded is the main camera (SetMainCamera). focalLength and
  verticalAperture are millimetres (35 and 24 when unauthored, the loader's initial values), fStop and
  focusDistance replace the defaults (f/22, 1 m) only when positive; an orthographic camera is refused (the
  reference asserts). The render attributes follow CalculateRenderAttribute (CameraComponent.cpp:120-128)
  and the posture CameraRenderProxy::OnTransformDirty (CameraRenderProxy.cpp:113-128): position = the
  node's translation, right / front / up = rows 0 / 1 / 2 of its world matrix (Transform::
  ExtractLocalBasis), focus plane from tan(vfov / 2), the frame's aspect ratio and the focus distance.

Where the reference would assert (missing normals), this module computes area-weighted vertex normals.
faceVarying / uniform / constant primvars are expanded to one vertex per face corner. The exporter writes
what USDExporter writes: a Z-up stage, one Xform (xformOp:transform) per mesh instance holding its Mesh,
materials under /_materials as UsdPreviewSurface networks with UsdUVTexture shaders, textures as PNG files
in textures/ beside the file, a gradient sky as a colour-only dome light, spheres skipped (the exporter
handles mesh primitives only) and cube skies skipped (their source map is not kept).
"""
from __future__ import annotations

import os
import re

import numpy as np

from .abi import SPK_SKY_GRADIENT, Instance, Material, Mesh, Scene, Sky, Texture, spk_camera

# --------------------------------------------------------------------------------------------------------
# Tokenizer and parser of the USDA subset.

_TOKEN = re.compile(r"""
    (?P<ws>\s+|\#[^\n]*) |
    (?P<str>"\"\"[\s\S]*?\"\"\"|"(?:[^"\\]|\\.)*"|'(?:[^'\\]|\\.)*') |
    (?P<asset>@[^@]*@) |
    (?P<path></?[^<>]*>) |
    (?P<num>[-+]?(?:\d+\.?\d*(?:[eE][-+]?\d+)?|\.\d+(?:[eE][-+]?\d+)?|inf|nan)(?![A-Za-z_:])) |
    (?P<ident>[A-Za-z_][A-Za-z0-9_:.\[\]]*(?:\[\])?) |
    (?P<punct>[()\[\]{}=,;:])
""", re.VERBOSE)


class UsdError(ValueError):
    pass


def _tokens(text):
    pos = 0
    out = []
    n = len(text)
    while pos < n:
        m = _TOKEN.match(text, pos)
        if not m:
            raise UsdError(f"unexpected character {text[pos]!r} at offset {pos}")
        kind = m.lastgroup
        if kind != "ws":
            out.append((kind, m.group(kind)))
        pos = m.end()
    return out


class _Prim:
    def __init__(self, spec, type_name, name):
        self.spec, self.type, self.name = spec, type_name, name
        self.attrs = {}   # name -> value
        self.meta = {}    # attribute name -> its metadata dict
        self.conns = {}   # attribute name -> connection target path
        self.rels = {}    # relationship name -> target path(s)
        self.children = []
        self.prim_meta = {}


class _Parser:
    def __init__(self, toks):
        self.t, self.i = toks, 0

    def peek(self, k=0):
        j = self.i + k
        return self.t[j] if j < len(self.t) else (None, None)

    def take(self, value=None):
        tok = self.peek()
        if tok[0] is None:
            raise UsdError("unexpected end of file")
        if value is not None and tok[1] != value:
            raise UsdError(f"expected {value!r}, found {tok[1]!r}")
        self.i += 1
        return tok

    def value(self):
        kind, v = self.peek()
        if v == "{":
            return self._braces()
        if v == "(":
            self.take("(")
            items = []
            while self.peek()[1] != ")":
                items.append(self.value())
                if self.peek()[1] == ",":
                    self.take(",")
            self.take(")")
            return tuple(items)
        if v == "[":
            self.take("[")
            items = []
            while self.peek()[1] != "]":
                items.append(self.value())
                if self.peek()[1] == ",":
                    self.take(",")
            self.take("]")
            return items
        self.take()
        if kind == "num":
            return float(v)
        if kind == "str":
            return v[3:-3] if v.startswith('"""') else v[1:-1]
        if kind == "asset":
            return ("@", v[1:-1])
        if kind == "path":
            return ("<", v[1:-1])
        if kind == "ident":
            return {"true": True, "false": False, "None": None}.get(v, v)
        raise UsdError(f"unexpected {v!r}")

    def metadata(self):
        """( key = value ... ) -> dict (bare strings such as doc comments are skipped)."""
        out = {}
        self.take("(")
        while self.peek()[1] != ")":
            kind, v = self.peek()
            if kind == "str":
                self.take()
                continue
            if v in ("prepend", "append", "add", "delete", "reorder"):
                self.take()
            key = self.take()[1]
            if self.peek()[1] == "=":
                self.take("=")
                out[key] = self.value()
            if self.peek()[1] in (",", ";"):
                self.take()
        self.take(")")
        return out

    def layer(self):
        if self.peek()[1] == "(":
            layer_meta = self.metadata()
        else:
            layer_meta = {}
        roots = []
        while self.peek()[0] is not None:
            roots.append(self.prim())
        return layer_meta, roots

    def prim(self):
        spec = self.take()[1]
        if spec not in ("def", "over", "class"):
            raise UsdError(f"expected a prim specifier, found {spec!r}")
        type_name = ""
        if self.peek()[0] == "ident":
            type_name = self.take()[1]
        name = self.value()
        if not isinstance(name, str):
            raise UsdError("prim name must be a string")
        p = _Prim(spec, type_name, name)
        if self.peek()[1] == "(":
            p.prim_meta = self.metadata()
        self.take("{")
        while self.peek()[1] != "}":
            kind, v = self.peek()
            if v in ("def", "over", "class"):
                p.children.append(self.prim())
            elif v == "variantSet":
                self._skip_block()
            else:
                self.property(p)
        self.take("}")
        return p

    def _braces(self):
        """{ time: value, ... } (timeSamples: the earliest sample) or a dictionary (skipped, None)."""
        self.take("{")
        if self.peek()[0] == "num" and self.peek(1)[1] == ":":
            samples = {}
            while self.peek()[1] != "}":
                t = float(self.take()[1])
                self.take(":")
                samples[t] = self.value()
                if self.peek()[1] == ",":
                    self.take(",")
            self.take("}")
            return samples[min(samples)] if samples else None
        depth = 1
        while depth:
            v = self.take()[1]
            depth += {"{": 1, "}": -1}.get(v, 0)
        return None

    def _skip_block(self):
        while self.peek()[1] != "{":
            self.take()
        depth = 0
        while True:
            v = self.take()[1]
            if v == "{":
                depth += 1
            elif v == "}":
                depth -= 1
                if depth == 0:
                    return

    _QUALIFIERS = ("custom", "uniform", "varying", "config", "prepend", "append", "add", "delete", "reorder")

    def property(self, p):
        """[qualifiers] type name [= value] [(metadata)], or rel name [= target(s)] [(metadata)]."""
        while self.peek()[0] == "ident" and self.peek()[1] in self._QUALIFIERS:
            self.take()
        kind, first = self.take()
        if kind != "ident":
            raise UsdError(f"unexpected {first!r} in prim {p.name!r}")
        kind, name = self.take()
        if kind != "ident":
            raise UsdError(f"expected a property name after {first!r} in prim {p.name!r}")
        value = None
        if self.peek()[1] == "=":
            self.take("=")
            value = self.value()
        meta = self.metadata() if self.peek()[1] == "(" else {}
        if first == "rel":
            p.rels[name] = value
        elif name.endswith(".connect"):
            p.conns[name[:-len(".connect")]] = value[0] if isinstance(value, list) and value else value
        elif name.endswith(".timeSamples"):
            p.attrs.setdefault(name[:-len(".timeSamples")], value)
        else:
            p.attrs[name] = value
            if meta:
                p.meta[name] = meta


def _parse(text):
    if not text.lstrip().startswith("#usda"):
        raise UsdError("not a USDA file (binary USDC / USDZ need tinyusdz)")
    return _Parser(_tokens(text)).layer()


# --------------------------------------------------------------------------------------------------------
# Import.

def _rot(axis, deg):
    a = np.deg2rad(deg)
    c, s = np.cos(a), np.sin(a)
    m = np.eye(4)
    i, j = {"X": (1, 2), "Y": (2, 0), "Z": (0, 1)}[axis]
    m[i, i], m[i, j], m[j, i], m[j, j] = c, -s, s, c
    return m


def _local_matrix(p):
    """Column-convention 4x4 of a prim's xformOps (xformOpOrder [A, B, C]: A @ B @ C)."""
    order = p.attrs.get("xformOpOrder") or []
    m = np.eye(4)
    for op in order:
        if op == "!resetXformStack!":
            continue
        inverse = op.startswith("!invert!")
        name = op[len("!invert!"):] if inverse else op
        v = p.attrs.get(name)
        kind = name.split(":")[1]
        if kind == "transform":
            o = np.array(v, np.float64).reshape(4, 4).T  # USD rows are row vectors (MatrixCast transposes)
        elif kind == "translate":
            o = np.eye(4)
            o[:3, 3] = v
        elif kind == "scale":
            o = np.diag([*(v if isinstance(v, tuple) else (v, v, v)), 1.0])
        elif kind == "orient":
            w, x, y, z = v  # quatf values are (real, i, j, k)
            o = np.eye(4)
            o[:3, :3] = [[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                         [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                         [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]]
        elif kind.startswith("rotate"):
            axes = kind[len("rotate"):]
            vals = v if isinstance(v, tuple) else (v,)
            o = np.eye(4)
            for ax, deg in zip(axes, vals):  # rotateXYZ: X applied first
                o = _rot(ax, deg) @ o
        else:
            raise UsdError(f"unsupported xformOp {name!r}")
        m = m @ (np.linalg.inv(o) if inverse else o)
    return m


def _interp(p, name):
    return (p.meta.get(name) or {}).get("interpolation", "vertex")


def _expand(values, interp, counts, indices, nfaces):
    """Per face corner values of a primvar (corner order = faceVertexIndices order)."""
    if interp in ("vertex", "varying"):
        return values[indices]
    if interp == "faceVarying":
        return values
    if interp == "uniform":
        return np.repeat(values, counts, axis=0)
    if interp == "constant":
        return np.repeat(values[:1], len(indices), axis=0)
    raise UsdError(f"unsupported interpolation {interp!r}")


def _major_axis(n):
    """GetPossibleMajorAxis (Utilities.h:222-234): Right, Front or Up."""
    inv_sqrt3 = np.float32(1.0 / np.sqrt(3.0))
    out = np.zeros_like(n)
    ax = np.abs(n[:, 0]) < inv_sqrt3
    ay = ~ax & (np.abs(n[:, 1]) < inv_sqrt3)
    out[ax, 0] = 1
    out[ay, 1] = 1
    out[~ax & ~ay, 2] = 1
    return out


def _load_mesh(p, prims_by_path, base_dir, textures, tex_cache, mat_cache, materials):
    binding = p.rels.get("material:binding")
    if isinstance(binding, list):
        binding = binding[0] if binding else None
    if not binding or binding[1] not in prims_by_path:
        return None, None  # the reference skips meshes without a material (USDLoader.cpp:282-286)
    mat_id = _load_material(prims_by_path[binding[1]], prims_by_path, base_dir, textures, tex_cache, mat_cache,
                            materials)
    pts = np.asarray(p.attrs.get("points") or [], np.float32).reshape(-1, 3)
    counts = np.asarray(p.attrs.get("faceVertexCounts") or [], np.int64)
    idx = np.asarray(p.attrs.get("faceVertexIndices") or [], np.int64)
    if counts.sum() != len(idx) or (len(idx) and (idx.min() < 0 or idx.max() >= len(pts))):
        raise UsdError(f"mesh {p.name!r}: inconsistent faceVertexCounts / faceVertexIndices")
    attrs = {}
    for key, width in (("normals", 3), ("primvars:normals", 3), ("primvars:st", 2), ("primvars:tangents", 0)):
        if p.attrs.get(key) is None:
            continue
        vals = np.asarray(p.attrs[key], np.float32)
        vals = vals.reshape(len(vals), -1) if vals.ndim > 1 else vals.reshape(-1, width or 4)
        ind = p.attrs.get(key + ":indices")
        if ind is not None:
            vals = vals[np.asarray(ind, np.int64)]
        attrs[key] = (vals, _interp(p, key))
    if "primvars:normals" in attrs:
        attrs["normals"] = attrs.pop("primvars:normals")
    per_vertex = all(i in ("vertex", "varying") for _, i in attrs.values())
    nfaces = len(counts)
    # Fan triangulation of every polygon in corner indices.
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.int64) if nfaces else np.zeros(0, np.int64)
    tri = [np.stack([np.full(c - 2, s), s + np.arange(1, c - 1), s + np.arange(2, c)], 1)
           for s, c in zip(starts, counts) if c >= 3]
    corners = np.concatenate(tri).astype(np.int64) if tri else np.zeros((0, 3), np.int64)
    if per_vertex:
        positions = pts
        faces = idx[corners]
        expanded = {k: v for k, (v, _) in attrs.items()}
    else:
        positions = pts[idx]
        faces = corners
        expanded = {k: _expand(v, i, counts, idx, nfaces) for k, (v, i) in attrs.items()}
    normals = expanded.get("normals")
    if normals is None:
        normals = _vertex_normals(positions, faces)
    uvs = expanded.get("primvars:st")
    tangents = expanded.get("primvars:tangents")
    if tangents is not None and tangents.shape[1] == 3:
        tangents = np.concatenate([tangents, np.ones((len(tangents), 1), np.float32)], 1)
    if tangents is None:
        n = normals.astype(np.float32)
        tangents = np.concatenate([np.cross(np.cross(n, _major_axis(n)), n), np.ones((len(n), 1), np.float32)], 1)
    mesh = Mesh(positions, normals, faces.astype(np.uint32), tangents=tangents.astype(np.float32),
                uvs=None if uvs is None else uvs.astype(np.float32))
    return mesh, mat_id


def _vertex_normals(pos, faces):
    n = np.zeros_like(pos, dtype=np.float64)
    if len(faces):
        fn = np.cross(pos[faces[:, 1]] - pos[faces[:, 0]], pos[faces[:, 2]] - pos[faces[:, 0]])
        for c in range(3):
            np.add.at(n, faces[:, c], fn)
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    return np.where(ln > 0, n / np.where(ln > 0, ln, 1), [0, 0, 1]).astype(np.float32)


_PREVIEW_DEFAULTS = {"diffuseColor": (0.18, 0.18, 0.18), "emissiveColor": (0.0, 0.0, 0.0), "metallic": 0.0,
                     "roughness": 0.5, "opacity": 1.0, "ior": 1.5}


def _surface_shader(mat, prims_by_path):
    target = mat.conns.get("outputs:surface")
    if target:
        path = target[1].split(".")[0]
        if path in prims_by_path:
            return prims_by_path[path]
    for c in mat.children:
        if c.attrs.get("info:id") == "UsdPreviewSurface":
            return c
    return None


def _load_texture(shader_path, prims_by_path, base_dir, srgb, textures, tex_cache):
    from .gltf import decode_image
    tex = prims_by_path.get(shader_path)
    if tex is None or tex.attrs.get("info:id") != "UsdUVTexture":
        raise UsdError(f"input connected to {shader_path!r}, which is not a UsdUVTexture")
    asset = tex.attrs.get("inputs:file")
    if not asset:
        raise UsdError(f"texture {shader_path!r} has no inputs:file")
    file = os.path.normpath(os.path.join(base_dir, asset[1]))
    key = (file, srgb)
    if key not in tex_cache:
        with open(file, "rb") as f:
            rgba = decode_image(f.read())
        tex_cache[key] = len(textures)
        textures.append(Texture(rgba, srgb=srgb))
    return tex_cache[key]


def _load_material(mat, prims_by_path, base_dir, textures, tex_cache, mat_cache, materials):
    key = id(mat)
    if key in mat_cache:
        return mat_cache[key]
    m = Material((1.0, 1.0, 1.0), (0.0, 0.0, 0.0), 1.0, 1.0)  # MaterialResource defaults (io/Material.h:9-14)
    shader = _surface_shader(mat, prims_by_path)
    dielectric, eta = False, 0.0
    if shader is not None:
        def value(name):
            v = shader.attrs.get("inputs:" + name)
            return _PREVIEW_DEFAULTS[name] if v is None else v

        def connected(name):
            c = shader.conns.get("inputs:" + name)
            return None if c is None else c[1].split(".")[0]

        dielectric = connected("opacity") is None and float(value("opacity")) < 1.0
        if connected("diffuseColor"):
            m.base_color_tex = _load_texture(connected("diffuseColor"), prims_by_path, base_dir, True, textures,
                                             tex_cache)
        else:
            m.base_color = tuple(float(x) for x in value("diffuseColor"))
        if connected("emissiveColor"):
            m.emissive_tex = _load_texture(connected("emissiveColor"), prims_by_path, base_dir, True, textures,
                                           tex_cache)
            m.emissive = (1.0, 1.0, 1.0)
        else:
            m.emissive = tuple(float(x) for x in value("emissiveColor"))
        if connected("normal"):
            m.normal_tex = _load_texture(connected("normal"), prims_by_path, base_dir, False, textures, tex_cache)
        if connected("metallic"):
            if connected("roughness") != connected("metallic"):
                raise UsdError("metallic and roughness must read one packed texture")
            m.metallic_roughness_tex = _load_texture(connected("metallic"), prims_by_path, base_dir, False, textures,
                                                     tex_cache)
        else:
            m.metallic = float(value("metallic"))
            m.roughness = float(value("roughness"))
        eta = float(value("ior"))
    if dielectric:
        m.dielectric = True
        m.eta = eta
    else:
        m.eta = 0.0
    mat_cache[key] = len(materials)
    materials.append(m)
    return mat_cache[key]


def _index(prims, prefix=""):
    out = {}
    for p in prims:
        path = f"{prefix}/{p.name}"
        out[path] = p
        out.update(_index(p.children, path))
    return out


def _dome_sky(p, base_dir, sky_size):
    def get(*names, default=None):
        for n in names:
            if p.attrs.get(n) is not None:
                return p.attrs[n]
        return default
    tex = get("inputs:texture:file", "texture:file")
    if tex:
        from .sky import sky_from_file
        return sky_from_file(os.path.normpath(os.path.join(base_dir, tex[1])), sky_size)
    color = np.asarray(get("inputs:color", "color", default=(1.0, 1.0, 1.0)), np.float32)
    scale = np.float32(get("inputs:intensity", "intensity", default=1.0)) * np.float32(
        2.0 ** float(get("inputs:exposure", "exposure", default=0.0)))
    return Sky(SPK_SKY_GRADIENT, tuple(float(x) for x in color * scale), None)


def load_usda(path, sky: Sky = None, sky_size: int = 1024) -> Scene:
    """Scene (meshes, instances, materials, textures, sky) of a USDA file. The first dome light of the
    default prim's subtree gives the sky unless `sky` is given; a textured dome light's cube has
    sky_size x sky_size faces (the reference cooks 1024)."""
    with open(path, "r", encoding="utf-8") as f:
        layer_meta, roots = _parse(f.read())
    roots = [r for r in roots if r.spec == "def"]
    prims_by_path = _index(roots)
    default = layer_meta.get("defaultPrim")
    root = next((r for r in roots if r.name == default), roots[0] if roots else None)
    meshes, instances, materials, textures = [], [], [], []
    tex_cache, mat_cache = {}, {}
    base_dir = os.path.dirname(os.path.abspath(path))
    domes = []

    def walk(node, parent_world):
        world = parent_world @ _local_matrix(node)
        for c in node.children:
            if c.spec != "def":
                continue
            if c.type == "Xform" or c.type == "":
                walk(c, world)
            elif c.type == "DomeLight":
                domes.append(c)
            elif c.type == "Mesh":
                mesh, mat_id = _load_mesh(c, prims_by_path, base_dir, textures, tex_cache, mat_cache, materials)
                if mesh is not None:
                    meshes.append(mesh)
                    instances.append(Instance(len(meshes) - 1, mat_id, world[:3].astype(np.float32)))

    if root is not None:
        walk(root, np.eye(4))
    if sky is None:
        sky = _dome_sky(domes[0], base_dir, sky_size) if domes else Sky()
    return Scene(meshes, instances, materials, sky, name=os.path.basename(path), textures=textures)


def _camera_prims(root):
    """(Camera prim, its parent node's world matrix) in LoadNode's traversal order."""
    out = []

    def walk(node, parent_world):
        world = parent_world @ _local_matrix(node)
        for c in node.children:
            if c.spec != "def":
                continue
            if c.type == "Xform" or c.type == "":
                walk(c, world)
            elif c.type == "Camera":
                out.append((c, world))

    walk(root, np.eye(4))
    return out


def load_usda_camera(path, width: int, height: int):
    """The main camera of a USDA file (the last Camera prim loaded) as an spk_camera for a width x height
    frame, or None when the file has no camera. Float32 arithmetic in the reference's order."""
    with open(path, "r", encoding="utf-8") as f:
        layer_meta, roots = _parse(f.read())
    roots = [r for r in roots if r.spec == "def"]
    default = layer_meta.get("defaultPrim")
    root = next((r for r in roots if r.name == default), roots[0] if roots else None)
    cams = _camera_prims(root) if root is not None else []
    if not cams:
        return None
    prim, world = cams[-1]
    if (prim.attrs.get("projection") or "perspective") != "perspective":
        raise UsdError(f"camera {prim.name!r}: only perspective cameras are supported")
    f32 = np.float32

    def scalar(name, default):
        v = prim.attrs.get(name)
        return f32(default if v is None else v)

    focal = scalar("focalLength", 35.0) * f32(0.001)
    sensor = scalar("verticalAperture", 24.0) * f32(0.001)
    f_stop, focus = scalar("fStop", 0.0), scalar("focusDistance", 0.0)
    aperture = f_stop if f_stop > 0 else f32(22.0)
    fd = focus if focus > 0 else f32(1.0)
    vfov = f32(2.0) * f32(np.arctan(sensor / (f32(2.0) * focal)))
    m = world.astype(np.float32)
    position = m[:3, 3]
    right, front, up = m[0, :3], m[1, :3], m[2, :3]
    aspect = f32(width) / f32(height)
    plane_h = f32(2.0) * f32(np.tan(vfov / f32(2.0))) * fd
    plane_w = aspect * plane_h
    max_u, max_v = right * plane_w, up * plane_h
    lower_left = position + front * fd - max_u * f32(0.5) - max_v * f32(0.5)
    cam = spk_camera()
    for name, v in (("position", position), ("right", right), ("up", up), ("front", front),
                    ("lower_left", lower_left), ("max_u", max_u), ("max_v", max_v)):
        getattr(cam, name)[:] = [float(x) for x in v]
    cam.aperture_radius = float(focal / aperture * f32(0.5))
    cam.exposure = 1.0
    cam.far_plane = 1000.0
    return cam


# --------------------------------------------------------------------------------------------------------
# Export.

def _valid_name(name):
    """MakeValidPrimName (USDExporter.cpp:29-52): [A-Za-z_][A-Za-z0-9_]*."""
    name = re.sub(r"[^A-Za-z0-9_]", "_", name or "prim")
    return "_" + name if name[0].isdigit() else name


def _f(x):
    return repr(float(x))


def _vec_array(a):
    return "[" + ", ".join("(" + ", ".join(_f(x) for x in row) + ")" for row in np.asarray(a)) + "]"


def _matrix(m4):
    rows = np.asarray(m4, np.float64).T  # column form -> USD rows
    return "( " + ", ".join("(" + ", ".join(_f(x) for x in r) + ")" for r in rows) + " )"


def _camera_lines(cam):
    """ExportCamera (USDExporter.cpp:392-406) of an spk_camera under an Xform holding its posture: the node
    matrix has rows right / front / up and the position as translation (what load_usda_camera reads back),
    the lens is the 24 mm sensor of CameraComponent's defaults with the focal length, f-stop and focus
    distance that reproduce the camera's focus plane and aperture radius (fStop 0, unauthored, for a
    pinhole camera: it reads back as f/22, the reference's default)."""
    f64 = lambda name: np.array(getattr(cam, name), np.float64)
    pos, right, front, up = f64("position"), f64("right"), f64("front"), f64("up")
    max_u, max_v, ll = f64("max_u"), f64("max_v"), f64("lower_left")
    plane_h = np.linalg.norm(max_v) / np.linalg.norm(up)
    fd = np.linalg.norm(ll + max_u * 0.5 + max_v * 0.5 - pos) / np.linalg.norm(front)
    sensor = 0.024
    focal = sensor * fd / plane_h  # tan(vfov / 2) = plane_h / (2 fd) = sensor / (2 focal)
    f_stop = focal / (2.0 * cam.aperture_radius) if cam.aperture_radius > 0 else 0.0
    node = np.eye(4)
    node[0, :3], node[1, :3], node[2, :3], node[:3, 3] = right, front, up, pos
    return ['    def Xform "camera_node"', "    {", f"        matrix4d xformOp:transform = {_matrix(node)}",
            '        uniform token[] xformOpOrder = ["xformOp:transform"]', '        def Camera "camera"', "        {",
            '            token projection = "perspective"', f"            float focalLength = {_f(focal * 1000.0)}",
            f"            float verticalAperture = {_f(sensor * 1000.0)}", f"            float fStop = {_f(f_stop)}",
            f"            float focusDistance = {_f(fd)}", "        }", "    }"]


def save_usda(scene: Scene, path, camera=None) -> None:
    """USDExporter::Export of a Scene: Z-up stage, one Xform per mesh instance, materials under /_materials,
    textures as PNG files in textures/ beside `path`; with `camera` (an spk_camera) also the camera."""
    from .native import write_png
    if not str(path).endswith(".usda"):
        raise UsdError("only .usda output is supported")
    out_dir = os.path.dirname(os.path.abspath(path))
    os.makedirs(os.path.join(out_dir, "textures"), exist_ok=True)
    tex_files = {}

    def texture_file(k):
        if k not in tex_files:
            t = scene.textures[k]
            rel = f"textures/{len(tex_files)}_texture_{k}.png"
            img = np.clip(np.rint(np.asarray(t.rgba, np.float64) * 255.0), 0, 255).astype(np.uint8)
            write_png(os.path.join(out_dir, rel), img)
            tex_files[k] = rel
        return tex_files[k]

    lines = ["#usda 1.0", "(", '    defaultPrim = "root"', "    metersPerUnit = 1", '    upAxis = "Z"', ")", "",
             'def Xform "root"', "{", f"    matrix4d xformOp:transform = {_matrix(np.eye(4))}",
             '    uniform token[] xformOpOrder = ["xformOp:transform"]']
    mat_lines, mat_names = [], {}

    def material_path(mid):
        if mid in mat_names:
            return mat_names[mid]
        m = scene.materials[mid]
        name = f"material_{len(mat_names)}"
        mp = f"/_materials/{name}"
        body = [f'    def Material "{name}"', "    {", f"        token outputs:surface.connect = <{mp}/surface.outputs:surface>",
                '        def Shader "st_reader"', "        {", '            uniform token info:id = "UsdPrimvarReader_float2"',
                '            string inputs:varname = "st"', "            float2 outputs:result", "        }"]
        surf = ['        def Shader "surface"', "        {", '            uniform token info:id = "UsdPreviewSurface"',
                "            int inputs:useSpecularWorkflow = 0"]

        def tex_shader(shader, k, srgb):
            body.extend([f'        def Shader "{shader}"', "        {", '            uniform token info:id = "UsdUVTexture"',
                         f"            asset inputs:file = @{texture_file(k)}@",
                         f'            token inputs:sourceColorSpace = "{"sRGB" if srgb else "raw"}"',
                         '            token inputs:wrapS = "repeat"', '            token inputs:wrapT = "repeat"',
                         f"            float2 inputs:st.connect = <{mp}/st_reader.outputs:result>",
                         "            float3 outputs:rgb", "            float outputs:g", "            float outputs:b", "        }"])
            return f"{mp}/{shader}"

        if m.base_color_tex >= 0:
            surf.append(f"            color3f inputs:diffuseColor.connect = <{tex_shader('base_color_tex', m.base_color_tex, True)}.outputs:rgb>")
        else:
            surf.append(f"            color3f inputs:diffuseColor = ({', '.join(_f(x) for x in m.base_color)})")
        if m.emissive_tex >= 0:
            surf.append(f"            color3f inputs:emissiveColor.connect = <{tex_shader('emissive_tex', m.emissive_tex, True)}.outputs:rgb>")
        else:
            surf.append(f"            color3f inputs:emissiveColor = ({', '.join(_f(x) for x in m.emissive)})")
        if m.normal_tex >= 0:
            surf.append(f"            normal3f inputs:normal.connect = <{tex_shader('normal_tex', m.normal_tex, False)}.outputs:rgb>")
        if m.metallic_roughness_tex >= 0:
            tp = tex_shader("metallic_roughness_tex", m.metallic_roughness_tex, False)
            surf.append(f"            float inputs:metallic.connect = <{tp}.outputs:b>")
            surf.append(f"            float inputs:roughness.connect = <{tp}.outputs:g>")
        else:
            surf.append(f"            float inputs:metallic = {_f(m.metallic)}")
            surf.append(f"            float inputs:roughness = {_f(m.roughness)}")
        if m.dielectric:  # transmissive: the loader maps opacity < 1 back to a dielectric
            surf.append("            float inputs:opacity = 0")
            surf.append(f"            float inputs:ior = {_f(m.eta)}")
        surf.extend(["            token outputs:surface", "        }"])
        mat_lines.extend(body + surf + ["    }"])
        mat_names[mid] = mp
        return mp

    if scene.sky is not None and scene.sky.mode == SPK_SKY_GRADIENT:  # procedural: a colour-only dome light
        lines += ['    def DomeLight "sky"', "    {", f"        color3f inputs:color = ({', '.join(_f(x) for x in scene.sky.color)})",
                  "        float inputs:intensity = 1", "    }"]
    for k, inst in enumerate(scene.instances):
        if inst.sphere:
            continue  # the exporter writes mesh primitives only
        mesh = scene.meshes[inst.mesh_id]
        world = np.eye(4)
        world[:3] = inst.transform
        lines += [f'    def Xform "node_{k}"', "    {", f"        matrix4d xformOp:transform = {_matrix(world)}",
                  '        uniform token[] xformOpOrder = ["xformOp:transform"]', f'        def Mesh "mesh_{k}"', "        {",
                  f"            int[] faceVertexCounts = [{', '.join(['3'] * mesh.num_faces)}]",
                  f"            int[] faceVertexIndices = [{', '.join(str(int(i)) for i in mesh.indices.reshape(-1))}]",
                  f"            normal3f[] normals = {_vec_array(mesh.normals)} (", '                interpolation = "vertex"',
                  "            )", f"            point3f[] points = {_vec_array(mesh.positions)}"]
        if mesh.uvs is not None:
            lines += [f"            texCoord2f[] primvars:st = {_vec_array(mesh.uvs)} (", '                interpolation = "vertex"',
                      "            )"]
        if mesh.tangents is not None:
            lines += [f"            float4[] primvars:tangents = {_vec_array(mesh.tangents)} (",
                      '                interpolation = "vertex"', "            )"]
        lines += [f"            rel material:binding = <{material_path(inst.material_id)}>", "        }", "    }"]
    if camera is not None:
        lines += _camera_lines(camera)
    lines.append("}")
    if mat_lines:
        lines += ["", 'def Scope "_materials"', "{"] + mat_lines + ["}"]
    with open(path, "w", encoding="utf-8") as f:
        f.write("\n".join(lines) + "\n")
