"""glTF 2.0 scene import into the path tracer's scene structs, with the reference loader's conventions.

Restates Sparkle's GLTFLoader (libraries/source/io/scene/GLTFLoader.cpp), which reads the file with
tinygltf (not in the reference tree); this module parses the glTF JSON, buffers and accessors itself.
What the reference does and this module mirrors:

* Materials (LoadMaterials, GLTFLoader.cpp:475-526): a factor is read only when its texture is present --
  base colour with baseColorTexture, metallic/roughness with metallicRoughnessTexture, emissive with
  emissiveTexture -- otherwise MaterialResource's defaults apply (base colour 1, emissive 0, metallic 1,
  roughness 1; io/Material.h:9-14). Textures (PNG or baseline JPEG images, embedded or external) become Scene textures:
  base colour and emissive as sRGB, metallic-roughness and normal maps as linear data.
* Nodes (ProcessNode, GLTFLoader.cpp:528-575): rotation = 90 degrees about +X times the node's quaternion
  (glTF is y-up, Sparkle z-up), applied at every node including children; the node's scale is baked into
  its vertex positions only (LoadPositionArray, :192-230) and the node transform keeps scale 1; local =
  translation * rotation (Transform.cpp:52-60), world = parent world * local (SceneNode.cpp:30-42). A
  node's `matrix` is ignored (only translation / rotation / scale are read).
* Primitives (LoadPrimitive, :329-473): triangle lists, fans and strips (fans and strips expanded to lists),
  POSITION / NORMAL / TANGENT / TEXCOORD_0; points and lines are skipped; one mesh instance per primitive
  with the primitive's material.
* Scenes (Load, :577-645): the default scene's root nodes (scene 0 without a default); a file without
  scenes treats every node as a root.

Where the reference would assert or read out of range, this module makes a choice and says so: a
primitive without indices gets 0..n-1, one without a material gets the default material, one without
normals gets area-weighted vertex normals.
"""
from __future__ import annotations

import base64
import json
import os
import struct
import zlib

import numpy as np

from .abi import Instance, Material, Mesh, Scene, Sky, Texture

_COMPONENT = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5126: np.float32}
_NCOMP = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT2": 4, "MAT3": 9, "MAT4": 16}
MODE_TRIANGLES, MODE_STRIP, MODE_FAN = 4, 5, 6


def _read_container(path: str):
    data = open(path, "rb").read()
    if data[:4] == b"glTF":  # binary container: header, JSON chunk, optional BIN chunk
        _, _, length = struct.unpack_from("<III", data, 0)
        off, doc, bin_chunk = 12, None, None
        while off < length:
            clen, ctype = struct.unpack_from("<II", data, off)
            chunk = data[off + 8:off + 8 + clen]
            if ctype == 0x4E4F534A:
                doc = json.loads(chunk.decode("utf-8"))
            elif ctype == 0x004E4942:
                bin_chunk = chunk
            off += 8 + clen
        return doc, bin_chunk
    return json.loads(data.decode("utf-8")), None


def _buffers(doc, base_dir, bin_chunk):
    out = []
    for k, b in enumerate(doc.get("buffers", [])):
        uri = b.get("uri")
        if uri is None:
            out.append(bin_chunk if k == 0 and bin_chunk is not None else b"")
        elif uri.startswith("data:"):
            out.append(base64.b64decode(uri.split(",", 1)[1]))
        else:
            out.append(open(os.path.join(base_dir, uri), "rb").read())
    return out


def _accessor(doc, buffers, index):
    acc = doc["accessors"][index]
    dtype = np.dtype(_COMPONENT[acc["componentType"]])
    ncomp = _NCOMP[acc["type"]]
    count = acc["count"]
    if "bufferView" not in acc:  # all zeros (sparse accessors are not supported)
        return np.zeros((count, ncomp), dtype)
    view = doc["bufferViews"][acc["bufferView"]]
    buf = buffers[view["buffer"]]
    start = view.get("byteOffset", 0) + acc.get("byteOffset", 0)
    elem = dtype.itemsize * ncomp
    stride = view.get("byteStride", elem) or elem
    raw = np.frombuffer(buf, np.uint8, count=(count - 1) * stride + elem if count else 0, offset=start)
    if stride == elem:
        arr = raw.view(dtype).reshape(count, ncomp)
    else:
        rows = np.lib.stride_tricks.as_strided(raw, shape=(count, elem), strides=(stride, 1))
        arr = np.ascontiguousarray(rows).view(dtype).reshape(count, ncomp)
    return arr.copy()


def _unfilter(raw: np.ndarray, h: int, stride: int, bpp: int) -> np.ndarray:
    """Undoes the PNG row filters (None, Sub, Up, Average, Paeth; bpp = bytes per complete pixel, at least
    1). None / Sub / Up rows are vectorised (Sub is a running sum mod 256 per byte lane); Average and Paeth
    depend on the reconstructed byte to the left and run as a plain loop over the row."""
    out = np.zeros((h, stride), np.uint8)
    prev = np.zeros(stride, np.uint8)
    for y in range(h):
        f, line = int(raw[y, 0]), raw[y, 1:]
        if f == 0:
            cur = line.copy()
        elif f == 1:
            pad = (-stride) % bpp
            lanes = np.concatenate([line, np.zeros(pad, np.uint8)]).reshape(-1, bpp).astype(np.uint32)
            cur = (np.cumsum(lanes, axis=0) & 0xFF).astype(np.uint8).reshape(-1)[:stride]
        elif f == 2:
            cur = (line.astype(np.uint16) + prev).astype(np.uint8)
        elif f in (3, 4):
            ln, pv = line.tolist(), prev.tolist()
            cb = [0] * stride
            if f == 3:
                for x in range(stride):
                    left = cb[x - bpp] if x >= bpp else 0
                    cb[x] = (ln[x] + ((left + pv[x]) >> 1)) & 0xFF
            else:
                for x in range(stride):
                    if x >= bpp:
                        a_, c_ = cb[x - bpp], pv[x - bpp]
                    else:
                        a_ = c_ = 0
                    b_ = pv[x]
                    pa, pb, pc = abs(b_ - c_), abs(a_ - c_), abs(a_ + b_ - 2 * c_)
                    pred = a_ if pa <= pb and pa <= pc else (b_ if pb <= pc else c_)
                    cb[x] = (ln[x] + pred) & 0xFF
            cur = np.array(cb, np.uint8)
        else:
            raise ValueError(f"bad PNG filter type {f}")
        out[y] = cur
        prev = cur
    return out


def _png_samples(rows: np.ndarray, w: int, h: int, ch: int, depth: int, ctype: int) -> np.ndarray:
    """Unfiltered scanlines -> (h, w, ch) uint8 samples (16-bit: high byte; 1/2/4-bit grey scaled to 8 bits,
    palette indices as they are)."""
    stride = rows.shape[1]
    if depth == 16:
        samples = rows.reshape(h, w * ch, 2)[..., 0]  # high byte of each big-endian sample
    elif depth == 8:
        samples = rows.reshape(h, w * ch)
    else:  # 1, 2 or 4 bits, one channel: unpack MSB first
        per = 8 // depth
        shifts = np.arange(per - 1, -1, -1, dtype=np.uint8) * depth
        unpacked = (rows[:, :, None] >> shifts) & ((1 << depth) - 1)
        samples = unpacked.reshape(h, stride * per)[:, :w]
        if ctype == 0:  # grey scaled to 8 bits
            samples = (samples.astype(np.uint32) * (255 // ((1 << depth) - 1))).astype(np.uint8)
    return samples.reshape(h, w, ch)


# Adam7 passes: (first column, first row, column step, row step).
_ADAM7 = ((0, 0, 8, 8), (4, 0, 8, 8), (0, 4, 4, 8), (2, 0, 4, 4), (0, 2, 2, 4), (1, 0, 2, 2), (0, 1, 1, 2))


def decode_png(data: bytes) -> np.ndarray:
    """PNG -> (H, W, 4) float32 in [0, 1] (ColorToVec): grey and palette at 1, 2, 4 or 8 bits (palette alpha
    from tRNS), grey+alpha / RGB / RGBA at 8 or 16 bits (16-bit samples keep their high byte, as the
    reference's image loader reduces them to 8 bits), non-interlaced or Adam7-interlaced."""
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise ValueError("not a PNG image (only PNG textures are decoded)")
    off, idat = 8, []
    w = h = ctype = depth = interlace = None
    palette = trns = None
    while off < len(data):
        n, = struct.unpack(">I", data[off:off + 4])
        kind = data[off + 4:off + 8]
        body = data[off + 8:off + 8 + n]
        off += 12 + n
        if kind == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
            ok = {0: (1, 2, 4, 8, 16), 2: (8, 16), 3: (1, 2, 4, 8), 4: (8, 16), 6: (8, 16)}
            if ctype not in ok or depth not in ok[ctype]:
                raise ValueError(f"unsupported PNG colour type {ctype} at {depth} bits")
            if interlace not in (0, 1):
                raise ValueError(f"unknown PNG interlace method {interlace}")
        elif kind == b"PLTE":
            palette = np.frombuffer(body, np.uint8).reshape(-1, 3)
        elif kind == b"tRNS":
            trns = np.frombuffer(body, np.uint8)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
    if w is None:
        raise ValueError("PNG without IHDR")
    ch = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    bits = ch * depth
    bpp = max(1, bits // 8)
    try:
        stream = np.frombuffer(zlib.decompress(b"".join(idat)), np.uint8)
    except zlib.error as e:
        raise ValueError(f"corrupt PNG image data: {e}") from None
    samples = np.zeros((h, w, ch), np.uint8)
    passes = _ADAM7 if interlace else ((0, 0, 1, 1),)
    pos = 0
    for x0, y0, dx, dy in passes:
        pw, ph = -(-(w - x0) // dx) if w > x0 else 0, -(-(h - y0) // dy) if h > y0 else 0
        if pw == 0 or ph == 0:
            continue  # an empty pass has no scanlines, not even filter bytes
        stride = (pw * bits + 7) // 8
        raw = stream[pos:pos + ph * (1 + stride)]
        if raw.size < ph * (1 + stride):
            raise ValueError("corrupt PNG: image data too short")
        pos += ph * (1 + stride)
        rows = _unfilter(raw.reshape(ph, 1 + stride), ph, stride, bpp)
        samples[y0::dy, x0::dx] = _png_samples(rows, pw, ph, ch, depth, ctype)
    rgba = np.ones((h, w, 4), np.float32)
    if ctype == 3:
        if palette is None:
            raise ValueError("palette PNG without PLTE")
        idx = samples[..., 0].astype(np.int64)
        if idx.max(initial=0) >= len(palette):
            raise ValueError("PNG palette index out of range")
        rgba[..., :3] = palette[idx].astype(np.float32) / 255.0
        if trns is not None:
            alpha = np.full(len(palette), 255, np.uint8)
            alpha[:min(len(trns), len(palette))] = trns[:len(palette)]
            rgba[..., 3] = alpha[idx].astype(np.float32) / 255.0
        return rgba
    px = samples.astype(np.float32) / 255.0
    if ch in (1, 2):
        rgba[..., :3] = px[..., :1]
    else:
        rgba[..., :3] = px[..., :3]
    if ch in (2, 4):
        rgba[..., 3] = px[..., -1]
    return rgba


def decode_image(data: bytes) -> np.ndarray:
    """A PNG or baseline JPEG file (told apart by their signatures) -> (H, W, 4) float32 in [0, 1]."""
    if data[:2] == b"\xff\xd8":
        from .jpeg import decode_jpeg
        return decode_jpeg(data)
    return decode_png(data)


def _image_bytes(doc, buffers, base_dir, image):
    if "bufferView" in image:
        v = doc["bufferViews"][image["bufferView"]]
        start = v.get("byteOffset", 0)
        return bytes(buffers[v["buffer"]][start:start + v["byteLength"]])
    uri = image["uri"]
    if uri.startswith("data:"):
        return base64.b64decode(uri.split(",", 1)[1])
    return open(os.path.join(base_dir, uri), "rb").read()


def _quat_matrix(q):
    """3x3 rotation of a glTF quaternion [x, y, z, w] (normalised first)."""
    x, y, z, w = (float(v) for v in q)
    n = np.sqrt(x * x + y * y + z * z + w * w)
    x, y, z, w = x / n, y / n, z / n, w / n
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


ROT_X90 = np.array([[1.0, 0.0, 0.0], [0.0, 0.0, -1.0], [0.0, 1.0, 0.0]])  # AngleAxis(90 deg, +X)


def default_material() -> Material:
    """MaterialResource's defaults (io/Material.h:9-14): white, metallic 1, roughness 1, no emission."""
    return Material((1.0, 1.0, 1.0), (0.0, 0.0, 0.0), 1.0, 1.0, 0.0, False)


def _material(m, texture) -> Material:
    """`texture(index, srgb)` returns the Scene texture index of glTF texture `index` (decoding it once)."""
    mat = default_material()
    pbr = m.get("pbrMetallicRoughness", {})
    base, emissive = mat.base_color, mat.emissive
    metallic, roughness = mat.metallic, mat.roughness
    maps = dict(base_color_tex=-1, metallic_roughness_tex=-1, emissive_tex=-1, normal_tex=-1)
    if pbr.get("baseColorTexture", {}).get("index", -1) >= 0:
        base = tuple(float(v) for v in pbr.get("baseColorFactor", [1, 1, 1, 1])[:3])
        maps["base_color_tex"] = texture(pbr["baseColorTexture"]["index"], True)
    if m.get("normalTexture", {}).get("index", -1) >= 0:
        maps["normal_tex"] = texture(m["normalTexture"]["index"], False)
    if pbr.get("metallicRoughnessTexture", {}).get("index", -1) >= 0:
        metallic = float(pbr.get("metallicFactor", 1.0))
        roughness = float(pbr.get("roughnessFactor", 1.0))
        maps["metallic_roughness_tex"] = texture(pbr["metallicRoughnessTexture"]["index"], False)
    if m.get("emissiveTexture", {}).get("index", -1) >= 0:
        emissive = tuple(float(v) for v in m.get("emissiveFactor", [0, 0, 0])[:3])
        maps["emissive_tex"] = texture(m["emissiveTexture"]["index"], True)
    return Material(base, emissive, metallic, roughness, 0.0, False, **maps)


def _vertex_normals(pos, idx):
    n = np.zeros_like(pos, dtype=np.float64)
    p = pos.astype(np.float64)
    fn = np.cross(p[idx[:, 1]] - p[idx[:, 0]], p[idx[:, 2]] - p[idx[:, 0]])  # area-weighted
    for c in range(3):
        np.add.at(n, idx[:, c], fn)
    ln = np.linalg.norm(n, axis=1, keepdims=True)
    n = np.where(ln > 0, n / np.maximum(ln, 1e-30), np.array([0.0, 0.0, 1.0]))
    return n.astype(np.float32)


def _primitive_mesh(doc, buffers, prim, scale):
    mode = prim.get("mode", MODE_TRIANGLES)
    if mode not in (MODE_TRIANGLES, MODE_STRIP, MODE_FAN):
        return None
    attrs = prim["attributes"]
    pos = _accessor(doc, buffers, attrs["POSITION"]).astype(np.float32) * np.asarray(scale, np.float32)
    nv = len(pos)
    idx = (_accessor(doc, buffers, prim["indices"]).reshape(-1).astype(np.int64) if "indices" in prim
           else np.arange(nv, dtype=np.int64))
    if mode == MODE_FAN:
        idx = np.stack([np.full(len(idx) - 2, idx[0]), idx[1:-1], idx[2:]], 1).reshape(-1)
    elif mode == MODE_STRIP:
        idx = np.stack([idx[:-2], idx[1:-1], idx[2:]], 1).reshape(-1)
    tris = idx[: len(idx) // 3 * 3].reshape(-1, 3)
    if len(tris) == 0:
        return None
    normals = (_accessor(doc, buffers, attrs["NORMAL"]).astype(np.float32) if "NORMAL" in attrs
               else _vertex_normals(pos, tris))
    tangents = _accessor(doc, buffers, attrs["TANGENT"]).astype(np.float32) if "TANGENT" in attrs else None
    uvs = _accessor(doc, buffers, attrs["TEXCOORD_0"]).astype(np.float32) if "TEXCOORD_0" in attrs else None
    return Mesh(pos, normals, tris.astype(np.uint32), tangents, uvs)


def load_gltf(path: str, sky: Sky | None = None) -> Scene:
    """Reads a .gltf (JSON with external or data-URI buffers) or .glb file into a Scene."""
    doc, bin_chunk = _read_container(path)
    buffers = _buffers(doc, os.path.dirname(os.path.abspath(path)), bin_chunk)
    base_dir = os.path.dirname(os.path.abspath(path))
    textures, tex_index = [], {}

    def texture(index, srgb):
        # CreateTexture (GLTFLoader.cpp:273-327): colour maps are sRGB, normal and metallic-roughness data
        key = (index, srgb)
        if key not in tex_index:
            image = doc["images"][doc["textures"][index]["source"]]
            textures.append(Texture(decode_image(_image_bytes(doc, buffers, base_dir, image)), srgb=srgb))
            tex_index[key] = len(textures) - 1
        return tex_index[key]

    materials = [_material(m, texture) for m in doc.get("materials", [])]
    default_index = None
    meshes, instances = [], []

    def process(node_id, parent):
        nonlocal default_index
        node = doc["nodes"][node_id]
        rot = ROT_X90 @ (_quat_matrix(node["rotation"]) if "rotation" in node else np.eye(3))
        t = np.asarray(node.get("translation", [0.0, 0.0, 0.0]), np.float64)
        local = np.eye(4)
        local[:3, :3] = rot
        local[:3, 3] = t
        world = parent @ local
        scale = node.get("scale", [1.0, 1.0, 1.0])
        if "mesh" in node:
            for prim in doc["meshes"][node["mesh"]].get("primitives", []):
                mesh = _primitive_mesh(doc, buffers, prim, scale)
                if mesh is None:
                    continue
                mat = prim.get("material", -1)
                if mat < 0:
                    if default_index is None:
                        materials.append(default_material())
                        default_index = len(materials) - 1
                    mat = default_index
                meshes.append(mesh)
                instances.append(Instance(len(meshes) - 1, mat, world[:3, :].astype(np.float32)))
        for c in node.get("children", []):
            process(c, world)

    scenes_list = doc.get("scenes", [])
    if scenes_list:
        roots = scenes_list[doc.get("scene", 0) if doc.get("scene", -1) > -1 else 0].get("nodes", [])
    else:
        roots = list(range(len(doc.get("nodes", []))))
    for r in roots:
        process(r, np.eye(4))
    return Scene(meshes, instances, materials, sky or Sky(), name=os.path.basename(path), textures=textures)
