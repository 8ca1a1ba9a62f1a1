"""glTF import (sparkle_gb300/gltf.py) with the reference loader's conventions (GLTFLoader.cpp): +90 degrees
about X at every node, node scale baked into positions only, world = parent x local, factors read only with
their texture, fans and strips expanded, every node a root when the file has no scenes. Files are written
here (data-URI .gltf and .glb); one GPU test renders an imported scene against the oracle."""
import base64
import json
import struct

import numpy as np
import pytest

from sparkle_gb300 import abi, gltf, scenes


def png_bytes(rgba8):
    """A minimal RGBA PNG (filter 0 rows) for the embedded textures."""
    import zlib
    h, w, _ = rgba8.shape
    raw = b"".join(b"\x00" + rgba8[y].tobytes() for y in range(h))

    def chunk(t, b):
        return struct.pack(">I", len(b)) + t + b + struct.pack(">I", zlib.crc32(t + b) & 0xFFFFFFFF)
    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(raw)) + chunk(b"IEND", b""))


TEX = np.array([[[255, 0, 0, 255], [0, 255, 0, 255]], [[0, 0, 255, 255], [255, 255, 255, 128]]], np.uint8)

QUAD_POS = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float32)
QUAD_NRM = np.tile(np.array([[0, 0, 1]], np.float32), (4, 1))


def build_doc(nodes, scenes_=None, materials=None, prims=None, glb=False):
    """A glTF document with one buffer: the quad's positions, normals and three index lists."""
    tri_idx = np.array([0, 1, 2, 0, 2, 3], np.uint16)
    fan_idx = np.array([0, 1, 2, 3], np.uint16)
    blob = QUAD_POS.tobytes() + QUAD_NRM.tobytes() + tri_idx.tobytes() + fan_idx.tobytes()
    views = [dict(buffer=0, byteOffset=0, byteLength=48), dict(buffer=0, byteOffset=48, byteLength=48),
             dict(buffer=0, byteOffset=96, byteLength=12), dict(buffer=0, byteOffset=108, byteLength=8)]
    accessors = [dict(bufferView=0, componentType=5126, count=4, type="VEC3", min=[0, 0, 0], max=[1, 1, 0]),
                 dict(bufferView=1, componentType=5126, count=4, type="VEC3"),
                 dict(bufferView=2, componentType=5123, count=6, type="SCALAR"),
                 dict(bufferView=3, componentType=5123, count=4, type="SCALAR")]
    prims = prims or [dict(attributes=dict(POSITION=0, NORMAL=1), indices=2, material=0)]
    doc = dict(asset=dict(version="2.0"), bufferViews=views, accessors=accessors, nodes=nodes,
               meshes=[dict(primitives=prims)], materials=materials or [dict()],
               images=[dict(uri="data:image/png;base64," + base64.b64encode(png_bytes(TEX)).decode())],
               textures=[dict(source=0)])
    if scenes_ is not None:
        doc["scenes"] = scenes_
        doc["scene"] = 0
    if glb:
        doc["buffers"] = [dict(byteLength=len(blob))]
        js = json.dumps(doc).encode()
        js += b" " * (-len(js) % 4)
        bb = blob + b"\0" * (-len(blob) % 4)
        body = struct.pack("<II", len(js), 0x4E4F534A) + js + struct.pack("<II", len(bb), 0x004E4942) + bb
        return struct.pack("<III", 0x46546C67, 2, 12 + len(body)) + body
    doc["buffers"] = [dict(byteLength=len(blob), uri="data:application/octet-stream;base64," +
                           base64.b64encode(blob).decode())]
    return json.dumps(doc).encode()


def write(tmp_path, data, name="s.gltf"):
    p = tmp_path / name
    p.write_bytes(data)
    return str(p)


def rz(deg):
    a = np.deg2rad(deg)
    return np.array([[np.cos(a), -np.sin(a), 0], [np.sin(a), np.cos(a), 0], [0, 0, 1]])


def test_node_transform_and_scale(tmp_path):
    q = [0, 0, np.sin(np.pi / 4), np.cos(np.pi / 4)]  # 90 degrees about z, glTF [x, y, z, w]
    nodes = [dict(mesh=0, translation=[1, 2, 3], rotation=q, scale=[2, 3, 4])]
    sc = gltf.load_gltf(write(tmp_path, build_doc(nodes, scenes_=[dict(nodes=[0])])))
    assert len(sc.meshes) == 1 and len(sc.instances) == 1
    np.testing.assert_allclose(sc.meshes[0].positions, QUAD_POS * np.array([2, 3, 4], np.float32))
    m = sc.instances[0].transform
    np.testing.assert_allclose(m[:, :3], gltf.ROT_X90 @ rz(90), atol=1e-6)
    np.testing.assert_allclose(m[:, 3], [1, 2, 3], atol=1e-6)
    assert sc.meshes[0].indices.shape == (2, 3)


def test_children_compose_and_rotate_again(tmp_path):
    nodes = [dict(children=[1], translation=[0, 0, 5]), dict(mesh=0, translation=[1, 0, 0])]
    sc = gltf.load_gltf(write(tmp_path, build_doc(nodes, scenes_=[dict(nodes=[0])])))
    parent = np.eye(4)
    parent[:3, :3] = gltf.ROT_X90
    parent[:3, 3] = [0, 0, 5]
    child = np.eye(4)
    child[:3, :3] = gltf.ROT_X90
    child[:3, 3] = [1, 0, 0]
    np.testing.assert_allclose(sc.instances[0].transform, (parent @ child)[:3], atol=1e-6)


def test_no_scenes_makes_every_node_a_root(tmp_path):
    nodes = [dict(children=[1]), dict(mesh=0)]
    sc = gltf.load_gltf(write(tmp_path, build_doc(nodes)))
    assert len(sc.instances) == 2  # node 1 once as node 0's child and once as a root


def test_material_factors_need_their_texture(tmp_path):
    mats = [dict(pbrMetallicRoughness=dict(baseColorFactor=[0.2, 0.3, 0.4, 1], metallicFactor=0.0,
                                           roughnessFactor=0.5), emissiveFactor=[1, 1, 1]),
            dict(pbrMetallicRoughness=dict(baseColorFactor=[0.2, 0.3, 0.4, 1], baseColorTexture=dict(index=0),
                                           metallicFactor=0.0, roughnessFactor=0.5,
                                           metallicRoughnessTexture=dict(index=0)),
                 emissiveFactor=[1, 2, 3], emissiveTexture=dict(index=0))]
    prims = [dict(attributes=dict(POSITION=0, NORMAL=1), indices=2, material=0),
             dict(attributes=dict(POSITION=0, NORMAL=1), indices=2, material=1),
             dict(attributes=dict(POSITION=0, NORMAL=1), indices=2)]
    sc = gltf.load_gltf(write(tmp_path, build_doc([dict(mesh=0)], scenes_=[dict(nodes=[0])], materials=mats,
                                                  prims=prims)))
    m0, m1 = sc.materials[0], sc.materials[1]
    assert (m0.base_color, m0.metallic, m0.roughness, m0.emissive) == ((1.0, 1.0, 1.0), 1.0, 1.0, (0.0, 0.0, 0.0))
    assert m1.base_color == pytest.approx((0.2, 0.3, 0.4)) and (m1.metallic, m1.roughness) == (0.0, 0.5)
    assert m1.emissive == (1.0, 2.0, 3.0)
    assert sc.instances[2].material_id == 2 and sc.materials[2].metallic == 1.0  # default material appended
    # texture 0 decoded once per colour space: sRGB for base colour / emissive, linear for metallic-roughness
    assert (m1.base_color_tex, m1.emissive_tex) == (0, 0) and m1.metallic_roughness_tex == 1
    assert sc.textures[0].srgb and not sc.textures[1].srgb
    np.testing.assert_allclose(sc.textures[0].rgba, TEX / 255.0, atol=1e-7)


@pytest.mark.parametrize("mode,ntri", [(6, 2), (5, 2)])
def test_fans_and_strips(tmp_path, mode, ntri):
    prims = [dict(attributes=dict(POSITION=0, NORMAL=1), indices=3, material=0, mode=mode)]
    sc = gltf.load_gltf(write(tmp_path, build_doc([dict(mesh=0)], scenes_=[dict(nodes=[0])], prims=prims)))
    idx = sc.meshes[0].indices
    assert idx.shape == (ntri, 3)
    if mode == 6:
        np.testing.assert_array_equal(idx, [[0, 1, 2], [0, 2, 3]])
    else:
        np.testing.assert_array_equal(idx, [[0, 1, 2], [1, 2, 3]])


def test_glb_and_missing_normals(tmp_path):
    prims = [dict(attributes=dict(POSITION=0), indices=2, material=0)]
    sc = gltf.load_gltf(write(tmp_path, build_doc([dict(mesh=0)], scenes_=[dict(nodes=[0])], prims=prims, glb=True),
                              "s.glb"))
    np.testing.assert_allclose(sc.meshes[0].normals, QUAD_NRM, atol=1e-6)


@pytest.mark.gpu
def test_imported_scene_renders_like_the_oracle(tmp_path):
    import oracle
    from sparkle_gb300 import native
    mats = [dict(pbrMetallicRoughness=dict(baseColorFactor=[0.7, 0.6, 0.5, 1], baseColorTexture=dict(index=0),
                                           metallicFactor=0.0, roughnessFactor=1.0,
                                           metallicRoughnessTexture=dict(index=0)))]
    nodes = [dict(mesh=0, translation=[-0.5, 0, -0.5])]
    sc = gltf.load_gltf(write(tmp_path, build_doc(nodes, scenes_=[dict(nodes=[0])], materials=mats)),
                        sky=abi.Sky(abi.SPK_SKY_GRADIENT, (0.5, 0.7, 1.0), None))
    cam = abi.camera_from_look((0, -3, 1), (0, 0, 0), (0, 0, 1), 0.8, 3.0, 0.0, 1.0, 48, 32)
    cfg = abi.make_config(48, 32, spp=1, bounce=3, seed=4)
    ctx = native.Context(0)
    ctx.set_scene(sc)
    ctx.set_config(cfg)
    ctx.set_camera(cam)
    ctx.render(2)
    hdr, _ = ctx.framebuffer()
    r = oracle.OracleRenderer(oracle.OracleScene(sc), cfg, cam)
    r.render(2, traversal=oracle.PRUNED)
    ref, _ = r.framebuffer()
    close = np.all(np.abs(hdr[..., :3] - ref[..., :3]) <= 1e-4 * (1 + np.abs(ref[..., :3])), axis=-1)
    assert close.mean() > 0.95
    ctx.close()


def test_jpeg_texture(tmp_path):
    """An embedded JPEG image (image/jpeg) decodes like a PNG one, within the JPEG's own rounding."""
    from test_jpeg import encode_jpeg, smooth_rgb
    img = smooth_rgb(16, 24, 7)
    jpg = encode_jpeg(img, q=1)
    mats = [dict(pbrMetallicRoughness=dict(baseColorTexture=dict(index=0)))]
    doc = json.loads(build_doc([dict(mesh=0)], scenes_=[dict(nodes=[0])], materials=mats))
    doc["images"] = [dict(uri="data:image/jpeg;base64," + base64.b64encode(jpg).decode())]
    sc = gltf.load_gltf(write(tmp_path, json.dumps(doc).encode()))
    tex = sc.textures[0].rgba
    assert tex.shape == (16, 24, 4)
    assert np.abs(np.rint(tex[..., :3] * 255) - img).max() <= 3.0
