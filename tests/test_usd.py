"""USDA import / export (sparkle_gb300/usd.py) with the reference's USDLoader / USDExporter conventions:
xformOps composed in xformOpOrder and transposed from USD's row-vector matrices, world = parent x local,
meshes take their parent Xform's transform, polygons fan-triangulated, faceVarying primvars expanded,
tangents from GetPossibleMajorAxis when absent, UsdPreviewSurface opacity < 1 -> dielectric with its ior,
connected inputs -> texture maps, meshes without a material skipped. Export -> import must give the scene
back; one GPU test renders an imported scene against the oracle."""
import numpy as np
import pytest

from sparkle_gb300 import abi, native, scenes, usd


def write(tmp_path, text, name="s.usda"):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


HEADER = '#usda 1.0\n(\n    defaultPrim = "root"\n    upAxis = "Z"\n)\n'

MAT = '''
def Scope "Looks"
{
    def Material "m"
    {
        token outputs:surface.connect = </Looks/m/pbr.outputs:surface>
        def Shader "pbr"
        {
            uniform token info:id = "UsdPreviewSurface"
            color3f inputs:diffuseColor = (0.5, 0.25, 0.125)
            float inputs:roughness = 0.75
            token outputs:surface
        }
    }
    def Material "glass"
    {
        token outputs:surface.connect = </Looks/glass/pbr.outputs:surface>
        def Shader "pbr"
        {
            uniform token info:id = "UsdPreviewSurface"
            float inputs:opacity = 0.1
            float inputs:ior = 1.33
            token outputs:surface
        }
    }
}
'''


def test_xform_ops_and_hierarchy(tmp_path):
    text = HEADER + '''
def Xform "root"
{
    float3 xformOp:translate = (1, 2, 3)
    float3 xformOp:rotateXYZ = (0, 0, 90)
    float3 xformOp:scale = (2, 2, 2)
    uniform token[] xformOpOrder = ["xformOp:translate", "xformOp:rotateXYZ", "xformOp:scale"]
    def Xform "child"
    {
        matrix4d xformOp:transform = ( (1, 0, 0, 0), (0, 1, 0, 0), (0, 0, 1, 0), (5, 0, 0, 1) )
        uniform token[] xformOpOrder = ["xformOp:transform"]
        def Mesh "tri"
        {
            float3 xformOp:translate = (100, 100, 100)
            uniform token[] xformOpOrder = ["xformOp:translate"]
            int[] faceVertexCounts = [3]
            int[] faceVertexIndices = [0, 1, 2]
            point3f[] points = [(0, 0, 0), (1, 0, 0), (0, 1, 0)]
            normal3f[] normals = [(0, 0, 1), (0, 0, 1), (0, 0, 1)] (interpolation = "vertex")
            rel material:binding = </Looks/m>
        }
    }
    def Mesh "unbound"
    {
        int[] faceVertexCounts = [3]
        int[] faceVertexIndices = [0, 1, 2]
        point3f[] points = [(0, 0, 0), (1, 0, 0), (0, 1, 0)]
    }
}
''' + MAT
    sc = usd.load_usda(write(tmp_path, text))
    assert len(sc.meshes) == 1 and len(sc.instances) == 1  # the unbound mesh is skipped
    rz = np.array([[0, -1, 0], [1, 0, 0], [0, 0, 1]], np.float64)
    parent = np.eye(4)
    parent[:3, :3] = rz * 2
    parent[:3, 3] = [1, 2, 3]
    child = np.eye(4)
    child[0, 3] = 5  # USD's translation row becomes the column; the mesh's own op is not read
    np.testing.assert_allclose(sc.instances[0].transform, (parent @ child)[:3], atol=1e-6)
    m = sc.materials[sc.instances[0].material_id]
    assert m.base_color == (0.5, 0.25, 0.125) and (m.metallic, m.roughness) == (0.0, 0.75) and not m.dielectric


def test_polygons_face_varying_and_generated_attributes(tmp_path):
    text = HEADER + '''
def Xform "root"
{
    def Mesh "poly"
    {
        int[] faceVertexCounts = [4, 5]
        int[] faceVertexIndices = [0, 1, 2, 3, 1, 4, 5, 6, 2]
        point3f[] points = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (2, 0, 0), (2.5, 0.5, 0), (2, 1, 0)]
        normal3f[] normals = [(0, 0, 1), (0, 1, 0)] (interpolation = "uniform")
        texCoord2f[] primvars:st = [(0, 0), (1, 0), (1, 1)] (interpolation = "faceVarying")
        int[] primvars:st:indices = [0, 1, 2, 0, 0, 1, 2, 1, 0]
        rel material:binding = </Looks/glass>
    }
    def Mesh "bare"
    {
        int[] faceVertexCounts = [3]
        int[] faceVertexIndices = [0, 2, 1]
        point3f[] points = [(0, 0, 0), (1, 0, 0), (0, 1, 0)]
        rel material:binding = </Looks/m>
    }
}
''' + MAT
    sc = usd.load_usda(write(tmp_path, text))
    poly, bare = sc.meshes
    assert poly.indices.shape == (5, 3)  # quad -> 2, pentagon -> 3 (fans)
    np.testing.assert_array_equal(poly.indices[:2], [[0, 1, 2], [0, 2, 3]])  # corners of the quad
    np.testing.assert_array_equal(poly.normals[:4], np.tile([0, 0, 1], (4, 1)))  # uniform: per face
    np.testing.assert_array_equal(poly.normals[4:], np.tile([0, 1, 0], (5, 1)))
    np.testing.assert_array_equal(poly.uvs[4:9], [[0, 0], [1, 0], [1, 1], [1, 0], [0, 0]])  # st[indices[4:9]]
    np.testing.assert_array_equal(poly.positions[4:9], [[1, 0, 0], [2, 0, 0], [2.5, 0.5, 0], [2, 1, 0], [1, 1, 0]])
    # no normals: area-weighted (the winding 0, 2, 1 faces -z); tangents: cross(cross(n, a), n), w = 1
    np.testing.assert_allclose(bare.normals, np.tile([0, 0, -1], (3, 1)))
    np.testing.assert_allclose(bare.tangents, np.tile([1, 0, 0, 1], (3, 1)))
    glass = sc.materials[sc.instances[0].material_id]
    assert glass.dielectric and glass.eta == pytest.approx(1.33) and glass.base_color == pytest.approx((0.18,) * 3)


def test_texture_connections(tmp_path):
    from sparkle_gb300 import native
    img = np.zeros((2, 2, 4), np.uint8)
    img[..., 0] = [[0, 255], [128, 64]]
    img[..., 3] = 255
    (tmp_path / "tex").mkdir()
    native.write_png(tmp_path / "tex" / "a.png", img)
    text = HEADER + '''
def Xform "root"
{
    def Mesh "q"
    {
        int[] faceVertexCounts = [3]
        int[] faceVertexIndices = [0, 1, 2]
        point3f[] points = [(0, 0, 0), (1, 0, 0), (0, 1, 0)]
        normal3f[] normals = [(0, 0, 1), (0, 0, 1), (0, 0, 1)]
        rel material:binding = </M/t>
    }
}
def Scope "M"
{
    def Material "t"
    {
        token outputs:surface.connect = </M/t/s.outputs:surface>
        def Shader "s"
        {
            uniform token info:id = "UsdPreviewSurface"
            color3f inputs:diffuseColor.connect = </M/t/img.outputs:rgb>
            color3f inputs:emissiveColor.connect = </M/t/img.outputs:rgb>
            float inputs:metallic.connect = </M/t/img.outputs:b>
            float inputs:roughness.connect = </M/t/img.outputs:g>
            normal3f inputs:normal.connect = </M/t/img.outputs:rgb>
            token outputs:surface
        }
        def Shader "img"
        {
            uniform token info:id = "UsdUVTexture"
            asset inputs:file = @tex/a.png@
            float3 outputs:rgb
        }
    }
}
'''
    sc = usd.load_usda(write(tmp_path, text))
    m = sc.materials[0]
    assert m.base_color == (1.0, 1.0, 1.0) and m.emissive == (1.0, 1.0, 1.0)  # factors stay at 1
    assert (m.base_color_tex, m.emissive_tex) == (0, 0) and m.metallic_roughness_tex == 1 and m.normal_tex == 1
    assert sc.textures[0].srgb and not sc.textures[1].srgb
    np.testing.assert_allclose(sc.textures[0].rgba, img / 255.0, atol=1e-7)


def test_export_then_import_gives_the_scene_back(tmp_path):
    scene, _ = scenes.cornell_box(2)
    tex = np.random.default_rng(0).integers(0, 256, (4, 4, 4)).astype(np.float32) / 255
    scene.textures = [abi.Texture(tex, srgb=True)]
    scene.materials[0].base_color = (1.0, 1.0, 1.0)
    scene.materials[0].base_color_tex = 0
    scene.materials[3] = abi.Material.glass((0.9, 0.95, 1.0), 1.45)
    scene.instances.append(abi.Instance(0, 1, np.eye(3, 4), sphere=True, radius=0.1))  # not exported
    p = tmp_path / "out" / "scene.usda"
    p.parent.mkdir()
    usd.save_usda(scene, p)
    assert (tmp_path / "out" / "textures").is_dir()
    back = usd.load_usda(str(p))
    assert len(back.instances) == len(scene.instances) - 1
    for a, b in zip(scene.instances, back.instances):
        ma, mb = scene.meshes[a.mesh_id], back.meshes[b.mesh_id]
        for f in ("positions", "normals", "indices", "uvs", "tangents"):
            np.testing.assert_array_equal(getattr(ma, f), getattr(mb, f), err_msg=f)
        np.testing.assert_array_equal(a.transform, b.transform)
        x, y = scene.materials[a.material_id], back.materials[b.material_id]
        assert x.dielectric == y.dielectric and x.base_color == pytest.approx(y.base_color)
        assert x.emissive == pytest.approx(y.emissive)
        if x.dielectric:
            assert x.eta == pytest.approx(y.eta)
        else:
            assert (x.metallic, x.roughness) == pytest.approx((y.metallic, y.roughness))
        assert (x.base_color_tex >= 0) == (y.base_color_tex >= 0)
    np.testing.assert_array_equal(back.textures[0].rgba, scene.textures[0].rgba)
    with pytest.raises(usd.UsdError):
        usd.save_usda(scene, tmp_path / "x.usdc")


def test_binary_files_are_refused(tmp_path):
    p = tmp_path / "b.usdc"
    p.write_bytes(b"PXR-USDC" + bytes(64))
    with pytest.raises((usd.UsdError, UnicodeDecodeError)):
        usd.load_usda(str(p))


@pytest.mark.gpu
def test_imported_scene_renders_like_the_oracle(tmp_path):
    import oracle
    from sparkle_gb300 import native
    scene, cam_args = scenes.cornell_box(1)
    p = tmp_path / "c.usda"
    usd.save_usda(scene, p)
    sc = usd.load_usda(str(p))
    W, H = 48, 40
    cam = scenes.make_camera(cam_args, W, H)
    cfg = abi.make_config(W, H, spp=1, bounce=4, seed=3)
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


CAMERA_USDA = '''#usda 1.0
(
    defaultPrim = "root"
)
def Xform "root"
{
    def Xform "first"
    {
        double3 xformOp:translate = (9, 9, 9)
        uniform token[] xformOpOrder = ["xformOp:translate"]
        def Camera "unused"
        {
        }
    }
    def Xform "cam_node"
    {
        double3 xformOp:translate = (1, 2, 3)
        uniform token[] xformOpOrder = ["xformOp:translate"]
        def Camera "cam"
        {
            float focalLength = 50
            float verticalAperture = 24
            float fStop = 2.8
            float focusDistance = 5
            double3 xformOp:translate = (100, 0, 0)
            uniform token[] xformOpOrder = ["xformOp:translate"]
        }
    }
}
'''


def _cam_fields(c):
    return {k: np.array(getattr(c, k), np.float32) for k in
            ("position", "right", "up", "front", "lower_left", "max_u", "max_v")}


def test_usd_camera_matches_the_library_camera(tmp_path):
    """The last camera wins, its own xformOps are not read (the parent node's transform is the camera's),
    and with an unrotated node the result equals spk_camera_from_look for the same posture and lens."""
    p = tmp_path / "cam.usda"
    p.write_text(CAMERA_USDA)
    c = usd.load_usda_camera(str(p), 640, 480)
    vfov = 2 * np.arctan(np.float32(0.024) / (2 * np.float32(0.05)))
    ref = native.camera_from_look((1, 2, 3), (1, 3, 3), (0, 0, 1), float(vfov), 5.0,
                                  float(np.float32(0.05) / np.float32(2.8) * np.float32(0.5)), 1.0, 640, 480)
    got, want = _cam_fields(c), _cam_fields(ref)
    for k in got:
        np.testing.assert_allclose(got[k], want[k], rtol=1e-6, atol=1e-6, err_msg=k)
    assert c.aperture_radius == pytest.approx(ref.aperture_radius, rel=1e-6)
    assert c.far_plane == ref.far_plane and c.exposure == 1.0


def test_usd_camera_defaults_rows_and_refusals(tmp_path):
    text = CAMERA_USDA.replace('''            float focalLength = 50
            float verticalAperture = 24
            float fStop = 2.8
            float focusDistance = 5
''', "").replace('double3 xformOp:translate = (1, 2, 3)\n        uniform token[] xformOpOrder = ["xformOp:translate"]',
                 'float3 xformOp:rotateXYZ = (0, 0, 30)\n        uniform token[] xformOpOrder = ["xformOp:rotateXYZ"]')
    p = tmp_path / "d.usda"
    p.write_text(text)
    c = usd.load_usda_camera(str(p), 100, 50)
    # unauthored lens: 35 mm, 24 mm sensor, f/22, focus distance 1
    assert c.aperture_radius == pytest.approx(0.035 / 22 * 0.5, rel=1e-6)
    m = np.eye(3)
    a = np.deg2rad(30)
    m[0, 0], m[0, 1], m[1, 0], m[1, 1] = np.cos(a), -np.sin(a), np.sin(a), np.cos(a)
    # right / front / up are the rows of the node's matrix (Transform::ExtractLocalBasis)
    np.testing.assert_allclose(_cam_fields(c)["right"], m[0], atol=1e-6)
    np.testing.assert_allclose(_cam_fields(c)["front"], m[1], atol=1e-6)
    vfov = 2 * np.arctan(0.024 / 0.07)
    plane_h = 2 * np.tan(vfov / 2)
    np.testing.assert_allclose(_cam_fields(c)["max_v"], m[2] * plane_h, rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(_cam_fields(c)["max_u"], m[0] * plane_h * 2, rtol=1e-5, atol=1e-6)
    ortho = text.replace('def Camera "cam"\n        {', 'def Camera "cam"\n        {\n            token projection = "orthographic"')
    (tmp_path / "o.usda").write_text(ortho)
    with pytest.raises(usd.UsdError):
        usd.load_usda_camera(str(tmp_path / "o.usda"), 100, 50)
    none = '#usda 1.0\ndef Xform "root"\n{\n}\n'
    (tmp_path / "n.usda").write_text(none)
    assert usd.load_usda_camera(str(tmp_path / "n.usda"), 100, 50) is None


def test_camera_export_round_trip(tmp_path, cornell):
    """save_usda(..., camera) writes ExportCamera's prim; load_usda_camera reads back the same camera."""
    scene, cam_args = cornell
    W, H = 320, 240
    cam = scenes.make_camera(cam_args, W, H)
    p = tmp_path / "with_cam.usda"
    usd.save_usda(scene, str(p), camera=cam)
    back = usd.load_usda_camera(str(p), W, H)
    got, want = _cam_fields(back), _cam_fields(cam)
    for k in got:
        np.testing.assert_allclose(got[k], want[k], rtol=1e-5, atol=1e-5, err_msg=k)
    if cam.aperture_radius > 0:
        assert back.aperture_radius == pytest.approx(cam.aperture_radius, rel=1e-5)
    assert len(usd.load_usda(str(p)).meshes) == len([i for i in scene.instances if not i.sphere])
