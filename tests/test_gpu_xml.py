"""Scenes in the reference's XML format (dl_scene_create_from_xml) against the
same scene built from arrays: identical geometry gives identical hits and
identical per-path radiance; malformed files fail with DL_ERR_PARSE."""
import numpy as np
import pytest

import make_golden as mg
from drawlab_gb300 import abi, api, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    return api.Context(0)


def cornell_xml(sc, obj_path):
    def v(x):
        return ", ".join("%.9g" % float(c) for c in x)

    quads = [((-1, -1, -1), (0, 0, 2), (2, 0, 0), (0.725, 0.725, 0.725)),
             ((-1, 1, -1), (2, 0, 0), (0, 0, 2), (0.725, 0.725, 0.725)),
             ((-1, -1, -1), (2, 0, 0), (0, 2, 0), (0.725, 0.725, 0.725)),
             ((-1, -1, -1), (0, 2, 0), (0, 0, 2), (0.63, 0.065, 0.05)),
             ((1, -1, -1), (0, 0, 2), (0, 2, 0), (0.14, 0.45, 0.09))]
    out = ['<?xml version="1.0"?>', "<!-- Cornell box in the reference's scene format -->", "<scene>",
           '  <integrator type="path"/>',
           '  <sampler type="independent"><integer name="sampleCount" value="7"/></sampler>',
           '  <camera type="virtual">',
           '    <vector name="eye" value="%s"/>' % v(sc.camera.eye),
           '    <vector name="lookat" value="%s"/>' % v(sc.camera.lookat),
           '    <vector name="up" value="%s"/>' % v(sc.camera.up),
           '    <float name="fov" value="%.9g"/>' % sc.camera.fov,
           '    <integer name="width" value="%d"/>' % sc.camera.width,
           '    <integer name="height" value="%d"/>' % sc.camera.height,
           '    <rfilter type="gaussian"/>',
           "  </camera>",
           '  <bsdf type="diffuse" id="white"><color name="albedo" value="0.725, 0.725, 0.725"/></bsdf>']
    for pos, a, b, alb in quads:
        out += ['  <mesh type="rectangle">', '    <vector name="pos" value="%s"/>' % v(pos),
                '    <vector name="v0" value="%s"/>' % v(a), '    <vector name="v1" value="%s"/>' % v(b),
                '    <bsdf type="diffuse"><color name="albedo" value="%s"/></bsdf>' % v(alb), "  </mesh>"]
    out += ['  <mesh type="obj">', '    <string name="filename" value="%s"/>' % obj_path,
            '    <ref id="white"/>', '    <transform name="toWorld">',
            '      <translate value="0.0, 0.0, 0.0"/>', "    </transform>", "  </mesh>",
            '  <mesh type="rectangle">', '    <vector name="pos" value="-0.25, 0.999, -0.2"/>',
            '    <vector name="v0" value="0.5, 0, 0"/>', '    <vector name="v1" value="0, 0, 0.4"/>',
            '    <bsdf type="diffuse"><color name="albedo" value="0, 0, 0"/></bsdf>',
            '    <emitter type="area"><color name="radiance" value="17, 12, 4"/></emitter>', "  </mesh>",
            "</scene>"]
    return "\n".join(out)


def write_obj(path, P, F, N):
    with open(path, "w") as f:
        f.write("# cuboid\n")
        for p in P:
            f.write("v %.9g %.9g %.9g\n" % tuple(p))
        for n in N:
            f.write("vn %.9g %.9g %.9g\n" % tuple(n))
        for t in F:
            f.write("f %d//%d %d//%d %d//%d\n" % (t[0] + 1, t[0] + 1, t[1] + 1, t[1] + 1, t[2] + 1, t[2] + 1))


def arrays_equivalent():
    """The XML scene as arrays: 5 quads, one cuboid mesh, the light quad."""
    s = scenes.SceneData("cornell_xml")
    base = scenes.cornell(width=40, height=32)
    s.camera = base.camera
    for m in base.meshes[:5]:
        s.meshes.append(m)
    s.materials = list(base.materials)
    white = s.add_material(scenes.Material(albedo=(0.725, 0.725, 0.725)))
    P, F, N = scenes.cuboid((0.34, -1 + 0.3 + 1e-3, 0.32), (0.6, 0.6, 0.6), -17.0)
    s.add_mesh(scenes.Mesh(P, F, N, material=white))
    p, f, n = scenes.rectangle((-0.25, 0.999, -0.2), (0.5, 0, 0), (0, 0, 0.4))
    li = s.add_mesh(scenes.Mesh(p, f, n, material=3))
    s.add_area_light(li, (17.0, 12.0, 4.0))
    return s, (P, F, N)


def test_xml_scene_matches_arrays(ctx, tmp_path):
    arr, (P, F, N) = arrays_equivalent()
    # the OBJ round-trips through text: write with 9 significant digits (exact for float32)
    write_obj(tmp_path / "cuboid.obj", P, F, N)
    (tmp_path / "scene.xml").write_text(cornell_xml(arr, "cuboid.obj"))
    gx = api.Scene.from_xml(ctx, str(tmp_path / "scene.xml"))
    ga = api.Scene.from_data(ctx, arr)
    ix, ia = gx.info(), ga.info()
    assert (ix.num_triangles, ix.num_lights, ix.width, ix.height) == (ia.num_triangles, ia.num_lights, 40, 32)
    d = gx.default_opts()
    assert d.spp == 7 and d.filter == abi.DL_FILTER_GAUSSIAN and d.rr_depth == 3 and d.max_depth == 0
    rays = mg.seeded_rays(arr, 20000, seed=5)
    a, b = gx.trace_closest(rays), ga.trace_closest(rays)
    for x, y in zip(a, b):
        np.testing.assert_array_equal(x, y)
    xys = np.array([(x, y, s) for y in range(32) for x in range(40) for s in range(2)], np.int32)
    opts = abi.make_opts(seed=3, max_depth=6)
    La, _ = gx.li(opts, xys)
    Lb, _ = ga.li(opts, xys)
    np.testing.assert_array_equal(La, Lb)


@pytest.mark.parametrize("text,needle", [
    ("<scene><integrator type='path'/>", "unterminated"),
    ("<scene><foo/></scene>", "unexpected tag"),
    ("<scene><integrator type='path'/></scene>", "No camera"),
    ("<scene><camera type='virtual'><vector name='eye' value='0,0'/></camera></scene>", "expected 3 values"),
    ("<scene><integrator type='path' bogus='1'/></scene>", "unexpected attribute"),
    ("<scene><mesh type='rectangle'><ref id='nothere'/></mesh></scene>", "can't find"),
])
def test_malformed_xml_is_reported(ctx, tmp_path, text, needle):
    p = tmp_path / "bad.xml"
    p.write_text(text)
    with pytest.raises(api.DrawlabError) as e:
        api.Scene.from_xml(ctx, str(p))
    assert e.value.status == abi.DL_ERR_PARSE
    assert needle in str(e.value)


def test_missing_file_is_io_error(ctx, tmp_path):
    with pytest.raises(api.DrawlabError) as e:
        api.Scene.from_xml(ctx, str(tmp_path / "none.xml"))
    assert e.value.status == abi.DL_ERR_IO


def test_unsupported_plugin_is_reported(ctx, tmp_path):
    p = tmp_path / "u.xml"
    p.write_text("<scene><integrator type='photonmapper'/></scene>")
    with pytest.raises(api.DrawlabError) as e:
        api.Scene.from_xml(ctx, str(p))
    assert e.value.status == abi.DL_ERR_UNSUPPORTED


def write_pfm(path, rgb):
    """PFM: rows bottom to top, little endian (negative scale)."""
    h, w, _ = rgb.shape
    with open(path, "wb") as f:
        f.write(b"PF\n%d %d\n-1.0\n" % (w, h))
        f.write(np.ascontiguousarray(rgb[::-1], dtype="<f4").tobytes())


def test_xml_envmap_matches_arrays(ctx, tmp_path):
    arr, (P, F, N) = arrays_equivalent()
    sky = scenes.sky_envmap(64, 32, sun_peak=50.0, sun_radius_deg=8.0)
    arr.lights.append(scenes.Light(type=abi.DL_LIGHT_ENVMAP, env_rgb=sky, env_scale=2.0, env_visual=0,
                                   env_background=(0.1, 0.2, 0.3)))
    write_obj(tmp_path / "cuboid.obj", P, F, N)
    write_pfm(tmp_path / "sky.pfm", sky)
    text = cornell_xml(arr, "cuboid.obj").replace(
        "</scene>",
        '  <color name="bg_color" value="0.1, 0.2, 0.3"/>\n'
        '  <emitter type="envmap"><string name="filename" value="sky.pfm"/>'
        '<float name="scale" value="2"/><boolean name="visual" value="false"/></emitter>\n</scene>')
    (tmp_path / "scene.xml").write_text(text)
    gx = api.Scene.from_xml(ctx, str(tmp_path / "scene.xml"))
    ga = api.Scene.from_data(ctx, arr)
    assert gx.info().num_lights == 2
    xys = np.array([(x, y, s) for y in range(32) for x in range(40) for s in range(2)], np.int32)
    opts = abi.make_opts(seed=4, max_depth=6)
    La, _ = gx.li(opts, xys)
    Lb, _ = ga.li(opts, xys)
    np.testing.assert_array_equal(La, Lb)
    assert (La > 0).any()


def test_xml_envmap_bad_image(ctx, tmp_path):
    (tmp_path / "bad.pfm").write_bytes(b"P6\n2 2\n255\n")
    (tmp_path / "s.xml").write_text(
        "<scene><integrator type='path'/><emitter type='envmap'>"
        "<string name='filename' value='bad.pfm'/></emitter></scene>")
    with pytest.raises(api.DrawlabError) as e:
        api.Scene.from_xml(ctx, str(tmp_path / "s.xml"))
    assert e.value.status == abi.DL_ERR_PARSE and "not a PFM image" in str(e.value)
    (tmp_path / "t.xml").write_text(
        "<scene><integrator type='path'/><emitter type='envmap'>"
        "<string name='filename' value='sky.exr'/></emitter></scene>")
    with pytest.raises(api.DrawlabError) as e:
        api.Scene.from_xml(ctx, str(tmp_path / "t.xml"))
    assert e.value.status == abi.DL_ERR_UNSUPPORTED


def matrix_xml(m):
    return '<matrix value="%s"/>' % ", ".join("%.9g" % float(x) for x in np.asarray(m, np.float32).reshape(16))


@pytest.mark.parametrize("kind", ["perspective", "opencv"])
def test_xml_cameras_and_normals_integrator(ctx, tmp_path, kind):
    """<camera type="perspective"> (toWorld, fov, clip planes) and
    <camera type="opencv"> (fx, fy, cx, cy, extrinsic) with
    <integrator type="normals">: the same paths as the scene built from
    arrays; the integrator lands in the scene's default options."""
    arr, (P, F, N) = arrays_equivalent()
    W, H = arr.camera.width, arr.camera.height
    if kind == "perspective":
        m = scenes.look_at((0.3, 0.2, 3.6), (0.0, -0.1, 0.0), (0.0, 1.0, 0.0)).astype(np.float32)
        cam_xml = ['  <camera type="perspective">', '    <float name="fov" value="50"/>',
                   '    <float name="farClip" value="100"/>',
                   '    <transform name="toWorld">', "      " + matrix_xml(m), "    </transform>"]
        arr.camera = scenes.Camera(width=W, height=H, type=abi.DL_CAMERA_PERSPECTIVE, fov=50.0,
                                   far_clip=100.0, transform=m)
    else:
        m = np.array([[1, 0, 0, 0.1], [0, -1, 0, 0.05], [0, 0, -1, 3.9], [0, 0, 0, 1]], np.float32)
        cam_xml = ['  <camera type="opencv">', '    <float name="fx" value="44"/>',
                   '    <float name="fy" value="46"/>', '    <float name="cx" value="21"/>',
                   '    <float name="cy" value="15.5"/>',
                   '    <transform name="extrinsic">', "      " + matrix_xml(m), "    </transform>"]
        arr.camera = scenes.Camera(width=W, height=H, type=abi.DL_CAMERA_OPENCV, fx=44.0, fy=46.0, cx=21.0,
                                   cy=15.5, transform=m)
    cam_xml += ['    <integer name="width" value="%d"/>' % W, '    <integer name="height" value="%d"/>' % H,
                "  </camera>"]
    text = cornell_xml(arr, "cuboid.obj").replace('<integrator type="path"/>', '<integrator type="normals"/>')
    lines = text.split("\n")
    a = next(i for i, x in enumerate(lines) if x.strip().startswith('<camera type="virtual">'))
    b = next(i for i, x in enumerate(lines) if x.strip() == "</camera>")
    lines[a:b + 1] = cam_xml
    write_obj(tmp_path / "cuboid.obj", P, F, N)
    (tmp_path / "scene.xml").write_text("\n".join(lines))
    gx = api.Scene.from_xml(ctx, str(tmp_path / "scene.xml"))
    ga = api.Scene.from_data(ctx, arr)
    d = gx.default_opts()
    assert d.flags & abi.DL_RENDER_NORMALS
    xys = np.array([(x, y, s) for y in range(H) for x in range(W) for s in range(2)], np.int32)
    La, pa = gx.li(d, xys)
    Lb, pb = ga.li(d, xys)
    np.testing.assert_array_equal(pa, pb)
    np.testing.assert_array_equal(La, Lb)
    assert (La.sum(1) > 0).mean() > 0.5


def test_xml_camera_errors(ctx, tmp_path):
    base = ("<scene><integrator type='path'/><camera type='%s'>%s</camera></scene>")
    cases = [("opencv", "<float name='fx' value='1'/><float name='fy' value='1'/><float name='cx' value='0'/>"
                        "<float name='cy' value='0'/>", abi.DL_ERR_PARSE),            # no extrinsic
             ("perspective", "<float name='nearClip' value='0.5'/>", abi.DL_ERR_INVALID_ARG),
             ("orthographic", "", abi.DL_ERR_UNSUPPORTED)]
    for k, (typ, body, status) in enumerate(cases):
        p = tmp_path / ("c%d.xml" % k)
        p.write_text(base % (typ, body))
        with pytest.raises(api.DrawlabError) as e:
            api.Scene.from_xml(ctx, str(p))
        assert e.value.status == status, (typ, e.value)


def test_command_line_renders_xml_to_exr_and_png(ctx, tmp_path):
    """python -m drawlab_gb300 scene.xml writes scene.exr and scene.png next
    to the file (the reference's output naming); the EXR holds the render."""
    import test_image_io as io
    from drawlab_gb300 import __main__ as cli

    arr, (P, F, N) = arrays_equivalent()
    write_obj(tmp_path / "cuboid.obj", P, F, N)
    (tmp_path / "scene.xml").write_text(cornell_xml(arr, str(tmp_path / "cuboid.obj")))
    assert cli.main([str(tmp_path / "scene.xml"), "--spp", "4", "--seed", "2"]) == 0
    img = io.read_exr(tmp_path / "scene.exr")
    gx = api.Scene.from_xml(ctx, str(tmp_path / "scene.xml"))
    o = gx.default_opts()
    o.spp, o.seed = 4, 2
    np.testing.assert_array_equal(img, gx.render(o))
    assert io.read_png(tmp_path / "scene.png").shape == img.shape


@pytest.mark.parametrize("fmt", ["png", "pfm"])
def test_xml_bitmap_texture_matches_arrays(ctx, tmp_path, fmt):
    """<texture type="bitmap" name="albedo"> on the floor's diffuse BSDF:
    the same paths as the arrays scene whose floor carries the texture in the
    texel order the reference uploads -- PNG rows as read (top row at t = 0),
    float images flipped (bottom row at t = 0) -- and the rectangle's
    texcoords (1, 0), (1, 1), (0, 0), (0, 1)."""
    import test_image_io as io
    arr, (P, F, N) = arrays_equivalent()
    rng = np.random.default_rng(8)
    if fmt == "png":
        px = rng.integers(0, 256, (6, 9, 3)).astype(np.uint8)
        (tmp_path / "tex.png").write_bytes(io.png_bytes(px, 2, [0, 1, 4]))
        tex = px.astype(np.float32) / np.float32(255)
    else:
        img = rng.uniform(0.05, 0.9, (6, 9, 3)).astype(np.float32)
        api.write_image(tmp_path / "tex.pfm", img)
        tex = np.ascontiguousarray(img[::-1])
    floor = arr.meshes[0]
    floor.texcoords = np.array([[1, 0], [1, 1], [0, 0], [0, 1]], np.float32)
    floor.material = arr.add_material(scenes.Material(albedo_texture=tex))
    text = cornell_xml(arr, "cuboid.obj")
    # the floor is the first rectangle: give its BSDF the texture
    first = text.index('<bsdf type="diffuse"><color name="albedo" value="0.725, 0.725, 0.725"/></bsdf>',
                       text.index('<mesh type="rectangle">'))
    text = (text[:first] + '<bsdf type="diffuse"><texture type="bitmap" name="albedo">'
            '<string name="filename" value="tex.%s"/></texture></bsdf>' % fmt
            + text[first + len('<bsdf type="diffuse"><color name="albedo" value="0.725, 0.725, 0.725"/></bsdf>'):])
    write_obj(tmp_path / "cuboid.obj", P, F, N)
    (tmp_path / "scene.xml").write_text(text)
    gx = api.Scene.from_xml(ctx, str(tmp_path / "scene.xml"))
    ga = api.Scene.from_data(ctx, arr)
    W, H = arr.camera.width, arr.camera.height
    xys = np.array([(x, y, s) for y in range(H) for x in range(W) for s in range(2)], np.int32)
    opts = abi.make_opts(seed=3, max_depth=6)
    La, _ = gx.li(opts, xys)
    Lb, _ = ga.li(opts, xys)
    np.testing.assert_array_equal(La, Lb)
    # and the texture is visible: differs from the untextured scene
    plain, _ = api.Scene.from_data(ctx, arrays_equivalent()[0]).li(opts, xys)
    assert np.abs(La - plain).max() > 0.05


def test_xml_texture_errors(ctx, tmp_path):
    (tmp_path / "t.pfm").write_bytes(b"PF\n1 1\n-1.0\n" + np.zeros(3, "<f4").tobytes())
    cases = [
        ("<bsdf type='mirror'><texture type='bitmap' name='albedo'><string name='filename' value='t.pfm'/>"
         "</texture></bsdf>", abi.DL_ERR_UNSUPPORTED),
        ("<bsdf type='aniso_ggx'><texture type='bitmap' name='normal'><string name='filename' value='t.pfm'/>"
         "</texture></bsdf>", abi.DL_ERR_UNSUPPORTED),            # tangent space by default
        ("<bsdf type='diffuse'><texture type='checkerboard' name='albedo'/></bsdf>", abi.DL_ERR_UNSUPPORTED),
        ("<bsdf type='diffuse'><texture type='bitmap' name='albedo'><string name='filename' value='none.png'/>"
         "</texture></bsdf>", abi.DL_ERR_IO),
    ]
    for k, (bsdf, status) in enumerate(cases):
        p = tmp_path / ("b%d.xml" % k)
        p.write_text("<scene><integrator type='path'/><camera type='virtual'><vector name='eye' value='0,0,3'/>"
                     "<vector name='lookat' value='0,0,0'/><vector name='up' value='0,1,0'/></camera>"
                     "<mesh type='rectangle'><vector name='pos' value='-1,-1,0'/><vector name='v0' value='2,0,0'/>"
                     "<vector name='v1' value='0,2,0'/>%s</mesh></scene>" % bsdf)
        with pytest.raises(api.DrawlabError) as e:
            api.Scene.from_xml(ctx, str(p))
        assert e.value.status == status, (k, e.value)
