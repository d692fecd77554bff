"""PBRT scene import (skwarka_gb300.pbrt), on the CPU: colour conversions
pinned to the reference's own code, the directives' transform semantics,
the camera and film, materials and their PBRT defaults, lights, volumes,
object instancing, orientation, the disk and cylinder meshes, Include, and the reported unsupported
features."""
import math
import os

import numpy as np
import pytest

from skwarka_gb300 import pbrt, scenes
from skwarka_gb300.render import MATTE, METAL, MIX, PLASTIC, SUBSTRATE, TRANSPARENT, UBER


def _ref():
    from oracle.api import Reference
    if not Reference.available():
        pytest.skip("oracle/_ref not built")
    return Reference()


def test_colours_match_the_reference_bit_for_bit():
    ref = _ref()
    rng = np.random.default_rng(3)
    rgb = rng.uniform(0, 20, size=(500, 3)).astype(np.float32)
    rgb[:50, 1] = rgb[:50, 0]
    rgb[:50, 2] = rgb[:50, 0]  # grey triples take the reference's special case
    want_r, want_e = ref.pbrt_rgb(0, rgb), ref.pbrt_rgb(1, rgb)
    got_r = np.array([pbrt.rgb_reflectance(c) for c in rgb])
    got_e = np.array([pbrt.rgb_emission(c) for c in rgb])
    assert np.array_equal(got_r, want_r)
    assert np.array_equal(got_e, want_e)


HEADER = '''
Scale -1 1 1
LookAt 0 -4 1  0 0 0.5  0 0 1
Camera "perspective" "float fov" [45]
Film "image" "integer xresolution" [64] "integer yresolution" [48]
Sampler "lowdiscrepancy" "integer pixelsamples" 4
WorldBegin
LightSource "point" "rgb I" [10 10 10] "point from" [1 1 3]
'''


def test_camera_film_and_light():
    s = pbrt.loads(HEADER + 'Shape "sphere"\nWorldEnd\n')
    cam = s.camera
    assert (cam.width, cam.height) == (64, 48)
    # the reference's rule: the fov spans the shorter image side
    want = 2.0 * math.atan(math.tan(math.radians(45.0) / 2.0) * (64.0 / 48.0))
    assert abs(cam.x_view_angle - want) < 1e-6
    # the camera sits at the LookAt eye, looks at the target, image y points down
    c2w = cam.camera_to_world
    assert np.allclose(c2w[:3, 3], (0, -4, 1))
    fwd = np.array([0, 4, -0.5]) / np.linalg.norm([0, 4, -0.5])
    assert np.allclose(c2w[:3, 2], fwd)
    assert c2w[2, 1] < 0  # camera +y (image rows) points down in the world
    assert np.allclose(c2w[:3, 0], (1, 0, 0))  # the handedness flip undone: image x = world +x here
    assert s.point_lights[0].position == (1.0, 1.0, 3.0)
    assert np.allclose(s.point_lights[0].intensity, pbrt.rgb_emission((10, 10, 10)))


def test_transforms_compose_like_pbrt():
    s = pbrt.loads(HEADER + '''
AttributeBegin
  Translate 1 2 3
  Rotate 90 0 0 1
  Scale 2 2 2
  Shape "trianglemesh" "point P" [1 0 0  0 1 0  0 0 1] "integer indices" [0 1 2]
AttributeEnd
Shape "trianglemesh" "point P" [1 0 0  0 1 0  0 0 1] "integer indices" [0 1 2]
WorldEnd''')
    v = s.prims[0].mesh.vertices
    # translate * rotate(z, 90) * scale(2): (1,0,0) -> (0,2,0) + t
    assert np.allclose(v, [[1, 4, 3], [-1, 2, 3], [1, 2, 5]], atol=1e-6)
    assert np.array_equal(s.prims[1].mesh.vertices, np.eye(3, dtype=np.float32))


def test_matrix_directives_and_coordinate_systems():
    s = pbrt.loads(HEADER + '''
CoordinateSystem "origin"
ConcatTransform [1 0 0 0  0 1 0 0  0 0 1 0  5 6 7 1]
Shape "trianglemesh" "point P" [0 0 0  1 0 0  0 1 0] "integer indices" [0 1 2]
CoordSysTransform "origin"
Transform [2 0 0 0  0 2 0 0  0 0 2 0  0 0 0 1]
Shape "trianglemesh" "point P" [0 0 0  1 0 0  0 1 0] "integer indices" [0 1 2]
WorldEnd''')
    assert np.allclose(s.prims[0].mesh.vertices[0], (5, 6, 7))  # column-major translation
    assert np.allclose(s.prims[1].mesh.vertices[1], (2, 0, 0))


def test_materials_and_defaults():
    s = pbrt.loads(HEADER + '''
Material "matte"
Shape "trianglemesh" "point P" [0 0 0 1 0 0 0 1 0] "integer indices" [0 1 2]
Material "plastic" "rgb Kd" [0.5 0.3 0.2] "float roughness" 0.05
Shape "trianglemesh" "point P" [0 0 0 1 0 0 0 1 0] "integer indices" [0 1 2]
Material "glass" "float index" 1.33
Shape "trianglemesh" "point P" [0 0 0 1 0 0 0 1 0] "integer indices" [0 1 2]
Material "mirror"
Shape "trianglemesh" "point P" [0 0 0 1 0 0 0 1 0] "integer indices" [0 1 2]
Material "metal"
Shape "trianglemesh" "point P" [0 0 0 1 0 0 0 1 0] "integer indices" [0 1 2]
Material "substrate" "float uroughness" 0.2 "float vroughness" 0.2
Shape "trianglemesh" "point P" [0 0 0 1 0 0 0 1 0] "integer indices" [0 1 2]
Material "uber" "rgb opacity" [0.5 0.5 0.5]
Shape "trianglemesh" "point P" [0 0 0 1 0 0 0 1 0] "integer indices" [0 1 2]
MakeNamedMaterial "a" "string type" "matte" "rgb Kd" [0.9 0.9 0.9]
MakeNamedMaterial "b" "string type" "plastic"
MakeNamedMaterial "ab" "string type" "mix" "string namedmaterial1" "a" "string namedmaterial2" "b" "rgb amount" [0.25 0.25 0.25]
NamedMaterial "ab"
Shape "trianglemesh" "point P" [0 0 0 1 0 0 0 1 0] "integer indices" [0 1 2]
Material "substrate" "float uroughness" 0.1 "float vroughness" 0.3
Shape "trianglemesh" "point P" [0 0 0 1 0 0 0 1 0] "integer indices" [0 1 2]
WorldEnd''')
    m = [s.materials[p.material] for p in s.prims]
    assert m[0].kind == MATTE and m[0].kd == (0.5, 0.5, 0.5) and m[0].sigma == 0.0
    assert m[1].kind == PLASTIC and m[1].kd == pbrt.rgb_reflectance((0.5, 0.3, 0.2)) and m[1].ks == (0.25,) * 3
    assert m[1].roughness == float(np.float32(0.05))
    assert m[2].kind == TRANSPARENT and m[2].kd == (1.0,) * 3 and m[2].ks == (1.0,) * 3
    assert m[2].refractive_index == float(np.float32(1.33))
    assert m[3].kind == TRANSPARENT and m[3].ks == (0.0,) * 3 and m[3].refractive_index == 1e10
    assert m[4].kind == METAL and m[4].eta == (1.165312, 0.950375, 0.35125) and m[4].roughness == 0.1
    # the factory's two-roughness constructor (AnisotropicDistribution) even for u == v
    assert m[5].kind == SUBSTRATE and m[5].kd == (0.5,) * 3 and m[5].roughness == float(np.float32(0.2))
    assert m[5].v_roughness == float(np.float32(0.2))
    assert m[6].kind == UBER and m[6].opacity == (0.5,) * 3 and m[6].kr == (0.0,) * 3
    assert m[7].kind == MIX and m[7].mix_scale == (0.25,) * 3
    a, b = (s.materials[i] for i in m[7].mix)
    assert a.kind == MATTE and a.kd == (float(np.float32(0.9)),) * 3 and b.kind == PLASTIC
    assert m[8].kind == SUBSTRATE and m[8].roughness == float(np.float32(0.1))
    assert m[8].v_roughness == float(np.float32(0.3)) and not s.warnings


def test_area_light_volume_and_constant_textures():
    s = pbrt.loads(HEADER + '''
Texture "k" "color" "constant" "rgb value" [0.2 0.4 0.6]
Texture "r" "float" "constant" "float value" 0.3
Texture "img" "color" "imagemap" "string filename" "x.png"
AttributeBegin
  AreaLightSource "diffuse" "rgb L" [4 4 4]
  Shape "trianglemesh" "point P" [0 0 2 1 0 2 0 1 2] "integer indices" [0 1 2]
AttributeEnd
Material "plastic" "texture Kd" "k" "texture roughness" "r"
Shape "trianglemesh" "point P" [0 0 0 1 0 0 0 1 0] "integer indices" [0 1 2]
Volume "homogeneous" "rgb sigma_a" [0.05 0.05 0.05] "rgb sigma_s" [0.2 0.2 0.2] "float g" 0.3 "point p0" [-1 -1 -1] "point p1" [1 1 1] "rgb Le" [0.1 0.1 0.1]
VolumeIntegrator "single" "float stepsize" 0.02
WorldEnd''')
    assert np.allclose(s.prims[0].emission, pbrt.rgb_emission((4, 4, 4)))
    assert s.prims[1].emission == (0.0, 0.0, 0.0)
    m = s.materials[s.prims[1].material]
    assert m.kd == pbrt.rgb_reflectance((0.2, 0.4, 0.6)) and m.roughness == float(np.float32(0.3))
    med = s.medium
    assert med.lo == (-1.0, -1.0, -1.0) and med.hi == (1.0, 1.0, 1.0)
    assert med.sigma_a == (float(np.float32(0.05)),) * 3 and med.g == float(np.float32(0.3))
    assert med.step == float(np.float32(0.02))
    assert any("imagemap" in w for w in s.warnings)


def test_sphere_shape_is_the_reference_mesh():
    s = pbrt.loads(HEADER + 'Translate 0 0 1\nShape "sphere" "float radius" 0.5\nWorldEnd')
    sv, st = scenes.sphere_mesh(5)
    p = s.prims[0]
    assert np.array_equal(p.mesh.triangles, st.astype(np.int32))
    assert np.array_equal(p.mesh.vertices, (sv * 0.5 + [0, 0, 1]).astype(np.float32))
    assert np.allclose(p.vertex_normals, sv, atol=1e-6)


def test_orientation_flips():
    base = 'Shape "trianglemesh" "point P" [0 0 0 1 0 0 0 1 0] "integer indices" [0 1 2]\n'
    s = pbrt.loads(HEADER + base + 'ReverseOrientation\n' + base + 'WorldEnd')
    assert s.prims[0].mesh.triangles.tolist() == [[0, 1, 2]]
    assert s.prims[1].mesh.triangles.tolist() == [[0, 2, 1]]
    # a mirroring transform flips the sphere's winding (its geometric normals
    # stay outward) and negates its shading normals, as Sphere::BuildMesh
    # does for an orientation-inverting transform (Shapes/Sphere.cpp:177-185)
    s = pbrt.loads(HEADER + 'Scale 1 1 -1\nShape "sphere"\nWorldEnd')
    p = s.prims[0]
    v, t = p.mesh.vertices.astype(np.float64), p.mesh.triangles
    n = np.cross(v[t[:, 1]] - v[t[:, 0]], v[t[:, 2]] - v[t[:, 0]])
    c = v[t].mean(1)
    assert (np.einsum("ij,ij->i", n, c) > 0).all()
    assert (np.einsum("ij,ij->i", p.vertex_normals.astype(np.float64), v) < 0).all()


def test_object_instances_share_their_mesh():
    s = pbrt.loads(HEADER + '''
ObjectBegin "tri"
Translate 0 0 1
Shape "trianglemesh" "point P" [0 0 0 1 0 0 0 1 0] "integer indices" [0 1 2]
ObjectEnd
Translate 2 0 0
ObjectInstance "tri"
Translate 2 0 0
ObjectInstance "tri"
WorldEnd''')
    a, b = s.prims
    assert a.mesh is b.mesh
    assert np.allclose(a.mesh.vertices[0], (0, 0, 1))
    assert np.allclose(a.mesh_to_world[:3, 3], (2, 0, 0)) and np.allclose(b.mesh_to_world[:3, 3], (4, 0, 0))


def test_include_and_errors(tmp_path):
    (tmp_path / "geo.pbrt").write_text(
        'Shape "trianglemesh" "point P" [0 0 0 1 0 0 0 1 0] "integer indices" [0 1 2] "normal N" [0 0 2 0 0 2 0 0 2]\n')
    (tmp_path / "scene.pbrt").write_text(HEADER + 'Include "geo.pbrt"\nWorldEnd\n')
    s = pbrt.load(str(tmp_path / "scene.pbrt"))
    assert len(s.prims) == 1 and np.allclose(s.prims[0].vertex_normals, [[0, 0, 1]] * 3)
    with pytest.raises(pbrt.PbrtError):
        pbrt.loads(HEADER + 'Shape "trianglemesh" "point P" [0 0 0\nWorldEnd')  # unterminated bracket
    with pytest.raises(pbrt.PbrtError):
        pbrt.loads(HEADER + 'WorldEnd')  # no primitives
    with pytest.raises(pbrt.PbrtError):
        pbrt.loads('WorldBegin\nShape "sphere"\nWorldEnd')  # no lights
    s = pbrt.loads(HEADER + 'Shape "cone"\nLightSource "spot"\nShape "sphere"\nWorldEnd')
    assert any('shape "cone"' in w for w in s.warnings) and any('light "spot"' in w for w in s.warnings)


def test_disk_and_cylinder_are_the_reference_meshes():
    s = pbrt.loads(HEADER + '''
Shape "disk" "float radius" 2 "float height" 1
Shape "disk" "float innerradius" 0.5 "float phimax" 180
Shape "cylinder" "float radius" 0.5 "float zmin" 0 "float zmax" 2
WorldEnd''')
    full, ring, cyl = s.prims
    # 360 segments; the factories pass phimax / pi (clamped to 2 pi): a full turn at 180 degrees too
    assert full.mesh.triangles.shape == (360, 3) and ring.mesh.triangles.shape == (720, 3)
    assert np.allclose(full.mesh.vertices[0], (0, 0, 1)) and np.allclose(np.abs(full.mesh.vertices[1:, :2]).max(), 2)
    r = np.linalg.norm(ring.mesh.vertices[:, :2], axis=1)
    assert np.allclose(r[0::2], 0.5, atol=1e-6) and np.allclose(r[1::2], 1.0, atol=1e-6)
    assert np.allclose(ring.mesh.vertices[-1], ring.mesh.vertices[1], atol=1e-6)  # the last step closes the ring
    for p in (full, ring):  # flat disks face +z and carry no shading normals
        v, t = p.mesh.vertices.astype(np.float64), p.mesh.triangles
        n = np.cross(v[t[:, 1]] - v[t[:, 0]], v[t[:, 2]] - v[t[:, 0]])
        assert (n[:, 2] > 0).all() and p.vertex_normals is None
    v, t = cyl.mesh.vertices.astype(np.float64), cyl.mesh.triangles
    assert np.allclose([v[:, 2].min(), v[:, 2].max()], [0, 2]) and np.allclose(np.linalg.norm(v[:, :2], axis=1), 0.5)
    n = np.cross(v[t[:, 1]] - v[t[:, 0]], v[t[:, 2]] - v[t[:, 0]])
    c = v[t].mean(1)
    assert (np.einsum("ij,ij->i", n[:, :2], c[:, :2]) > 0).all()  # outward
    assert np.allclose(cyl.vertex_normals[:, :2] * 0.5, v[:, :2], atol=1e-6)


def test_shading_tangent_sources():
    s = pbrt.loads(HEADER + '''
Shape "trianglemesh" "point P" [0 0 0 1 0 0 0 1 0] "integer indices" [0 1 2]
Shape "trianglemesh" "point P" [0 0 0 1 0 0 0 1 0] "integer indices" [0 1 2] "float uv" [0 0 0 1 1 0]
Shape "sphere"
Shape "cylinder"
Shape "disk"
WorldEnd''')
    a, b, sph, cyl, dsk = s.prims
    # PBRT's default uvs (0, 0), (1, 0), (1, 1): u increases along the first edge
    assert a.triangle_uvs.tolist() == [[0, 0, 1, 0, 1, 1]] and a.vertex_tangents is None
    assert b.triangle_uvs.tolist() == [[0, 0, 0, 1, 1, 0]]
    # the shapes' tangents: (0, 0, 1) x v for the sphere, (-sin, cos, 0) around the cylinder and disk
    v = sph.mesh.vertices.astype(np.float64)
    want = np.cross([0.0, 0.0, 1.0], v)
    ln = np.linalg.norm(want, axis=1)
    ok = ln > 1e-6
    assert np.allclose(sph.vertex_tangents[ok], want[ok] / ln[ok, None], atol=1e-6)
    assert np.allclose(sph.vertex_tangents[~ok], [1, 0, 0])
    c = cyl.mesh.vertices[:, :2].astype(np.float64)
    assert np.allclose(cyl.vertex_tangents[:, :2], np.stack([-c[:, 1], c[:, 0]], 1), atol=1e-6)
    assert np.allclose(dsk.vertex_tangents[0], 0) and np.allclose(np.abs(dsk.vertex_tangents[1:, 2]), 0)
    assert cyl.triangle_uvs is None and sph.triangle_uvs is None
