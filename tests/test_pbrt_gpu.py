"""A PBRT scene file rendered on the GPU: the imported scene renders exactly
as the same scene built through the API (same meshes, materials, lights and
camera give the same image bit for bit), and a point light over a white
plane written as a PBRT file gives the known answer L = I / d^2 / pi."""
import numpy as np
import pytest

from skwarka_gb300 import pbrt
from skwarka_gb300.accel import TriangleMesh
from skwarka_gb300.render import Camera, Material, PointLight, RenderPrimitive, RenderScene, PLASTIC

pytestmark = pytest.mark.gpu

SCENE = '''
LookAt 0 -3 2  0 0 0.3  0 0 1
Camera "perspective" "float fov" [50]
Film "image" "integer xresolution" [48] "integer yresolution" [32]
WorldBegin
LightSource "point" "color I" [6 5 4] "point from" [1.5 -1 3]
AttributeBegin
  AreaLightSource "diffuse" "rgb L" [3 3 3]
  Translate 0 0 2.8
  ReverseOrientation
  Shape "trianglemesh" "point P" [-0.4 -0.4 0  0.4 -0.4 0  0.4 0.4 0  -0.4 0.4 0] "integer indices" [0 1 2 0 2 3]
AttributeEnd
Material "matte" "rgb Kd" [0.6 0.6 0.5]
Shape "trianglemesh" "point P" [-3 -3 0  3 -3 0  3 3 0  -3 3 0] "integer indices" [0 1 2 0 2 3]
Material "plastic" "rgb Kd" [0.3 0.5 0.7] "float roughness" 0.1
Translate 0 0 0.6
Shape "sphere" "float radius" 0.6
WorldEnd
'''


def test_imported_scene_renders_like_the_same_scene_built_directly(gpu):
    s = pbrt.loads(SCENE)
    assert not s.warnings
    img = s.render_scene().render_direct(s.camera, 2, 2, seed=5).cpu().numpy()
    # the same scene through the API, from the importer's own arrays
    prims = [RenderPrimitive(TriangleMesh(p.mesh.vertices.copy(), p.mesh.triangles.copy()), p.material,
                             p.mesh_to_world, p.vertex_normals, None, p.emission, p.vertex_tangents,
                             p.triangle_uvs) for p in s.prims]
    mats = [Material(**m.__dict__) for m in s.materials]
    lights = [PointLight(l.position, l.intensity) for l in s.point_lights]
    cam = Camera(s.camera.camera_to_world.copy(), s.camera.x_view_angle, s.camera.width, s.camera.height)
    img2 = RenderScene(prims, mats, lights).render_direct(cam, 2, 2, seed=5).cpu().numpy()
    assert img.shape == (32, 48, 3)
    assert np.array_equal(img, img2)
    assert img.mean() > 0.0 and np.isfinite(img).all()
    assert s.materials[s.prims[2].material].kind == PLASTIC


def test_point_light_known_answer_from_a_pbrt_file(gpu):
    """A point light at distance 9 above a white Lambertian plane
    (DirectLightingIntegrator.test.h:46-71): L = I / 81 / pi, with I the
    reference's conversion of "rgb I [100 100 100]" (sRGB D65 -> spectrum)."""
    s = pbrt.loads('''
LookAt 0 0 5  0 0 0  0 1 0
Camera "perspective" "float fov" [0.05]
Film "image" "integer xresolution" [4] "integer yresolution" [4]
WorldBegin
LightSource "point" "rgb I" [100 100 100] "point from" [0 0 9]
Material "matte" "rgb Kd" [1 1 1]
Shape "trianglemesh" "point P" [-50 -50 0  50 -50 0  50 50 0  -50 50 0] "integer indices" [0 1 2 0 2 3]
WorldEnd
''')
    img = s.render_scene().render_direct(s.camera, 1, 1).cpu().numpy()
    want = np.array(pbrt.rgb_emission((100, 100, 100))) / 81.0 / np.pi
    assert np.allclose(img, want[None, None, :], rtol=1e-4), (img.mean((0, 1)), want)
