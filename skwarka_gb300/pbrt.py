"""PBRT scene import: a pbrt-v2 scene file into this library's render scene.

Restates the reference's importer (CADImport/SceneImporters/
PbrtSceneImporter*, the `PbrtSceneImporter` class): the same directives,
transform semantics, parameter types and defaults, and the same mapping of
PBRT's shapes, materials, lights, camera, film and volumes onto the
renderer's types, for the part of PBRT that the renderer here implements:

* shapes: ``trianglemesh`` (P, indices, N), ``sphere`` (the reference's
  sphere mesh at 5 subdivisions, ShapeFactory.h:62-78), ``disk`` and
  ``cylinder`` (the reference's 360-step meshes) -- meshes in world
  space as the reference builds them (Convert<float>(Transform(P)) in
  double); ``ReverseOrientation`` and orientation-inverting transforms flip
  a mesh's winding (the reference's TriangleMesh orientation flag);
* materials: matte, plastic, glass, mirror, metal, substrate (isotropic),
  uber, mix, measured (MaterialFactory.h) with PBRT's defaults;
* lights: point lights and diffuse area lights (``AreaLightSource``
  attaches emission to the shapes that follow); spot, distant, infinite
  and goniometric lights are reported and skipped;
* camera: ``perspective`` with the reference's field-of-view rule
  (CameraFactory.h:52-63) and the camera-space flip of PBRT's left-handed
  ``Scale -1 1 1`` (PbrtSceneImporter_hooks.cpp:136-150); film ``image``
  resolution;
* volumes: ``homogeneous`` (VolumeRegionFactory.h:45-56) as the medium;
* object instancing (``ObjectBegin`` / ``ObjectInstance``): the
  instances share their mesh, with the instance's transform;
* colours: ``rgb`` / ``color`` and ``xyz`` values converted as the
  reference's ParamSet converts them (PbrtParamSet.cpp:99-153: a grey
  reflectance as is, else sRGB with white point E, emission sRGB with D65,
  then XYZ to the renderer's three spectrum coefficients).

What the renderer does not implement (textures other than constants,
other shapes, lights, cameras and volumes) is listed in
``PbrtScene.warnings`` and skipped, as the reference logs and skips the
features it does not support.
"""
from __future__ import annotations

import math
import os
import re
from dataclasses import dataclass, field

import numpy as np

from .accel import TriangleMesh
from .render import (MATTE, MEASURED, METAL, MIX, PLASTIC, SUBSTRATE, TRANSPARENT, UBER, Camera, Material,
                     MeasuredBRDF, Medium, PointLight, RenderPrimitive, RenderScene)
from . import scenes


# ---------------------------------------------------------------- colours --
def _hexm(rows):
    return np.array([[float.fromhex(h) for h in r] for r in rows], np.float64)


# RGB -> XYZ of the reference's sRGB colour systems (Core/Color.cpp:17-18,
# ColorSystem::ColorSystem, Core/Color.h:274-330), white point E
# (reflectances) and D65 (emission), and XYZ -> the renderer's spectrum
# coefficients (SpectrumRoutines::XYZToSpectrum): the reference's doubles.
_RGB_TO_XYZ_E = _hexm([["0x1.fcd8dcf9c3460p-2", "0x1.5b3a5407f3635p-2", "0x1.4fd99dfc92adap-3"],
                       ["0x1.065fd1f0c8b0dp-2", "0x1.5b3a5407f3631p-1", "0x1.0cae17fd42268p-4"],
                       ["0x1.7da2a5bb5271ep-6", "0x1.cef8700a99da9p-4", "0x1.ba33dcd0d2310p-1"]])
_RGB_TO_XYZ_D65 = _hexm([["0x1.a649c610130a0p-2", "0x1.6e2a96ccdcb16p-2", "0x1.719fe95deffb8p-3"],
                         ["0x1.b37c144093a15p-3", "0x1.6e2a96ccdcb1bp-1", "0x1.27b32117f332cp-4"],
                         ["0x1.3cb7548c0e3adp-6", "0x1.e838c911263fep-4", "0x1.e6ac26776ae6bp-1"]])
_XYZ_TO_SPECTRUM = _hexm([["0x1.368e683d1c8e4p-4", "-0x1.0c40314b9028fp-3", "0x1.0e07e946862fdp+0"],
                          ["-0x1.432fb70f599bep+0", "0x1.14a5623a99345p+1", "0x1.9e954c8d546b1p-4"],
                          ["0x1.040236acfe51bp+1", "-0x1.6cd6c8f911e96p-1", "-0x1.4672dbc94b232p-2"]])


def _mat3(m, v):
    """Matrix3x3 * vector as the reference evaluates it: (m0 v0 + m1 v1) + m2 v2 per row."""
    return tuple(float((m[i, 0] * v[0] + m[i, 1] * v[1]) + m[i, 2] * v[2]) for i in range(3))


def rgb_reflectance(rgb) -> tuple:
    """A PBRT rgb reflectance (ParamSet::AddRGBSpectrumCoef): float values; a
    grey triple as is, else sRGB (white E) -> XYZ -> spectrum coefficients."""
    r, g, b = (float(np.float32(x)) for x in rgb)
    if r == g and r == b:
        return (r, r, r)
    return _mat3(_XYZ_TO_SPECTRUM, _mat3(_RGB_TO_XYZ_E, (r, g, b)))


def rgb_emission(rgb) -> tuple:
    """A PBRT rgb emission (ParamSet::AddRGBSpectrum): sRGB (white D65) -> XYZ -> spectrum."""
    v = tuple(float(np.float32(x)) for x in rgb)
    return _mat3(_XYZ_TO_SPECTRUM, _mat3(_RGB_TO_XYZ_D65, v))


def xyz_spectrum(xyz) -> tuple:
    """A PBRT xyz value (ParamSet::AddXYZSpectrum / AddXYZSpectrumCoef)."""
    return _mat3(_XYZ_TO_SPECTRUM, tuple(float(np.float32(x)) for x in xyz))


# ------------------------------------------------------------- transforms --
def translate(d) -> np.ndarray:
    m = np.eye(4)
    m[:3, 3] = d
    return m


def scale(s) -> np.ndarray:
    return np.diag([float(s[0]), float(s[1]), float(s[2]), 1.0])


def rotate(angle_deg: float, axis) -> np.ndarray:
    """MakeRotation(DegreesToRadians(angle), axis) (Math/Transform.cpp:78-112)."""
    a = np.asarray(axis, np.float64)
    a = a / math.sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2])
    t = float(angle_deg) * (math.pi / 180.0)
    s, c = math.sin(t), math.cos(t)
    x, y, z = a
    m = np.eye(4)
    m[0, :3] = [x * x + (1.0 - x * x) * c, x * y * (1.0 - c) - z * s, x * z * (1.0 - c) + y * s]
    m[1, :3] = [x * y * (1.0 - c) + z * s, y * y + (1.0 - y * y) * c, y * z * (1.0 - c) - x * s]
    m[2, :3] = [x * z * (1.0 - c) - y * s, y * z * (1.0 - c) + x * s, z * z + (1.0 - z * z) * c]
    return m


def look_at(eye, target, up) -> np.ndarray:
    """MakeLookAt (Math/Transform.cpp:138-166): the world-to-camera matrix,
    camera x right, y down (image rows), z forward."""
    eye = np.asarray(eye, np.float64)
    d = np.asarray(target, np.float64) - eye
    d = d / math.sqrt(float(d @ d))
    r = np.cross(d, np.asarray(up, np.float64))
    r = r / math.sqrt(float(r @ r))
    new_up = np.cross(r, d)
    m = np.eye(4)
    m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3] = r, -new_up, d, eye
    return np.linalg.inv(m)


def inverts_orientation(m: np.ndarray) -> bool:
    """Transform::InvertsOrientation (Math/Transform.h:202-214)."""
    det = ((m[0, 0] * (m[1, 1] * m[2, 2] - m[1, 2] * m[2, 1]))
           - (m[0, 1] * (m[1, 0] * m[2, 2] - m[1, 2] * m[2, 0]))
           + (m[0, 2] * (m[1, 0] * m[2, 1] - m[1, 1] * m[2, 0])))
    return det < 0.0


def apply_point(m: np.ndarray, p: np.ndarray) -> np.ndarray:
    """Transform::operator()(Point3D_d) on (n, 3) doubles, evaluated in the
    reference's order, with the homogeneous divide when w != 1."""
    x, y, z = p[:, 0], p[:, 1], p[:, 2]
    out = np.stack([((m[i, 0] * x + m[i, 1] * y) + m[i, 2] * z) + m[i, 3] for i in range(3)], 1)
    w = ((m[3, 0] * x + m[3, 1] * y) + m[3, 2] * z) + m[3, 3]
    if np.any(w != 1.0):
        out = np.where((w == 1.0)[:, None], out, out / w[:, None])
    return out


def apply_vector(m: np.ndarray, v: np.ndarray) -> np.ndarray:
    """Transform::operator()(Vector3D_d), normalised (the shapes' tangents)."""
    x, y, z = v[:, 0], v[:, 1], v[:, 2]
    out = np.stack([(m[i, 0] * x + m[i, 1] * y) + m[i, 2] * z for i in range(3)], 1)
    ln = np.sqrt((out * out).sum(1))
    return np.where(ln[:, None] > 0, out / np.where(ln > 0, ln, 1.0)[:, None], out)


def apply_normal(m: np.ndarray, n: np.ndarray) -> np.ndarray:
    """Transform::TransformNormal: the inverse transpose, normalised."""
    inv = np.linalg.inv(m)
    x, y, z = n[:, 0], n[:, 1], n[:, 2]
    out = np.stack([(inv[0, i] * x + inv[1, i] * y) + inv[2, i] * z for i in range(3)], 1)
    return out / np.sqrt((out * out).sum(1))[:, None]


# ------------------------------------------------------------------ shapes --
def disk_mesh(m: np.ndarray, max_phi: float, inner: float, subdivisions: int = 360):
    """Disk::BuildMesh (Shapes/Disk.cpp:57-171) through transform m: the
    unit disk (or the ring from `inner` to 1) in the z = 0 plane, its phi
    stepped by accumulation; flat (no shading normals).  Returns float32
    vertices, int32 triangles and float32 vertex tangents (T(-sin, cos, 0)
    normalised; the centre's is 0)."""
    d_phi = max_phi / subdivisions
    ring, phi = [], 0.0
    for _ in range(subdivisions + 1):
        ring.append((math.cos(phi), math.sin(phi)))
        phi += d_phi
    c = np.array(ring, np.float64)
    tang = apply_vector(m, np.stack([-c[:, 1], c[:, 0], np.zeros(len(c))], 1))
    i = np.arange(subdivisions)
    if inner == 0.0:
        pts = np.concatenate([[[0.0, 0.0, 0.0]], np.stack([c[:, 0], c[:, 1], np.zeros(len(c))], 1)])
        tan = np.concatenate([[[0.0, 0.0, 0.0]], tang])
        tris = np.stack([np.zeros(subdivisions, np.int64), i + 1, i + 2], 1)
    else:
        pts = np.empty((2 * len(c), 3))
        pts[0::2] = np.stack([inner * c[:, 0], inner * c[:, 1], np.zeros(len(c))], 1)
        pts[1::2] = np.stack([c[:, 0], c[:, 1], np.zeros(len(c))], 1)
        tan = np.repeat(tang, 2, axis=0)
        tris = np.concatenate([np.stack([2 * i, 2 * i + 1, 2 * i + 3], 1),
                               np.stack([2 * i + 3, 2 * i + 2, 2 * i], 1)], 1).reshape(-1, 3)
    return apply_point(m, pts).astype(np.float32), tris.astype(np.int32), tan.astype(np.float32)


def cylinder_mesh(m: np.ndarray, max_phi: float, subdivisions: int = 360):
    """Cylinder::BuildMesh (Shapes/Cylinder.cpp:48-103) through transform m:
    the unit cylinder from z = 0 to 1, smooth.  Returns float32 vertices,
    int32 triangles, float32 shading normals (negated for a mirroring m, as
    the reference does) and tangents (T(-sin, cos, 0) normalised)."""
    d_phi = max_phi / subdivisions
    ang, phi = [], 0.0
    for _ in range(subdivisions + 1):
        ang.append((math.cos(phi), math.sin(phi)))
        phi += d_phi
    c = np.array(ang, np.float64)
    pts = np.empty((2 * len(c), 3))
    pts[0::2] = np.stack([c[:, 0], c[:, 1], np.zeros(len(c))], 1)
    pts[1::2] = np.stack([c[:, 0], c[:, 1], np.ones(len(c))], 1)
    sign = -1.0 if inverts_orientation(m) else 1.0
    nrm = sign * apply_normal(m, np.stack([c[:, 0], c[:, 1], np.zeros(len(c))], 1))
    tan = apply_vector(m, np.stack([-c[:, 1], c[:, 0], np.zeros(len(c))], 1))
    i = np.arange(subdivisions)
    tris = np.concatenate([np.stack([2 * i + 1, 2 * i, 2 * i + 2], 1),
                           np.stack([2 * i + 2, 2 * i + 3, 2 * i + 1], 1)], 1).reshape(-1, 3)
    return (apply_point(m, pts).astype(np.float32), tris.astype(np.int32),
            np.repeat(nrm, 2, axis=0).astype(np.float32), np.repeat(tan, 2, axis=0).astype(np.float32))


def _max_phi(phimax_deg: float) -> float:
    """The factories pass phimax * INV_PI (ShapeFactory.h:86, :100), which the
    shapes clamp to [0, 2 pi]; kept as the reference computes it."""
    return max(0.0, min(2.0 * math.pi, phimax_deg * (1.0 / math.pi)))


# ------------------------------------------------------------- the parser --
_TOKEN = re.compile(r'\s*(?:#[^\n]*|"([^"]*)"|(\[)|(\])|([^\s\[\]"#]+))')

_DIRECTIVES = {
    "Accelerator", "ActiveTransform", "AreaLightSource", "AttributeBegin", "AttributeEnd", "Camera",
    "ConcatTransform", "CoordinateSystem", "CoordSysTransform", "Film", "Identity", "Include", "LightSource",
    "LookAt", "MakeNamedMaterial", "Material", "NamedMaterial", "ObjectBegin", "ObjectEnd", "ObjectInstance",
    "PixelFilter", "Renderer", "ReverseOrientation", "Rotate", "Sampler", "Scale", "Shape", "SurfaceIntegrator",
    "Texture", "TransformBegin", "TransformEnd", "Transform", "TransformTimes", "Translate", "Volume",
    "VolumeIntegrator", "WorldBegin", "WorldEnd",
}


class PbrtError(ValueError):
    """A malformed scene file."""


def _tokens(text: str):
    pos, n = 0, len(text)
    while pos < n:
        m = _TOKEN.match(text, pos)
        if not m or m.end() == pos:
            if text[pos:].strip() == "":
                return
            raise PbrtError(f"cannot read the scene at offset {pos}: {text[pos:pos + 40]!r}")
        pos = m.end()
        if m.group(1) is not None:
            yield ("s", m.group(1))
        elif m.group(2):
            yield ("[", None)
        elif m.group(3):
            yield ("]", None)
        elif m.group(4):
            yield ("w", m.group(4))


def _commands(text: str):
    """(directive, [arguments]) with arguments as ('s', str), ('w', word) or
    ('l', [tokens of a bracketed list])."""
    cur = None
    it = iter(_tokens(text))
    for kind, val in it:
        if kind == "w" and val in _DIRECTIVES:
            if cur is not None:
                yield cur
            cur = (val, [])
            continue
        if cur is None:
            raise PbrtError(f"a value before any directive: {val!r}")
        if kind == "[":
            items = []
            for k2, v2 in it:
                if k2 == "]":
                    break
                if k2 == "[":
                    raise PbrtError("nested brackets")
                items.append((k2, v2))
            else:
                raise PbrtError("unterminated bracket")
            cur[1].append(("l", items))
        elif kind == "]":
            raise PbrtError("unmatched ]")
        else:
            cur[1].append((kind, val))
    if cur is not None:
        yield cur


def _values(arg):
    return arg[1] if arg[0] == "l" else [arg]


class _Params:
    """A parameter list: {name: (type, [raw values])} (the reference's ParamSet)."""

    def __init__(self, args):
        self.items = {}
        i = 0
        while i < len(args):
            kind, val = args[i]
            if kind != "s":
                raise PbrtError(f"expected a \"type name\" string, found {val!r}")
            parts = val.split()
            if len(parts) != 2:
                raise PbrtError(f"invalid parameter declaration {val!r}")
            if i + 1 >= len(args):
                raise PbrtError(f"parameter {val!r} has no value")
            t, name = parts
            if t == "color":
                t = "rgb"
            self.items[name] = (t, [v for _, v in _values(args[i + 1])])
            i += 2

    def _get(self, name, types):
        it = self.items.get(name)
        if it is None or it[0] not in types:
            return None
        return it[1]

    def floats(self, name):
        v = self._get(name, ("float",))
        return None if v is None else [float(np.float32(float(x))) for x in v]  # std::stof

    def float1(self, name, default):
        v = self.floats(name)
        return v[0] if v else default

    def ints(self, name):
        v = self._get(name, ("integer",))
        return None if v is None else [int(x) for x in v]

    def int1(self, name, default):
        v = self.ints(name)
        return v[0] if v else default

    def string1(self, name, default=""):
        v = self._get(name, ("string", "texture"))
        return v[0] if v else default

    def points(self, name, types=("point",)):
        v = self._get(name, types)
        if v is None:
            return None
        a = np.array([float(x) for x in v], np.float64)  # std::stod
        return a[: len(a) // 3 * 3].reshape(-1, 3)

    def point1(self, name, default):
        v = self.points(name)
        return tuple(v[0]) if v is not None and len(v) else tuple(default)

    def bool1(self, name, default):
        v = self._get(name, ("bool",))
        return (v[0] == "true") if v else default

    def coef(self, name, default, textures):
        """A reflectance-like value (FindOneSpectrumCoef / GetSpectrumCoefTexture)."""
        it = self.items.get(name)
        if it is None:
            return tuple(float(x) for x in default)
        t, v = it
        if t == "rgb":
            return rgb_reflectance([float(x) for x in v[:3]])
        if t == "xyz":
            return xyz_spectrum([float(x) for x in v[:3]])
        if t == "texture":
            tex = textures.get(v[0])
            if tex is None:
                raise _Unsupported(f"texture \"{v[0]}\" is not a constant texture")
            return tex
        if t == "spectrum":
            raise _Unsupported(f"\"{t} {name}\" values")
        return tuple(float(x) for x in default)  # another type: not a spectrum (the default)

    def emission(self, name, default):
        """An emitted spectrum (FindOneSpectrum): rgb in sRGB D65."""
        it = self.items.get(name)
        if it is None:
            return tuple(float(x) for x in default)
        t, v = it
        if t == "rgb":
            return rgb_emission([float(x) for x in v[:3]])
        if t == "xyz":
            return xyz_spectrum([float(x) for x in v[:3]])
        if t == "spectrum":
            raise _Unsupported(f"\"{t} {name}\" values")
        return tuple(float(x) for x in default)  # another type: not a spectrum (the default)

    def scalar(self, name, default, textures):
        """A float parameter or a constant float texture (GetFloatTexture)."""
        it = self.items.get(name)
        if it is None:
            return float(default)
        t, v = it
        if t == "float":
            return float(np.float32(float(v[0])))
        if t == "texture":
            tex = textures.get(v[0])
            if tex is None:
                raise _Unsupported(f"texture \"{v[0]}\" is not a constant texture")
            return float(tex[0])
        raise _Unsupported(f"\"{t} {name}\" values")

    def merged(self, base: "_Params") -> "_Params":
        """A shape's parameters over its material's (TextureParams lookup order)."""
        p = _Params([])
        p.items = dict(base.items)
        p.items.update(self.items)
        return p


class _Unsupported(Exception):
    pass


@dataclass
class PbrtScene:
    """The imported scene: render primitives, materials, point lights, the
    medium, the camera and its film size, and what was skipped."""
    prims: list = field(default_factory=list)
    materials: list = field(default_factory=list)
    point_lights: list = field(default_factory=list)
    medium: Medium | None = None
    camera: Camera | None = None
    warnings: list = field(default_factory=list)

    def render_scene(self, ctx=None) -> RenderScene:
        """The scene on the GPU (RenderScene)."""
        return RenderScene(self.prims, self.materials, self.point_lights, ctx=ctx, medium=self.medium)


@dataclass
class _State:
    material: tuple = ("matte", None)   # (name, _Params) or ("@named", name)
    area_light: tuple | None = None     # (name, _Params)
    reverse: bool = False
    float_textures: dict = field(default_factory=dict)
    color_textures: dict = field(default_factory=dict)
    named: dict = field(default_factory=dict)

    def copy(self) -> "_State":
        return _State(self.material, self.area_light, self.reverse, dict(self.float_textures),
                      dict(self.color_textures), dict(self.named))


# PBRT's copper, the metal default (MaterialFactory.h, _CreateMetalMaterial)
_COPPER_ETA = (1.165312, 0.950375, 0.351250)
_COPPER_K = (2.397625, 2.576500, 3.010750)


class _Importer:
    def __init__(self, ctx=None, device=True):
        self.ctx, self.device = ctx, device
        self.out = PbrtScene()
        self.ctm = np.eye(4)
        self.named_cs = {}
        self.gs = _State()
        self.stack = []        # (state, ctm) pushed by AttributeBegin
        self.tstack = []       # ctm pushed by TransformBegin
        self.camera = ("perspective", _Params([]), np.eye(4))
        self.film = _Params([])
        self.world = False
        self.instances = {}
        self.current_instance = None
        self.material_index = {}
        self.medium_step = None

    def warn(self, msg):
        if msg not in self.out.warnings:
            self.out.warnings.append(msg)

    # ---- materials (MaterialFactory.h)
    def _material(self, name: str, p: _Params, key) -> int:
        if key in self.material_index:
            return self.material_index[key]
        m = self._make_material(name, p)
        self.out.materials.append(m)
        self.material_index[key] = len(self.out.materials) - 1
        return self.material_index[key]

    def _make_material(self, name: str, p: _Params) -> Material:
        ct, ft = self.gs.color_textures, self.gs.float_textures
        try:
            if name == "matte":
                return Material(MATTE, kd=p.coef("Kd", (0.5,) * 3, ct), sigma=p.scalar("sigma", 0.0, ft))
            if name == "plastic":
                return Material(PLASTIC, kd=p.coef("Kd", (0.25,) * 3, ct), ks=p.coef("Ks", (0.25,) * 3, ct),
                                roughness=p.scalar("roughness", 0.1, ft))
            if name == "glass":
                return Material(TRANSPARENT, kd=p.coef("Kr", (1.0,) * 3, ct), ks=p.coef("Kt", (1.0,) * 3, ct),
                                refractive_index=p.scalar("index", 1.5, ft))
            if name == "mirror":
                return Material(TRANSPARENT, kd=p.coef("Kr", (1.0,) * 3, ct), ks=(0.0, 0.0, 0.0),
                                refractive_index=1e10)
            if name == "metal":
                return Material(METAL, eta=p.coef("eta", _COPPER_ETA, ct), k=p.coef("k", _COPPER_K, ct),
                                roughness=p.scalar("roughness", 0.1, ft))
            if name == "substrate":
                # the factory takes the two-roughness constructor
                # (AnisotropicDistribution), whatever the two values
                u, v = p.scalar("uroughness", 0.1, ft), p.scalar("vroughness", 0.1, ft)
                return Material(SUBSTRATE, kd=p.coef("Kd", (0.5,) * 3, ct), ks=p.coef("Ks", (0.5,) * 3, ct),
                                roughness=u, v_roughness=max(v, 1e-30))
            if name == "uber":
                return Material(UBER, kd=p.coef("Kd", (0.25,) * 3, ct), ks=p.coef("Ks", (0.25,) * 3, ct),
                                kr=p.coef("Kr", (0.0,) * 3, ct), roughness=p.scalar("roughness", 0.1, ft),
                                refractive_index=p.scalar("index", 1.5, ft),
                                opacity=p.coef("opacity", (1.0,) * 3, ct))
            if name == "mix":
                idx = []
                for key in ("namedmaterial1", "namedmaterial2"):
                    nm = p.string1(key, "")
                    if nm not in self.gs.named:
                        self.warn(f"named material \"{nm}\" undefined: using matte")
                        idx.append(self._material("matte", p, ("matte-fallback", id(p))))
                    else:
                        idx.append(self.gs.named[nm])
                return Material(MIX, mix=tuple(idx), mix_scale=p.coef("amount", (0.5,) * 3, ct))
            if name == "measured":
                fn = p.string1("filename", "")
                if not fn.lower().endswith("binary"):
                    raise _Unsupported(f"measured material file {fn!r} (MERL .binary only)")
                with open(os.path.join(self.base_dir, fn), "rb") as f:
                    return Material(MEASURED, measured=MeasuredBRDF(f.read(), self.ctx, self.device))
            raise _Unsupported(f"material \"{name}\"")
        except _Unsupported as e:
            self.warn(f"{e} is not supported: matte used instead")
            return Material(MATTE)

    def _current_material(self, shape_params: _Params) -> int:
        kind, val = self.gs.material
        if kind == "@named":
            if val not in self.gs.named:
                self.warn(f"named material \"{val}\" undefined: using matte")
                return self._material("matte", _Params([]), ("matte-default",))
            return self.gs.named[val]
        p = val if val is not None else _Params([])
        if shape_params.items:
            p = shape_params.merged(p)
        return self._material(kind, p, (kind, repr(sorted(p.items.items())), id(self.gs.color_textures)))

    # ---- shapes (ShapeFactory.h)
    def _shape(self, name: str, p: _Params):
        m = self.ctm
        normals = tangents = uvs = None
        if name == "trianglemesh":
            P, idx = p.points("P"), p.ints("indices")
            if P is None or idx is None:
                self.warn("trianglemesh without P or indices skipped")
                return
            idx = np.asarray(idx, np.int64)
            if idx.size % 3 or (idx.size and (idx.min() < 0 or idx.max() >= len(P))):
                self.warn("trianglemesh with out-of-range vertex indices skipped")
                return
            v = apply_point(m, P).astype(np.float32)
            t = idx.reshape(-1, 3).astype(np.int32)
            N = p.points("N", ("normal",))
            if N is not None:
                if len(N) != len(P):
                    self.warn("trianglemesh: the number of N does not match P; normals ignored")
                else:
                    N = N / np.sqrt((N * N).sum(1))[:, None]
                    normals = apply_normal(m, N).astype(np.float32)
            # per-triangle uvs: the "uv" (or "st") of the vertices, else
            # (0, 0), (1, 0), (1, 1) as the factory sets them (ShapeFactory.h)
            uv = p.floats("uv") or p.floats("st")
            if uv is not None and len(uv) < 2 * len(P):
                self.warn("trianglemesh: not enough uvs; discarded")
                uv = None
            if uv is not None:
                uvv = np.asarray(uv[: 2 * len(P)], np.float32).reshape(-1, 2)
                uvs = uvv[t].reshape(-1, 6)
            else:
                uvs = np.tile(np.array([0, 0, 1, 0, 1, 1], np.float32), (len(t), 1))
            flip = self.gs.reverse
        elif name == "sphere":
            radius = p.float1("radius", 1.0)
            for key, d in (("zmin", -radius), ("zmax", radius), ("phimax", 360.0)):
                if p.float1(key, d) != d:
                    self.warn(f"sphere parameter {key} is not supported")
            sm = m @ scale((radius, radius, radius))
            sv, st = scenes.sphere_mesh(5)
            v = apply_point(sm, sv).astype(np.float32)
            t = st.astype(np.int32)
            sign = -1.0 if inverts_orientation(sm) else 1.0
            normals = (sign * apply_normal(sm, sv)).astype(np.float32)
            # tangents (0, 0, 1) x v, or (1, 0, 0) at the poles, through the transform
            tv = np.cross(np.array([0.0, 0.0, 1.0]), sv)
            ln = np.sqrt((tv * tv).sum(1))
            tv = np.where(ln[:, None] > 0, tv / np.where(ln > 0, ln, 1.0)[:, None], [1.0, 0.0, 0.0])
            tangents = apply_vector(sm, tv).astype(np.float32)
            flip = self.gs.reverse != inverts_orientation(sm)
        elif name == "disk":
            height, radius = p.float1("height", 0.0), p.float1("radius", 1.0)
            inner = p.float1("innerradius", 0.0)
            dm = m @ translate((0.0, 0.0, height)) @ scale((radius, radius, 1.0))
            v, t, tangents = disk_mesh(dm, _max_phi(p.float1("phimax", 360.0)), inner / radius)
            flip = self.gs.reverse != inverts_orientation(dm)
        elif name == "cylinder":
            radius, zmin, zmax = p.float1("radius", 1.0), p.float1("zmin", -1.0), p.float1("zmax", 1.0)
            cm = m @ translate((0.0, 0.0, zmin)) @ scale((radius, radius, zmax - zmin))
            v, t, normals, tangents = cylinder_mesh(cm, _max_phi(p.float1("phimax", 360.0)))
            flip = self.gs.reverse != inverts_orientation(cm)
        else:
            self.warn(f"shape \"{name}\" is not supported")
            return
        if flip:
            t = t[:, [0, 2, 1]].copy()
            if uvs is not None:
                uvs = uvs[:, [0, 1, 4, 5, 2, 3]].copy()
        mat = self._current_material(p)
        emission = (0.0, 0.0, 0.0)
        if self.gs.area_light is not None:
            lname, lp = self.gs.area_light
            if lname in ("area", "diffuse"):
                L = lp.emission("L", (1.0, 1.0, 1.0))
                sc = lp.coef("scale", (1.0, 1.0, 1.0), {})
                emission = tuple(float(a * b) for a, b in zip(L, sc))
            else:
                self.warn(f"area light \"{lname}\" is not supported")
        prim = RenderPrimitive(TriangleMesh(v, t), mat, None, normals, None, emission, tangents,
                               uvs if tangents is None else None)
        if self.current_instance is not None:
            if any(emission):
                self.warn("area lights in object instances are not supported")
            self.current_instance.append(prim)
        else:
            self.out.prims.append(prim)

    # ---- lights (LightSourceFactory.h)
    def _light(self, name: str, p: _Params):
        if name == "point":
            I = p.emission("I", (1.0, 1.0, 1.0))
            sc = p.coef("scale", (1.0, 1.0, 1.0), {})
            pos = apply_point(self.ctm, np.asarray([p.point1("from", (0, 0, 0))], np.float64))[0]
            self.out.point_lights.append(PointLight(tuple(float(x) for x in pos),
                                                    tuple(float(a * b) for a, b in zip(I, sc))))
        else:
            self.warn(f"light \"{name}\" is not supported")

    def _volume(self, name: str, p: _Params):
        if name != "homogeneous":
            self.warn(f"volume \"{name}\" is not supported")
            return
        if self.out.medium is not None:
            self.warn("more than one volume: only the first is used")
            return
        ends = apply_point(self.ctm, np.asarray([p.point1("p0", (0, 0, 0)), p.point1("p1", (1, 1, 1))], np.float64))
        lo, hi = np.minimum(ends[0], ends[1]), np.maximum(ends[0], ends[1])
        med = Medium(lo=tuple(float(x) for x in lo), hi=tuple(float(x) for x in hi),
                     sigma_a=p.coef("sigma_a", (0.0,) * 3, {}), sigma_s=p.coef("sigma_s", (0.0,) * 3, {}),
                     emission=p.emission("Le", (0.0, 0.0, 0.0)), g=p.float1("g", 0.0))
        if self.medium_step is not None:
            med.step = self.medium_step
        self.out.medium = med

    def _make_camera(self):
        name, p, cam_to_world = self.camera
        if name != "perspective":
            self.warn(f"camera \"{name}\" is not supported")
            return
        xres, yres = self.film.int1("xresolution", 640), self.film.int1("yresolution", 480)
        if self.film.floats("cropwindow"):
            self.warn("film cropwindow is not supported: the whole image is rendered")
        fov = p.float1("fov", 90.0)
        half = p.float1("halffov", -1.0)
        if half > 0.0:
            fov = float(np.float32(2.0 * half))
        frame = p.float1("frameaspectratio", float(np.float32(xres / float(np.float32(yres)))))
        x_view = math.atan(math.tan(fov * (math.pi / 180.0) / 2.0) * max(1.0, frame)) * 2.0
        if p.float1("lensradius", 0.0) != 0.0:
            self.warn("camera lensradius (depth of field) is not supported")
        self.out.camera = Camera(cam_to_world, x_view, xres, yres)

    # ---- the directives (PbrtSceneImporter_hooks.cpp)
    def run(self, text: str, base_dir: str):
        self.base_dir = base_dir
        for name, args in _commands(text):
            try:
                self._do(name, args)
            except (IndexError, ValueError) as e:
                if isinstance(e, PbrtError):
                    raise
                raise PbrtError(f"{name}: {e}") from e

    def _nums(self, args, n):
        vals = [v for a in args for v in _values(a)]
        if len(vals) < n:
            raise PbrtError(f"expected {n} numbers, found {len(vals)}")
        return [float(np.float32(float(x[1]))) for x in vals[:n]]

    def _str(self, args, i=0):
        if i >= len(args) or args[i][0] != "s":
            raise PbrtError("expected a string")
        return args[i][1]

    def _do(self, name, args):
        if name == "Include":
            fn = os.path.join(self.base_dir, self._str(args))
            with open(fn) as f:
                sub = f.read()
            saved = self.base_dir
            self.run(sub, os.path.dirname(fn))
            self.base_dir = saved
        elif name == "Identity":
            self.ctm = np.eye(4)
        elif name == "Translate":
            self.ctm = self.ctm @ translate(self._nums(args, 3))
        elif name == "Scale":
            self.ctm = self.ctm @ scale(self._nums(args, 3))
        elif name == "Rotate":
            a, x, y, z = self._nums(args, 4)
            self.ctm = self.ctm @ rotate(a, (x, y, z))
        elif name == "LookAt":
            v = self._nums(args, 9)
            self.ctm = self.ctm @ look_at(v[0:3], v[3:6], v[6:9])
        elif name in ("Transform", "ConcatTransform"):
            v = self._nums(args, 16)
            t = np.array(v, np.float64).reshape(4, 4).T  # PBRT lists the matrix column by column
            self.ctm = t if name == "Transform" else self.ctm @ t
        elif name == "CoordinateSystem":
            self.named_cs[self._str(args)] = self.ctm.copy()
        elif name == "CoordSysTransform":
            nm = self._str(args)
            if nm in self.named_cs:
                self.ctm = self.named_cs[nm].copy()
            else:
                self.warn(f"named coordinate system \"{nm}\" undefined")
        elif name in ("ActiveTransform", "TransformTimes"):
            self.warn(f"{name} (motion blur) is not supported")
        elif name == "Camera":
            ctm = self.ctm
            if inverts_orientation(ctm):
                ctm = scale((-1.0, 1.0, 1.0)) @ ctm
            c2w = np.linalg.inv(ctm)
            self.camera = (self._str(args), _Params(args[1:]), c2w)
            self.named_cs["camera"] = c2w
        elif name == "Film":
            if self._str(args) != "image":
                self.warn(f"film \"{self._str(args)}\" is not supported")
            self.film = _Params(args[1:])
        elif name == "VolumeIntegrator":
            p = _Params(args[1:])
            step = p.floats("stepsize")
            if step:
                self.medium_step = step[0]
                if self.out.medium is not None:
                    self.out.medium.step = step[0]
        elif name in ("PixelFilter", "Sampler", "SurfaceIntegrator", "Renderer", "Accelerator"):
            pass  # the renderer's own sampler, integrator and accelerator are chosen by its caller
        elif name == "WorldBegin":
            self.world = True
            self.ctm = np.eye(4)
            self.named_cs["world"] = self.ctm.copy()
        elif name == "WorldEnd":
            self.world = False
            self._make_camera()
        elif name == "AttributeBegin":
            self.stack.append((self.gs.copy(), self.ctm.copy()))
        elif name == "AttributeEnd":
            if not self.stack:
                self.warn("unmatched AttributeEnd ignored")
            else:
                self.gs, self.ctm = self.stack.pop()
        elif name == "TransformBegin":
            self.tstack.append(self.ctm.copy())
        elif name == "TransformEnd":
            if not self.tstack:
                self.warn("unmatched TransformEnd ignored")
            else:
                self.ctm = self.tstack.pop()
        elif name == "ReverseOrientation":
            self.gs.reverse = not self.gs.reverse
        elif name == "Texture":
            tname, ttype, tclass = self._str(args, 0), self._str(args, 1), self._str(args, 2)
            p = _Params(args[3:])
            if tclass != "constant":
                self.warn(f"texture \"{tclass}\" is not supported (constant textures only)")
                return
            try:
                if ttype == "float":
                    self.gs.float_textures[tname] = (p.scalar("value", 1.0, self.gs.float_textures),)
                elif ttype in ("color", "spectrum"):
                    self.gs.color_textures[tname] = p.coef("value", (1.0,) * 3, self.gs.color_textures)
                else:
                    self.warn(f"texture type \"{ttype}\" unknown")
            except _Unsupported as e:
                self.warn(f"texture \"{tname}\": {e} is not supported")
        elif name == "Material":
            self.gs.material = (self._str(args), _Params(args[1:]))
        elif name == "MakeNamedMaterial":
            p = _Params(args[1:])
            kind = p.string1("type", "")
            if not kind:
                self.warn("MakeNamedMaterial without a \"string type\"")
                return
            nm = self._str(args)
            self.gs.named[nm] = self._material(kind, p, ("named", nm, repr(sorted(p.items.items()))))
        elif name == "NamedMaterial":
            self.gs.material = ("@named", self._str(args))
        elif name == "LightSource":
            self._light(self._str(args), _Params(args[1:]))
        elif name == "AreaLightSource":
            self.gs.area_light = (self._str(args), _Params(args[1:]))
        elif name == "Shape":
            self._shape(self._str(args), _Params(args[1:]))
        elif name == "Volume":
            self._volume(self._str(args), _Params(args[1:]))
        elif name == "ObjectBegin":
            self.stack.append((self.gs.copy(), self.ctm.copy()))
            if self.current_instance is not None:
                self.warn("ObjectBegin inside an object definition")
                return
            self.current_instance = self.instances.setdefault(self._str(args), [])
        elif name == "ObjectEnd":
            self.current_instance = None
            if self.stack:
                self.gs, self.ctm = self.stack.pop()
        elif name == "ObjectInstance":
            nm = self._str(args)
            if nm not in self.instances:
                self.warn(f"object \"{nm}\" undefined")
                return
            for prim in self.instances[nm]:
                # the shared mesh (built in its definition's space) with this instance's transform
                self.out.prims.append(RenderPrimitive(prim.mesh, prim.material, self.ctm.copy(),
                                                      prim.vertex_normals, None, prim.emission,
                                                      prim.vertex_tangents, prim.triangle_uvs))


def loads(text: str, base_dir: str = ".", ctx=None, device: bool = True) -> PbrtScene:
    """Imports a pbrt scene from a string (``Include`` and measured-material
    file names relative to base_dir; measured materials are loaded for the
    GPU of ctx, or for the host only with device=False)."""
    imp = _Importer(ctx, device)
    imp.run(text, base_dir)
    if imp.out.camera is None and imp.world is False:
        imp._make_camera()
    if not imp.out.prims and imp.out.medium is None:
        raise PbrtError("no primitives or volume regions in the scene description")
    if not imp.out.point_lights and not any(any(p.emission) for p in imp.out.prims):
        raise PbrtError("no lights in the scene description")
    return imp.out


def load(path: str, ctx=None, device: bool = True) -> PbrtScene:
    """Imports a pbrt scene file (PbrtSceneImporter(filename).GetScene() / GetCameras())."""
    with open(path) as f:
        text = f.read()
    return loads(text, os.path.dirname(os.path.abspath(path)), ctx, device)
