// Device-side description of a render scene, shared by the host layer
// (skw_render_api.cpp) and the kernels (render.cu).  All pointers are
// device pointers; arrays are in "mesh order": global triangle
// g = prim_tri_offset[prim] + mesh triangle index.
#pragma once

#include <vector_types.h>

#include <cstdint>

#include "merl.h"

namespace skw {

enum BsdfKind : int32_t {
  kLambert = 0,
  kOrenNayar = 1,
  kPlastic = 2,
  kMetal = 3,
  kMeasured = 4,
  kTransparent = 5,
  kSubstrate = 6,
  kUber = 7,
  kMix = 8
};

// Material constants after the reference's clamps (MatteMaterial.cpp:29-50,
// PlasticMaterial.cpp:33-53, MetalMaterial.cpp:58-101).  kTransparent
// (TransparentMaterial.cpp:29-55): kd = specular reflectance, ks = specular
// transmittance (both clamped to [0, 1]), ior = refractive index inside.
struct DevMaterial {
  int32_t kind;
  float kd[3];
  float ks[3];
  float exponent;      // Blinn exponent = 1 / clamp(roughness, 0.001, 1)
  float on_a, on_b;    // Oren-Nayar A, B
  float eta[3], k2[3]; // conductor refractive index and squared absorption
  MerlDev merl;        // kMeasured: the tabulated BRDF
  float ior;           // kTransparent, kUber: refractive index (outside: 1); kPlastic 1.5
  float kr[3];         // kUber: specular reflectance
  float kt[3];         // kUber: specular transmittance (1 - opacity; 0 for an opaque surface)
  float pdiff;         // kSubstrate: probability of sampling the diffuse lobe
  int32_t mix[2];      // kMix: the two materials (indices; mix[1] may be -1)
  float mix_scale[3];  // kMix: the first material's scale (the second's is 1 - scale)
  float ev;            // kSubstrate: < 0 Blinn (exponent); else Ashikhmin-Shirley with exponents (exponent, ev)
};

struct AreaLight {
  float radiance[3];
  float area;          // total area of the light's triangles
  int32_t prim;
  int32_t tri_begin;   // range in light_tri / light_cdf
  int32_t tri_count;
  int32_t pad;
  // IrradianceLightsSamplingStrategy (LightsSamplingStrategies/
  // IrradianceLightsSamplingStrategy.cpp:19-31): the mesh bounds and
  // luminance(power) / (pi * bounds area)
  float lo[3], hi[3];
  float intensity;
  float pad2;
};

struct PointLightDev {
  float position[3];
  float intensity[3];
};

// Homogeneous participating medium (HomogeneousVolumeRegion with an
// HGPhaseFunction, VolumeRegions/HomogeneousVolumeRegion.cpp:20-73,
// PhaseFunctions/HGPhaseFunction.h:53-57) and the march step.
struct MediumDev {
  int32_t on;
  float lo[3], hi[3];
  float sigma_s[3], sigma_t[3], emission[3];
  float g;
  float step;
  int32_t max_steps;  // per camera ray (the media queue holds n * max_steps rays)
};

struct SceneDev {
  // geometry in mesh order
  const float *vpos;          // 3 floats per global vertex (world)
  const float *vnrm;          // 3 floats per global vertex (world shading normal), or null per prim
  const int32_t *tri_vidx;    // 3 global vertex ids per global triangle
  const float *tri_albedo;    // 3 floats per global triangle, NaN in [0] = use the material
  const int32_t *prim_tri_offset;
  const int32_t *prim_material;
  const int32_t *prim_light;      // area light index or -1
  const int32_t *prim_has_normals;
  const int32_t *prim_xform;      // 1 where the primitive has a mesh-to-world matrix
  // The shading tangent's source per primitive (0: CoordinateSystem of the
  // shading normal, 1: vertex tangents, 2: triangle uvs), the vertex
  // tangents (3 floats per global vertex, world; null if no primitive has
  // them) and the triangle uvs (6 floats per global triangle; null if none).
  const int32_t *prim_frame;
  const float *vtan;
  const float *tri_uv;
  // Primitives whose mesh is shared (the accelerator traces them in mesh
  // space through their world-to-mesh matrix): prim_inst[p] = 1, their
  // world-to-mesh matrices (16 doubles per primitive, row-major, the
  // accelerator's) and the mesh-space vertex positions (3 floats per global
  // vertex).  All null when no mesh is shared.
  const int32_t *prim_inst;
  const double *prim_w2m;
  const float *vpos_mesh;
  const DevMaterial *materials;
  const AreaLight *area_lights;
  int32_t n_area_lights;
  const int32_t *light_tri;       // global triangle ids of all light triangles
  const float *light_cdf;         // normalised cumulative area per light range
  // Per light triangle (light_tri order), the accelerator leaf that holds
  // it: 8 words -- the leaf's float box (min xyz, max xyz), its first
  // triangle slot and slot count (int bits) -- for the reference-exact test
  // of medium light samples that end on the light (render.cu,
  // own_light_leaf_occludes); accel_tris: the accelerator's triangle slots.
  const float *light_leaf;
  const float4 *accel_tris;
  const PointLightDev *point_lights;
  int32_t n_point_lights;
  float scene_abs;                // largest absolute vertex coordinate
  float emission_scale;           // multiplies every area light's radiance
  MediumDev medium;
  int32_t has_specular;           // some primitive has a kTransparent material
  int32_t max_spec_depth;         // DirectLightingLTEIntegratorParams::m_max_specular_depth
};

struct CameraDev {
  double c2w[16];
  double x_tan, y_tan;
  int32_t width, height;
  // float copies for the ray generation: the 3x4 camera-to-world rows and
  // 2 tan / size per axis
  float m[12];
  float sx, sy;
};

// One view of a render: its camera, the index of its first pixel in the
// concatenation of all views' films (pixel-major, RGB float), and the seed of
// its random numbers.  A sample's random numbers depend only on (seed, the
// sample's index within its own view), so a view renders the same whether
// it is rendered alone or in a batch.
struct ViewDev {
  CameraDev cam;
  int64_t px_begin;
  uint64_t seed;
};

}  // namespace skw
