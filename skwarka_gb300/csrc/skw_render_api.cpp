// C ABI (include/skw.h): render scenes and the direct-lighting render.
#include "../../include/skw.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <new>
#include <string>
#include <vector>

#include "kernels.h"
#include "photon_map_internal.h"
#include "photon_types.h"
#include "render_scene.h"
#include "skw_internal.h"

using skw::cuda_fail;
using skw::fail;

extern "C" skw::MerlDev skw_merl_device_view(const skw_merl *m);

namespace {

template <class T>
cudaError_t upload(skw_scene *s, const std::vector<T> &v, const T **out) {
  *out = nullptr;
  if (v.empty()) return cudaSuccess;
  void *p = nullptr;
  cudaError_t e = cudaMalloc(&p, v.size() * sizeof(T));
  if (e != cudaSuccess) return e;
  s->buffers.push_back(p);
  e = cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
  *out = (const T *)p;
  return e;
}

inline float clamp01(float v) { return std::min(1.0f, std::max(0.0f, v)); }
// The reference's luminance of an RGB coefficient (SpectrumRoutines::Luminance).
inline float lum(float r, float g, float b) { return 0.05316285f * r + 0.58515348f * g + 0.36168367f * b; }

// Transform::operator()(Point3D<float>) (Math/Transform.h:219-230), like the
// accelerator builder, so shading points agree with the traced triangles.
void xform_point(const double *m, const float *p, float *out) {
  if (!m) {
    out[0] = p[0];
    out[1] = p[1];
    out[2] = p[2];
    return;
  }
  const float x = p[0], y = p[1], z = p[2];
  const float xp = (float)(m[0] * x + m[1] * y + m[2] * z + m[3]);
  const float yp = (float)(m[4] * x + m[5] * y + m[6] * z + m[7]);
  const float zp = (float)(m[8] * x + m[9] * y + m[10] * z + m[11]);
  const float wp = (float)(m[12] * x + m[13] * y + m[14] * z + m[15]);
  if (wp == 1.0f) {
    out[0] = xp;
    out[1] = yp;
    out[2] = zp;
  } else {
    const double inv = 1.0 / (double)wp;
    out[0] = (float)(xp * inv);
    out[1] = (float)(yp * inv);
    out[2] = (float)(zp * inv);
  }
}

// Transform::TransformNormal (Math/Transform.h:283-292): inverse transpose,
// normalised.  inv is the inverse of the 3x3 part.
void xform_normal(const double *inv, const float *n, float *out) {
  double v[3] = {n[0], n[1], n[2]};
  if (inv) {
    v[0] = inv[0] * n[0] + inv[3] * n[1] + inv[6] * n[2];
    v[1] = inv[1] * n[0] + inv[4] * n[1] + inv[7] * n[2];
    v[2] = inv[2] * n[0] + inv[5] * n[1] + inv[8] * n[2];
  }
  const double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  for (int k = 0; k < 3; ++k) out[k] = (float)(l > 0 ? v[k] / l : v[k]);
}

// Transform::operator()(Vector3D) on a mesh tangent, normalised (the
// world-space tangent of a transformed primitive's differential geometry).
void xform_tangent(const double *m, const float *t, float *out) {
  double v[3] = {t[0], t[1], t[2]};
  if (m) {
    v[0] = m[0] * t[0] + m[1] * t[1] + m[2] * t[2];
    v[1] = m[4] * t[0] + m[5] * t[1] + m[6] * t[2];
    v[2] = m[8] * t[0] + m[9] * t[1] + m[10] * t[2];
  }
  const double l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  for (int k = 0; k < 3; ++k) out[k] = (float)(l > 0 ? v[k] / l : v[k]);
}

// Vector3D<float>::Normalized (Math/Vector3D.h:259-276), as TriangleMesh
// stores its shading normals (TriangleMesh.cpp:208-213): the squared length
// and its square root in float, the reciprocal in double, each coordinate
// times it rounded to float.
void ref_normalize_f(const float *n, float *out) {
  const float l2 = n[0] * n[0] + n[1] * n[1] + n[2] * n[2];
  if (!(l2 > 0.0f)) {
    out[0] = n[0];
    out[1] = n[1];
    out[2] = n[2];
    return;
  }
  const double inv = 1.0 / (double)std::sqrt(l2);
  for (int k = 0; k < 3; ++k) out[k] = (float)((double)n[k] * inv);
}

bool inverse3(const double *m4, double *inv) {
  const double a = m4[0], b = m4[1], c = m4[2], d = m4[4], e = m4[5], f = m4[6], g = m4[8], h = m4[9], i = m4[10];
  const double det = a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
  if (det == 0.0) return false;
  const double r = 1.0 / det;
  inv[0] = (e * i - f * h) * r;
  inv[1] = (c * h - b * i) * r;
  inv[2] = (b * f - c * e) * r;
  inv[3] = (f * g - d * i) * r;
  inv[4] = (a * i - c * g) * r;
  inv[5] = (c * d - a * f) * r;
  inv[6] = (d * h - e * g) * r;
  inv[7] = (b * g - a * h) * r;
  inv[8] = (a * e - b * d) * r;
  return true;
}

}  // namespace

extern "C" {

int skw_scene_create(skw_ctx *ctx, const skw_mesh *meshes, int32_t n_meshes, const skw_render_primitive *prims,
                     int32_t n_prims, const skw_material *materials, int32_t n_materials,
                     const skw_point_light *point_lights, int32_t n_point_lights, skw_scene **out) {
  if (!ctx || !out || (n_meshes > 0 && !meshes) || (n_prims > 0 && !prims) || (n_materials > 0 && !materials) ||
      (n_point_lights > 0 && !point_lights) || n_meshes < 0 || n_prims < 0 || n_materials < 0 || n_point_lights < 0)
    return fail(ctx, SKW_ERR_ARG, "null or negative argument");
  *out = nullptr;
  for (int32_t p = 0; p < n_prims; ++p) {
    if (prims[p].mesh < 0 || prims[p].mesh >= n_meshes) return fail(ctx, SKW_ERR_ARG, "primitive mesh out of range");
    if (prims[p].material < 0 || prims[p].material >= n_materials)
      return fail(ctx, SKW_ERR_ARG, "primitive material out of range");
    const bool light = prims[p].emission[0] > 0 || prims[p].emission[1] > 0 || prims[p].emission[2] > 0;
    if (light && prims[p].mesh_to_world)
      return fail(ctx, SKW_ERR_UNSUPPORTED,
                  "an area light samples its mesh in mesh space (DiffuseAreaLightSource); give it an identity transform");
  }
  auto *s = new (std::nothrow) skw_scene();
  if (!s) return fail(ctx, SKW_ERR_OOM, "host allocation failed");
  s->ctx = ctx;
  // Accelerator over the same primitives.
  std::vector<skw_primitive> ap((size_t)n_prims);
  for (int32_t p = 0; p < n_prims; ++p) ap[(size_t)p] = skw_primitive{prims[p].mesh, prims[p].mesh_to_world};
  int rc = skw_accel_create(ctx, meshes, n_meshes, ap.data(), n_prims, &s->accel);
  if (rc != SKW_OK) {
    delete s;
    return rc;
  }
  // Mesh-order geometry.
  std::vector<float> vpos, vnrm, vtan, tri_uv, albedo, vpos_mesh;
  std::vector<double> prim_w2m;
  std::vector<int32_t> prim_inst((size_t)std::max(n_prims, 1), 0);
  {
    std::vector<int> uses((size_t)std::max(n_meshes, 1), 0);
    for (int32_t p = 0; p < n_prims; ++p) ++uses[(size_t)prims[p].mesh];
    bool any = false;
    for (int32_t p = 0; p < n_prims; ++p) any |= (prim_inst[(size_t)p] = uses[(size_t)prims[p].mesh] > 1 ? 1 : 0) != 0;
    if (any) {
      // the accelerator's world-to-mesh matrices (identity for unshared meshes)
      const double id[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};
      prim_w2m.assign(16 * (size_t)n_prims, 0.0);
      for (int32_t p = 0; p < n_prims; ++p) {
        double *o = prim_w2m.data() + 16 * (size_t)p;
        if (!skw::invert4(prims[p].mesh_to_world ? prims[p].mesh_to_world : id, o)) std::memcpy(o, id, sizeof(id));
      }
    }
  }
  const bool instanced = !prim_w2m.empty();
  std::vector<int32_t> tri_vidx, prim_tri_offset((size_t)std::max(n_prims, 1)), prim_material((size_t)std::max(n_prims, 1)),
      prim_light((size_t)std::max(n_prims, 1), -1), prim_has_normals((size_t)std::max(n_prims, 1), 0),
      prim_xform((size_t)std::max(n_prims, 1), 0), prim_frame((size_t)std::max(n_prims, 1), 0);
  // Per-triangle albedo is always present (NaN = the material's kd) so that
  // skw_scene_set_triangle_albedo can replace it.
  bool any_albedo = true, any_normals = false;
  bool any_tangents = false, any_uvs = false;
  for (int32_t p = 0; p < n_prims; ++p) {
    any_normals |= prims[p].vertex_normals != nullptr;
    any_tangents |= prims[p].vertex_tangents != nullptr;
    any_uvs |= prims[p].vertex_tangents == nullptr && prims[p].triangle_uvs != nullptr;
  }
  std::vector<skw::AreaLight> lights;
  std::vector<int32_t> light_tri;
  std::vector<float> light_cdf;
  int32_t tri_count = 0;
  for (int32_t p = 0; p < n_prims; ++p) {
    const skw_mesh &m = meshes[prims[p].mesh];
    const int32_t voff = (int32_t)(vpos.size() / 3);
    prim_tri_offset[(size_t)p] = tri_count;
    prim_material[(size_t)p] = prims[p].material;
    prim_has_normals[(size_t)p] = prims[p].vertex_normals ? 1 : 0;
    prim_xform[(size_t)p] = prims[p].mesh_to_world ? 1 : 0;
    prim_frame[(size_t)p] = prims[p].vertex_tangents ? 1 : (prims[p].triangle_uvs ? 2 : 0);
    double inv[9];
    const bool has_inv = prims[p].mesh_to_world && inverse3(prims[p].mesh_to_world, inv);
    for (int64_t v = 0; v < m.n_vertices; ++v) {
      float w[3];
      xform_point(prims[p].mesh_to_world, m.vertices + 3 * v, w);
      vpos.insert(vpos.end(), w, w + 3);
      if (instanced) vpos_mesh.insert(vpos_mesh.end(), m.vertices + 3 * v, m.vertices + 3 * v + 3);
      if (any_normals) {
        float nn[3] = {0, 0, 1};
        if (prims[p].vertex_normals) {
          ref_normalize_f(prims[p].vertex_normals + 3 * v, nn);  // the mesh's stored normal
          if (has_inv) {
            const float mn[3] = {nn[0], nn[1], nn[2]};
            xform_normal(inv, mn, nn);
          }
        }
        vnrm.insert(vnrm.end(), nn, nn + 3);
      }
      if (any_tangents) {
        float tt[3] = {1, 0, 0};
        if (prims[p].vertex_tangents) {
          ref_normalize_f(prims[p].vertex_tangents + 3 * v, tt);  // the mesh's stored tangent
          const float mt[3] = {tt[0], tt[1], tt[2]};
          xform_tangent(prims[p].mesh_to_world, mt, tt);
        }
        vtan.insert(vtan.end(), tt, tt + 3);
      }
    }
    const bool light = prims[p].emission[0] > 0 || prims[p].emission[1] > 0 || prims[p].emission[2] > 0;
    skw::AreaLight L{};
    if (light) {
      L.radiance[0] = prims[p].emission[0];
      L.radiance[1] = prims[p].emission[1];
      L.radiance[2] = prims[p].emission[2];
      L.prim = p;
      L.tri_begin = (int32_t)light_tri.size();
    }
    double area_sum = 0.0;
    std::vector<double> areas;
    int32_t kept = 0;
    float mesh_area = 0.0f;
    for (int64_t t = 0; t < m.n_triangles; ++t) {
      const int32_t *ix = m.triangles + 3 * t;
      bool bad = false;
      for (int k = 0; k < 3; ++k)
        if (ix[k] < 0 || (int64_t)ix[k] >= m.n_vertices) bad = true;
      if (bad || ix[0] == ix[1] || ix[0] == ix[2] || ix[1] == ix[2]) continue;  // TriangleMesh.cpp:176-182
      for (int k = 0; k < 3; ++k) tri_vidx.push_back(voff + ix[k]);
      if (any_uvs) {
        if (prim_frame[(size_t)p] == 2) {
          tri_uv.insert(tri_uv.end(), prims[p].triangle_uvs + 6 * t, prims[p].triangle_uvs + 6 * t + 6);
        } else {
          tri_uv.insert(tri_uv.end(), {0, 0, 0, 0, 0, 0});
        }
      }
      if (any_albedo) {
        const float nanv = std::nanf("");
        if (prims[p].triangle_albedo) {
          for (int k = 0; k < 3; ++k) albedo.push_back(prims[p].triangle_albedo[3 * t + k]);
        } else {
          albedo.insert(albedo.end(), {nanv, nanv, nanv});
        }
      }
      if (light) {
        // Triangle3D<float>::GetArea on the mesh's vertices (DiffuseAreaLightSource.cpp:26-54)
        const float *a = m.vertices + 3 * ix[0], *b = m.vertices + 3 * ix[1], *c = m.vertices + 3 * ix[2];
        const double e1[3] = {(double)b[0] - a[0], (double)b[1] - a[1], (double)b[2] - a[2]};
        const double e2[3] = {(double)c[0] - a[0], (double)c[1] - a[1], (double)c[2] - a[2]};
        const double cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        const double ar = 0.5 * std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
        area_sum += ar;
        areas.push_back(area_sum);
        light_tri.push_back(tri_count + kept);
      }
      ++kept;
      // TriangleMesh's area: Triangle3D<float>::GetArea summed in float
      // (Core/TriangleMesh.cpp:193-205, Math/Triangle3D.h:82-86)
      {
        const float *a = m.vertices + 3 * ix[0], *b = m.vertices + 3 * ix[1], *c = m.vertices + 3 * ix[2];
        const float e1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]}, e2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
        const float cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        mesh_area += 0.5f * std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
      }
    }
    s->total_area += (double)mesh_area;
    if (light) {
      L.tri_count = (int32_t)areas.size();
      L.area = (float)area_sum;
      // mesh bounds (TriangleMesh::GetBounds: over the triangles' vertices)
      float blo[3] = {INFINITY, INFINITY, INFINITY}, bhi[3] = {-INFINITY, -INFINITY, -INFINITY};
      for (int64_t t = 0; t < m.n_triangles; ++t)
        for (int k = 0; k < 3; ++k) {
          const int32_t vi = m.triangles[3 * t + k];
          if (vi < 0 || (int64_t)vi >= m.n_vertices) continue;
          for (int c = 0; c < 3; ++c) {
            blo[c] = std::min(blo[c], m.vertices[3 * vi + c]);
            bhi[c] = std::max(bhi[c], m.vertices[3 * vi + c]);
          }
        }
      const double bx = std::fabs((double)bhi[0] - blo[0]), by = std::fabs((double)bhi[1] - blo[1]),
                   bz = std::fabs((double)bhi[2] - blo[2]);
      const double barea = 2.0 * (bx * by + bx * bz + by * bz);
      const double lum = 0.05316285 * L.radiance[0] + 0.58515348 * L.radiance[1] + 0.36168367 * L.radiance[2];
      for (int c = 0; c < 3; ++c) {
        L.lo[c] = blo[c];
        L.hi[c] = bhi[c];
      }
      // luminance(Power()) / (pi * area) with Power() = pi * A * L
      L.intensity = barea > 0.0 ? (float)(area_sum * lum / barea) : 0.0f;
      for (double a : areas) light_cdf.push_back(area_sum > 0 ? (float)(a / area_sum) : 1.0f);
      if (L.tri_count > 0 && area_sum > 0) {
        prim_light[(size_t)p] = (int32_t)lights.size();
        lights.push_back(L);
      }
    }
    tri_count += kept;
  }
  // Materials after the reference's clamps.
  std::vector<skw::DevMaterial> mats((size_t)n_materials);
  for (int32_t i = 0; i < n_materials; ++i) {
    const skw_material &m = materials[i];
    skw::DevMaterial &d = mats[(size_t)i];
    std::memset(&d, 0, sizeof(d));
    for (int k = 0; k < 3; ++k) {
      d.kd[k] = clamp01(m.kd[k]);
      d.ks[k] = clamp01(m.ks[k]);
      d.eta[k] = m.eta[k];
      d.k2[k] = m.k[k] * m.k[k];
    }
    const float rough = std::min(1.0f, std::max(0.001f, m.roughness));
    d.exponent = std::min(1000.0f, std::max(0.0f, 1.0f / rough));  // BlinnDistribution clamps to [0, 1000]
    d.ev = -1.0f;
    if (m.kind == SKW_MATERIAL_MATTE) {
      const float sig = clamp01(m.sigma);
      if (sig < 2.220446e-16f) {
        d.kind = skw::kLambert;
      } else {
        d.kind = skw::kOrenNayar;  // OrenNayar.cpp:19-27
        const double s2 = (double)sig * sig;
        d.on_a = (float)(1.0 - (0.5 * s2 / (s2 + 0.33)));
        d.on_b = (float)(0.45 * s2 / (s2 + 0.09));
      }
    } else if (m.kind == SKW_MATERIAL_PLASTIC) {
      d.kind = skw::kPlastic;
      d.ior = 1.5f;  // PlasticMaterial.cpp:43: FresnelDielectric(1.5, 1)
    } else if (m.kind == SKW_MATERIAL_SUBSTRATE) {
      d.kind = skw::kSubstrate;
      if (m.v_roughness > 0.0f) {
        // AnisotropicDistribution(1 / clamp(u), 1 / clamp(v)), each exponent
        // clamped to [0, 1000] (AnisotropicDistribution.h: constructor)
        const float rv = std::min(1.0f, std::max(0.001f, m.v_roughness));
        d.ev = std::min(1000.0f, std::max(0.0f, 1.0f / rv));
      }
      // The lobe-sampling probability only shapes the variance (the
      // estimator divides by the mixture density it samples): the share of
      // the diffuse term's luminance in the two terms' luminances, kept in
      // [0.1, 0.9] so that neither lobe goes unsampled.
      const float ld = lum(d.kd[0] * (1 - d.ks[0]), d.kd[1] * (1 - d.ks[1]), d.kd[2] * (1 - d.ks[2]));
      const float ls = lum(d.ks[0], d.ks[1], d.ks[2]);
      d.pdiff = ld + ls > 0.0f ? std::min(0.9f, std::max(0.1f, ld / (ld + ls))) : 0.5f;
    } else if (m.kind == SKW_MATERIAL_UBER) {
      if (!(m.refractive_index > 0.0f)) {
        skw_scene_destroy(s);
        return fail(ctx, SKW_ERR_ARG, "an uber material needs a positive refractive index");
      }
      d.kind = skw::kUber;
      d.ior = m.refractive_index;
      bool opaque = true;
      for (int k = 0; k < 3; ++k) {
        const float op = clamp01(m.opacity[k]);
        opaque = opaque && op >= 1.0f - 1e-2f && op <= 1.0f + 1e-2f;
        d.kd[k] = clamp01(op * m.kd[k]);
        d.ks[k] = clamp01(op * m.ks[k]);
        d.kr[k] = clamp01(m.kr[k]);
      }
      for (int k = 0; k < 3; ++k) d.kt[k] = opaque ? 0.0f : 1.0f - clamp01(m.opacity[k]);
      // BlinnDistribution(1 / roughness), clamped to [0, 1000] by the distribution
      const float inv = m.roughness > 0.0f ? 1.0f / m.roughness : 1000.0f;
      d.exponent = std::min(1000.0f, std::max(0.0f, inv));
    } else if (m.kind == SKW_MATERIAL_MIX) {
      d.kind = skw::kMix;
      for (int k = 0; k < 2; ++k) {
        const int32_t j = m.mix[k];
        if (j < -1 || j >= n_materials || (k == 0 && j < 0)) {
          skw_scene_destroy(s);
          return fail(ctx, SKW_ERR_ARG, "a mix material's materials must be indices into the material array");
        }
        if (j >= 0 && materials[j].kind == SKW_MATERIAL_MIX) {
          skw_scene_destroy(s);
          return fail(ctx, SKW_ERR_UNSUPPORTED, "a mix of mix materials");
        }
        d.mix[k] = j;
      }
      for (int k = 0; k < 3; ++k) d.mix_scale[k] = clamp01(m.mix_scale[k]);
    } else if (m.kind == SKW_MATERIAL_METAL) {
      d.kind = skw::kMetal;
    } else if (m.kind == SKW_MATERIAL_MEASURED) {
      if (!m.measured) {
        skw_scene_destroy(s);
        return fail(ctx, SKW_ERR_ARG, "a measured material needs its skw_merl");
      }
      d.kind = skw::kMeasured;
      d.merl = skw_merl_device_view(m.measured);
    } else if (m.kind == SKW_MATERIAL_TRANSPARENT) {
      if (!(m.refractive_index > 0.0f)) {  // TransparentMaterial.cpp:22-27 asserts a positive index
        skw_scene_destroy(s);
        return fail(ctx, SKW_ERR_ARG, "a transparent material needs a positive refractive index");
      }
      d.kind = skw::kTransparent;  // kd: reflectance, ks: transmittance (clamped above)
      d.ior = m.refractive_index;
    } else {
      skw_scene_destroy(s);
      return fail(ctx, SKW_ERR_UNSUPPORTED, "unknown material kind");
    }
  }
  std::vector<skw::PointLightDev> pls((size_t)n_point_lights);
  for (int32_t i = 0; i < n_point_lights; ++i)
    for (int k = 0; k < 3; ++k) {
      pls[(size_t)i].position[k] = point_lights[i].position[k];
      pls[(size_t)i].intensity[k] = point_lights[i].intensity[k];
    }
  // The accelerator leaf of every light triangle (its box and slot range).
  std::vector<float> light_leaf(8 * std::max<size_t>(light_tri.size(), 1), 0.0f);
  {
    const std::vector<skw::DevNode> &nodes = s->accel->h_nodes;
    const std::vector<skw::DevTri> &slots = s->accel->h_tris;
    std::vector<int32_t> leaf_of_slot(slots.size(), -1), slot_of_tri((size_t)std::max(tri_count, 1), -1);
    // a leaf's triangle-slot range (leaves holding instances keep it in the ext table)
    auto leaf_range = [&](const skw::DevNode &nd, uint32_t &first, uint32_t &count) {
      if (nd.b & skw::kLeafExt) {
        first = s->accel->h_leaf_ext[nd.a].tri_first;
        count = s->accel->h_leaf_ext[nd.a].tri_count;
      } else {
        first = nd.a;
        count = nd.b >> 8;
      }
    };
    for (size_t n = 0; n < nodes.size(); ++n)
      if ((nodes[n].b & 3u) == 0u) {
        uint32_t first, count;
        leaf_range(nodes[n], first, count);
        for (uint32_t k = 0; k < count; ++k) leaf_of_slot[first + k] = (int32_t)n;
      }
    for (size_t k = 0; k < slots.size(); ++k)  // (a shared mesh's slots, prim -1, belong to no one primitive)
      if (slots[k].prim >= 0)
        slot_of_tri[(size_t)(prim_tri_offset[(size_t)slots[k].prim] + slots[k].tri)] = (int32_t)k;
    for (size_t j = 0; j < light_tri.size(); ++j) {
      const int32_t slot = slot_of_tri[(size_t)light_tri[j]];
      const int32_t leaf = slot >= 0 ? leaf_of_slot[(size_t)slot] : -1;
      float *o = light_leaf.data() + 8 * j;
      if (leaf < 0) {  // an instanced light mesh: an empty range tests nothing
        o[0] = o[1] = o[2] = INFINITY;
        o[3] = o[4] = o[5] = -INFINITY;
        continue;
      }
      const skw::DevNode &L = nodes[(size_t)leaf];
      for (int c = 0; c < 3; ++c) {
        o[c] = L.lo[c];
        o[3 + c] = L.hi[c];
      }
      uint32_t ufirst, ucount;
      leaf_range(L, ufirst, ucount);
      const int32_t first = (int32_t)ufirst, count = (int32_t)ucount;
      std::memcpy(o + 6, &first, 4);
      std::memcpy(o + 7, &count, 4);
    }
  }
  cudaError_t e = cudaSetDevice(ctx->device);
  skw::SceneDev &D = s->dev;
  D.accel_tris = (const float4 *)s->accel->d_tris;
  if (e == cudaSuccess) e = upload(s, light_leaf, &D.light_leaf);
  if (e == cudaSuccess) e = upload(s, vpos, &D.vpos);
  if (e == cudaSuccess) e = upload(s, vnrm, &D.vnrm);
  if (e == cudaSuccess) e = upload(s, tri_vidx, &D.tri_vidx);
  if (e == cudaSuccess) e = upload(s, albedo, &D.tri_albedo);
  if (e == cudaSuccess) e = upload(s, prim_tri_offset, &D.prim_tri_offset);
  if (e == cudaSuccess) e = upload(s, prim_material, &D.prim_material);
  if (e == cudaSuccess) e = upload(s, prim_light, &D.prim_light);
  if (e == cudaSuccess) e = upload(s, prim_has_normals, &D.prim_has_normals);
  if (e == cudaSuccess) e = upload(s, prim_xform, &D.prim_xform);
  if (e == cudaSuccess) e = upload(s, prim_frame, &D.prim_frame);
  if (e == cudaSuccess) e = upload(s, vtan, &D.vtan);
  if (e == cudaSuccess) e = upload(s, tri_uv, &D.tri_uv);
  if (instanced) {
    if (e == cudaSuccess) e = upload(s, prim_inst, &D.prim_inst);
    if (e == cudaSuccess) e = upload(s, prim_w2m, &D.prim_w2m);
    if (e == cudaSuccess) e = upload(s, vpos_mesh, &D.vpos_mesh);
  }
  if (e == cudaSuccess) e = upload(s, mats, &D.materials);
  if (e == cudaSuccess) e = upload(s, lights, &D.area_lights);
  if (e == cudaSuccess) e = upload(s, light_tri, &D.light_tri);
  if (e == cudaSuccess) e = upload(s, light_cdf, &D.light_cdf);
  if (e == cudaSuccess) e = upload(s, pls, &D.point_lights);
  if (e != cudaSuccess) {
    skw_scene_destroy(s);
    return cuda_fail(ctx, e, "render scene upload");
  }
  D.n_area_lights = (int32_t)lights.size();
  D.n_point_lights = n_point_lights;
  D.emission_scale = 1.0f;
  // Specular components of a material: a transparent one's, an uber one's
  // reflection (kr) and transmission (kt); a mix's from its two materials,
  // of which at most one may have any (one specular reflection and one
  // transmission per BSDF, as the specular stages follow them).
  auto has_spec = [&](const skw::DevMaterial &d) {
    auto nb = [](const float *v) { return v[0] != 0.0f || v[1] != 0.0f || v[2] != 0.0f; };
    return d.kind == skw::kTransparent || (d.kind == skw::kUber && (nb(d.kr) || nb(d.kt)));
  };
  for (int32_t i = 0; i < n_materials; ++i) {
    const skw::DevMaterial &d = mats[(size_t)i];
    if (d.kind == skw::kMix && d.mix[1] >= 0 && has_spec(mats[(size_t)d.mix[0]]) &&
        has_spec(mats[(size_t)d.mix[1]])) {
      skw_scene_destroy(s);
      return fail(ctx, SKW_ERR_UNSUPPORTED, "a mix of two materials that both have specular components");
    }
  }
  D.has_specular = 0;
  for (int32_t p = 0; p < n_prims; ++p) {
    const skw::DevMaterial &d = mats[(size_t)prims[p].material];
    if (has_spec(d) || (d.kind == skw::kMix && (has_spec(mats[(size_t)d.mix[0]]) ||
                                                (d.mix[1] >= 0 && has_spec(mats[(size_t)d.mix[1]])))))
      D.has_specular = 1;
  }
  D.max_spec_depth = 10;  // the GUI's DirectLightParams / PhotonMapParams default
  s->n_triangles = tri_count;
  D.scene_abs = s->accel->scene_abs;
  *out = s;
  return SKW_OK;
}

void skw_scene_destroy(skw_scene *s) {
  if (!s) return;
  for (void *p : s->buffers) cudaFree(p);
  skw_accel_destroy(s->accel);
  delete s;
}

skw_accel *skw_scene_accel(skw_scene *s) { return s ? s->accel : nullptr; }

double skw_scene_total_area(const skw_scene *s) { return s ? s->total_area : -1.0; }


}  // extern "C"

// ---------------------------------------------------------------------------
// Render passes.  Both the single-camera render and the batch lay the views'
// pixels end to end and process them in passes of whole pixels; a pass runs
// camera -> closest hit -> shade (queues shadow and BSDF rays) -> any hit on
// the shadow queue -> closest hit on the BSDF queue -> resolve -> film.
namespace {

struct PassConfig {
  int64_t samples_per_pass = (int64_t)1 << 21;
  int stack_cap = 0;         // 0: the accelerator's own
  int trace_ctas_per_sm = 0;
  int shade_block = 128;
  int overlap = 0;
  int extra_slots = 0;       // contribution slots after the direct-lighting ones (final gather)
  bool media = true;         // march the scene's medium (if any) along the camera rays (one more slot, last)
  bool specular = true;      // follow specular reflection / transmission (if the scene has such materials)
};

// Entries of the largest specular level of a pass (the pass is sized so
// that every branch of every sample's specular tree fits).  2^25 entries
// (about 10 GB of level, shadow and BSDF queues, kept by the context's
// pool) hold a 256 x 256 x 4 frame at depth 6 in one pass: measured on the
// glass-sphere frame, 2^23: 4 passes, 200 launches, 5.74 ms; 2^24: 3.88 ms;
// 2^25: 1 pass, 50 launches, 2.33 ms.
#ifndef SKW_SPEC_ENTRIES_LOG2
#define SKW_SPEC_ENTRIES_LOG2 25
#endif
constexpr int64_t kSpecEntries = (int64_t)1 << SKW_SPEC_ENTRIES_LOG2;
// Deepest specular depth: a sample's tree then holds up to 2^12 - 1 rays.
constexpr int kMaxSpecDepth = 11;

struct Plan {
  std::vector<skw::ViewDev> views;
  std::vector<int64_t> film_offset;  // floats
  int sppx = 1, sppy = 1, spp = 1, nl = 0, npl = 0, slots = 1;
  int ld = 0;  // LDSampler (sppx = spp, a power of two; sppy = 1)
  int64_t n_px_total = 0, chunk_px = 0, cap_samples = 0, cap_shadow = 0, cap_bsdf = 0;
  bool media = false;
  int media_slot = 0;
  int64_t cap_media = 0;  // media light-sample queue: cap_samples * max_steps
  int spec_levels = 0;    // specular depths traced after the camera rays (0: none)
  int spec_slot = 0;
  int64_t cap_spec = 0;   // entries of a specular level buffer: cap_samples << spec_levels
  PassConfig cfg;
};

// Device buffers of one workspace (one pass in flight).
struct Workspace {
  void *rays = nullptr, *hits = nullptr, *srays = nullptr, *brays = nullptr, *bhits = nullptr;
  float *contrib = nullptr, *srgb = nullptr, *brgb = nullptr, *bnrm = nullptr;
  int *starget = nullptr, *btarget = nullptr, *counts = nullptr;
  uint8_t *occ = nullptr;
  // medium
  float *tcam = nullptr, *mval = nullptr, *mdem = nullptr;
  void *mrays = nullptr;
  int *mtarget = nullptr;
  uint8_t *mocc = nullptr;
  // specular levels: two ping-pong queues and the hits of the level traced
  void *qrays[2] = {nullptr, nullptr}, *qhits = nullptr;
  float *qw[2] = {nullptr, nullptr};
  int *qsample[2] = {nullptr, nullptr}, *qnode[2] = {nullptr, nullptr};
};

inline size_t al256(int64_t x) { return (size_t)((x + 255) & ~(int64_t)255); }

size_t workspace_bytes(const Plan &P) {
  const int64_t cs = P.cap_samples, sh = std::max<int64_t>(P.cap_shadow, 1), bs = std::max<int64_t>(P.cap_bsdf, 1);
  const int64_t cm = std::max<int64_t>(P.cap_media, 1);
  const size_t media = P.media ? al256(cs * 12) + al256(cm * 32) + al256(cm * 4) + 2 * al256(cm * 12) + al256(cm) : 0;
  const int64_t cq = P.cap_spec;
  const size_t spec = P.spec_levels ? 2 * (al256(cq * 32) + al256(cq * 12) + 2 * al256(cq * 4)) + al256(cq * 16) : 0;
  return al256(cs * 32) + al256(cs * 16) + al256(cs * P.slots * 12) + al256(sh * 32) + al256(sh * 4) +
         al256(sh * 12) + al256(sh) + al256(bs * 32) + al256(bs * 4) + al256(bs * 16) + al256(bs * 16) + 256 + media +
         al256(bs * 12) + spec;
}

void workspace_carve(const Plan &P, char *base, Workspace *W) {
  const int64_t cs = P.cap_samples, sh = std::max<int64_t>(P.cap_shadow, 1), bs = std::max<int64_t>(P.cap_bsdf, 1);
  char *p = base;
  auto take = [&](size_t b) {
    char *r = p;
    p += b;
    return r;
  };
  W->rays = take(al256(cs * 32));
  W->hits = take(al256(cs * 16));
  W->contrib = (float *)take(al256(cs * P.slots * 12));
  W->srays = take(al256(sh * 32));
  W->starget = (int *)take(al256(sh * 4));
  W->srgb = (float *)take(al256(sh * 12));
  W->occ = (uint8_t *)take(al256(sh));
  W->brays = take(al256(bs * 32));
  W->btarget = (int *)take(al256(bs * 4));
  W->brgb = (float *)take(al256(bs * 16));
  W->bhits = take(al256(bs * 16));
  W->counts = (int *)take(256);  // [0] shadow, [1] BSDF, [2] media queue length, [3], [4] specular levels
  W->bnrm = (float *)take(al256(bs * 12));
  if (P.media) {
    const int64_t cm = std::max<int64_t>(P.cap_media, 1);
    W->tcam = (float *)take(al256(cs * 12));
    W->mrays = take(al256(cm * 32));
    W->mtarget = (int *)take(al256(cm * 4));
    W->mval = (float *)take(al256(cm * 12));
    W->mdem = (float *)take(al256(cm * 12));
    W->mocc = (uint8_t *)take(al256(cm));
  }
  if (P.spec_levels) {
    const int64_t cq = P.cap_spec;
    for (int k = 0; k < 2; ++k) {
      W->qrays[k] = take(al256(cq * 32));
      W->qw[k] = (float *)take(al256(cq * 12));
      W->qsample[k] = (int *)take(al256(cq * 4));
      W->qnode[k] = (int *)take(al256(cq * 4));
    }
    W->qhits = take(al256(cq * 16));
  }
}

int valid_cap(int c) { return c == 48 || c == 96 || c == 192 || c == 416; }

// Validates the cameras and parameters and lays out the passes.
int plan_make(skw_scene *s, const skw_camera *cams, int n_views, const skw_render_params *params,
              const uint64_t *seeds, const PassConfig &cfg, Plan *P) {
  skw_ctx *ctx = s->ctx;
  if (n_views <= 0 || n_views > (1 << 20)) return fail(ctx, SKW_ERR_ARG, "bad number of views");
  if (params->spp_x <= 0 || params->spp_y <= 0 || params->spp_x > 1024 || params->spp_y > 1024 ||
      params->light_samples < 0 || params->light_samples > 64 ||
      (params->sampler != SKW_SAMPLER_STRATIFIED && params->sampler != SKW_SAMPLER_LD) ||
      (params->sampler == SKW_SAMPLER_LD && (int64_t)params->spp_x * params->spp_y > 4096))
    return fail(ctx, SKW_ERR_ARG, "bad render parameters");
  if (cfg.stack_cap != 0 && (!valid_cap(cfg.stack_cap) || cfg.stack_cap < s->accel->stack_cap))
    return fail(ctx, SKW_ERR_ARG, "stack_cap must be 48, 96, 192 or 416 and cover the tree's depth");
  if (cfg.shade_block != 64 && cfg.shade_block != 128) return fail(ctx, SKW_ERR_ARG, "shade_block must be 64 or 128");
  if (cfg.samples_per_pass < 1 || cfg.trace_ctas_per_sm < 0) return fail(ctx, SKW_ERR_ARG, "bad pass configuration");
  P->views.assign((size_t)n_views, skw::ViewDev{});
  P->film_offset.assign((size_t)n_views, 0);
  int64_t px = 0;
  for (int v = 0; v < n_views; ++v) {
    const skw_camera *cam = cams + v;
    if (cam->width <= 0 || cam->height <= 0 || !(cam->x_view_angle > 0.0) || !(cam->x_view_angle < 3.14159265358979))
      return fail(ctx, SKW_ERR_ARG, "bad camera");
    skw::ViewDev &V = P->views[(size_t)v];
    std::memcpy(V.cam.c2w, cam->camera_to_world, sizeof(V.cam.c2w));
    V.cam.x_tan = std::tan(cam->x_view_angle / 2.0);  // PerspectiveCamera.cpp:19-33
    V.cam.y_tan = V.cam.x_tan * (double)cam->height / cam->width;
    V.cam.width = cam->width;
    V.cam.height = cam->height;
    for (int k = 0; k < 12; ++k) V.cam.m[k] = (float)cam->camera_to_world[k];
    V.cam.sx = (float)(2.0 * V.cam.x_tan / cam->width);
    V.cam.sy = (float)(2.0 * V.cam.y_tan / cam->height);
    V.px_begin = px;
    V.seed = seeds ? seeds[v] : params->seed + (uint64_t)v;
    P->film_offset[(size_t)v] = 3 * px;
    px += (int64_t)cam->width * cam->height;
  }
  P->sppx = params->spp_x;
  P->sppy = params->spp_y;
  P->nl = params->light_samples;
  P->ld = params->sampler == SKW_SAMPLER_LD;
  if (P->ld) {  // LDSampler / Sampler::AddSamplesSequence*: counts rounded up to powers of two
    int spp = 1, nl = 1;
    while (spp < P->sppx * P->sppy) spp <<= 1;
    while (nl < P->nl) nl <<= 1;
    P->sppx = spp;
    P->sppy = 1;
    if (P->nl > 0) P->nl = nl;
  }
  P->spp = P->sppx * P->sppy;
  P->npl = s->dev.n_point_lights;
  P->media = cfg.media && s->dev.medium.on;
  P->spec_levels = cfg.specular && s->dev.has_specular ? s->dev.max_spec_depth + 1 : 0;
  P->slots = 1 + 2 * P->nl + P->npl + cfg.extra_slots + (P->spec_levels ? 1 : 0) + (P->media ? 1 : 0);
  P->media_slot = P->slots - 1;
  P->spec_slot = P->slots - 1 - (P->media ? 1 : 0);
  P->n_px_total = px;
  P->cfg = cfg;
  if (P->cfg.stack_cap == 0) P->cfg.stack_cap = s->accel->stack_cap;
  int64_t per_pass = cfg.samples_per_pass;
  if (P->media)  // the media queue holds max_steps light samples per camera ray: at most 2^25 per pass
    per_pass = std::min<int64_t>(per_pass, std::max<int64_t>(((int64_t)1 << 25) / s->dev.medium.max_steps, 1));
  if (P->spec_levels)  // every sample's full specular tree fits the largest level's queue
    per_pass = std::min<int64_t>(per_pass, std::max<int64_t>(kSpecEntries >> P->spec_levels, 1));
  P->chunk_px = std::max<int64_t>(1, std::min<int64_t>(px, per_pass / P->spp));
  P->cap_samples = P->chunk_px * P->spp;
  P->cap_media = P->media ? P->cap_samples * s->dev.medium.max_steps : 0;
  P->cap_spec = P->spec_levels ? P->cap_samples << P->spec_levels : 0;
  const int64_t shaded = std::max(P->cap_samples, P->cap_spec);  // entries of the largest shade launch
  P->cap_shadow = shaded * (P->nl + P->npl);
  P->cap_bsdf = shaded * P->nl;
  if (P->cap_shadow > INT32_MAX / 2 || P->cap_bsdf > INT32_MAX / 2 || P->cap_samples > INT32_MAX / 2 ||
      P->cap_samples * P->slots * 3 > ((int64_t)1 << 40))
    return fail(ctx, SKW_ERR_ARG, "render pass too large");
  return SKW_OK;
}

// The medium stages of a pass: march + light samples, their any-hit
// traversal, and their resolve (forward: radiance into the medium slot;
// adjoint: the emission-scale gradient).
cudaError_t record_media(skw_scene *s, const Plan &P, const Workspace &W, const skw::ViewDev *d_views, int64_t px0,
                         int n, bool adjoint, const float *dfilm, double *g_emission, cudaStream_t st) {
  skw_accel *a = s->accel;
  cudaError_t e = skw::launch_media(adjoint, s->dev, d_views, (int)P.views.size(), n, px0, P.spp, P.slots, P.media_slot,
                                    dfilm, W.rays, W.hits, W.contrib, W.tcam, W.mrays, W.mtarget, W.mval, W.mdem,
                                    W.counts + 2, a->d_status, st);
  const int64_t cm = (int64_t)n * s->dev.medium.max_steps;
  if (e == cudaSuccess)
    e = skw::launch_traversal(false, P.cfg.stack_cap, a->d_nodes, a->d_tris, W.mrays, cm, W.counts + 2, a->scene_abs,
                              nullptr, W.mocc, a->d_status, st, P.cfg.trace_ctas_per_sm, W.counts + 8);
  if (e == cudaSuccess)
    e = skw::launch_resolve_media(adjoint, cm, W.mocc, W.mtarget, W.mval, W.mdem, W.counts + 2, P.slots, P.media_slot,
                                  W.contrib, g_emission, st);
  return e;
}

// The specular levels of a pass (after the camera level queued its
// children in queue 0): level L (1 .. spec_levels) holds at most n << L
// rays; each is traced, shaded (emission and direct lighting added into its
// sample's specular slot) and queues its children while L <= the scene's
// max_spec_depth.
// Extra stages for the entries of a specular level (the photon-map render's
// caustic and gather terms): called after the level's direct lighting with
// the level's queue (its rays, their hits, weights, samples, nodes), its
// device count and its capacity.
struct SpecLevel {
  const void *rays, *hits;
  const float *w;
  const int *sample, *node, *count;
  int64_t capacity;
};
using SpecHook = std::function<cudaError_t(const SpecLevel &)>;

// The medium along specular level L's rays (LTEIntegrator::Radiance of each
// specular ray), queue qi holding at most cl entries, marched in chunks of
// the pass's sample count (the media queue's capacity).  On a stream the
// level's length is read back and the chunks launched for it; in a graph
// capture the chunks run in a conditional while-node whose body advances a
// device offset (counts[11]) until it passes the level's device length, so
// the graph needs no host round trip.  body: a stream not otherwise in use
// by the capture, on which the loop's body is captured.  adjoint: the
// entries' weights and the in-scattering's emission-scale derivative only.
cudaError_t record_media_level(skw_scene *s, const Plan &P, const Workspace &W, const skw::ViewDev *d_views,
                               int64_t px0, int qi, int64_t cl, bool adjoint, const float *dfilm, double *g_emission,
                               cudaStream_t st, cudaStream_t body) {
  skw_accel *a = s->accel;
  const int nv = (int)P.views.size(), cap = P.cfg.stack_cap, ctas = P.cfg.trace_ctas_per_sm;
  const int chunk = (int)P.cap_samples;
  const int64_t cm = (int64_t)chunk * s->dev.medium.max_steps;
  int *count = W.counts + 3 + qi, *off = W.counts + 11;
  // one chunk: the march, the light samples' occlusion, their resolve
  auto run = [&](const void *rays, const void *hits, const int *sample, float *w, const int *node, int m,
                 const skw::MediaChunk &c, cudaStream_t sq) -> cudaError_t {
    cudaError_t r = cudaMemsetAsync(W.counts + 2, 0, sizeof(int), sq);
    if (r == cudaSuccess)
      r = skw::launch_media_specular(adjoint, s->dev, d_views, nv, m, px0, P.spp, P.slots, P.spec_slot, rays, hits,
                                     sample, w, node, c, dfilm, adjoint ? W.tcam : nullptr, W.contrib, W.mrays,
                                     W.mtarget, W.mval, W.mdem, W.counts + 2, a->d_status, sq);
    if (r == cudaSuccess)
      r = skw::launch_traversal(false, cap, a->d_nodes, a->d_tris, W.mrays, (int64_t)m * s->dev.medium.max_steps,
                                W.counts + 2, a->scene_abs, nullptr, W.mocc, a->d_status, sq, ctas, W.counts + 8);
    if (r == cudaSuccess)
      r = skw::launch_resolve_media(adjoint, cm, W.mocc, W.mtarget, W.mval, W.mdem, W.counts + 2, 1, 0, W.contrib,
                                    g_emission, sq);
    return r;
  };
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(st, &cs);
  if (e != cudaSuccess) return e;
  if (cs != cudaStreamCaptureStatusActive) {
    int cnt = 0;
    if ((e = cudaMemcpyAsync(&cnt, count, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (e = cudaStreamSynchronize(st)) != cudaSuccess)
      return e;
    cnt = (int)std::min<int64_t>(cnt, cl);
    for (int o = 0; o < cnt && e == cudaSuccess; o += chunk) {
      const int m = std::min(chunk, cnt - o);
      e = run((const char *)W.qrays[qi] + 32 * (int64_t)o, (const char *)W.qhits + 16 * (int64_t)o,
              W.qsample[qi] + o, W.qw[qi] + 3 * (int64_t)o, W.qnode[qi] + o, m, skw::MediaChunk{}, st);
    }
    return e;
  }
  if (!body) return cudaErrorNotSupported;
  if ((e = cudaMemsetAsync(off, 0, sizeof(int), st)) != cudaSuccess) return e;
  cudaGraph_t g = nullptr;
  const cudaGraphNode_t *deps = nullptr;
  size_t nd = 0;
  if ((e = cudaStreamGetCaptureInfo(st, &cs, nullptr, &g, &deps, nullptr, &nd)) != cudaSuccess) return e;
  cudaGraphConditionalHandle h;
  if ((e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault)) != cudaSuccess) return e;
  cudaGraphNodeParams np{};
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = h;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node = nullptr;
  if ((e = cudaGraphAddNode(&node, g, deps, nullptr, nd, &np)) != cudaSuccess) return e;
  cudaGraph_t bg = np.conditional.phGraph_out[0];
  if ((e = cudaStreamBeginCaptureToGraph(body, bg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)) !=
      cudaSuccess)
    return e;
  cudaError_t eb = run(W.qrays[qi], W.qhits, W.qsample[qi], W.qw[qi], W.qnode[qi], chunk,
                       skw::MediaChunk{off, count, cl}, body);
  if (eb == cudaSuccess) eb = skw::launch_media_advance(h, off, count, chunk, cl, body);
  e = cudaStreamEndCapture(body, &bg);
  if (eb != cudaSuccess) return eb;
  if (e != cudaSuccess) return e;
  return cudaStreamUpdateCaptureDependencies(st, &node, nullptr, 1, cudaStreamSetCaptureDependencies);
}

cudaError_t record_specular(skw_scene *s, const Plan &P, const Workspace &W, const skw::ViewDev *d_views, int64_t px0,
                            int n, cudaStream_t st, const SpecHook *hook, cudaStream_t body) {
  skw_accel *a = s->accel;
  const int nv = (int)P.views.size(), cap = P.cfg.stack_cap, ctas = P.cfg.trace_ctas_per_sm;
  cudaError_t e = cudaSuccess;
  for (int L = 1; L <= P.spec_levels; ++L) {
    const int qi = (L - 1) & 1, qo = L & 1;
    const int64_t cl = (int64_t)n << L;
    skw::SpecQueues q{};
    q.in_rays = W.qrays[qi];
    q.in_w = W.qw[qi];
    q.in_sample = W.qsample[qi];
    q.in_node = W.qnode[qi];
    q.in_count = W.counts + 3 + qi;
    q.spec_slot = P.spec_slot;
    if (L < P.spec_levels) {  // depth L <= max_spec_depth: children go to the next level
      q.out_rays = W.qrays[qo];
      q.out_w = W.qw[qo];
      q.out_sample = W.qsample[qo];
      q.out_node = W.qnode[qo];
      q.out_count = W.counts + 3 + qo;
      if ((e = cudaMemsetAsync(W.counts + 3 + qo, 0, sizeof(int), st)) != cudaSuccess) return e;
    }
    if ((e = cudaMemsetAsync(W.counts, 0, 2 * sizeof(int), st)) != cudaSuccess) return e;
    if ((e = skw::launch_traversal(true, cap, a->d_nodes, a->d_tris, W.qrays[qi], cl, W.counts + 3 + qi, a->scene_abs,
                                   nullptr, W.qhits, a->d_status, st, ctas, W.counts + 8, true)) != cudaSuccess)
      return e;
    if (P.media && (e = record_media_level(s, P, W, d_views, px0, qi, cl, false, nullptr, nullptr, st, body)) !=
                       cudaSuccess)
      return e;
    if ((e = skw::launch_shade_specular(s->dev, d_views, nv, cl, px0, P.spp, P.slots, P.nl, q, L, W.qhits, W.contrib,
                                        W.srays, W.starget, W.srgb, W.counts, W.brays, W.btarget, W.brgb,
                                        W.counts + 1, W.bnrm, st)) != cudaSuccess)
      return e;
    const int64_t csh = cl * (P.nl + P.npl), cbs = cl * P.nl;
    if (csh > 0 && (e = skw::launch_traversal(false, cap, a->d_nodes, a->d_tris, W.srays, csh, W.counts,
                                              a->scene_abs, nullptr, W.occ, a->d_status, st, ctas, W.counts + 8, true)) != cudaSuccess)
      return e;
    if (cbs > 0 && (e = skw::launch_traversal(true, cap, a->d_nodes, a->d_tris, W.brays, cbs, W.counts + 1,
                                              a->scene_abs, nullptr, W.bhits, a->d_status, st, ctas, W.counts + 8, true)) != cudaSuccess)
      return e;
    if ((e = skw::launch_resolve(s->dev, (int)std::max(csh, cbs), P.nl, W.occ, W.starget, W.srgb, W.counts, W.brays,
                                 W.bhits, W.btarget, W.brgb, W.counts + 1, W.bnrm, W.contrib, st, true)) !=
        cudaSuccess)
      return e;
    if (hook && (e = (*hook)(SpecLevel{W.qrays[qi], W.qhits, W.qw[qi], W.qsample[qi], W.qnode[qi],
                                       W.counts + 3 + qi, cl})) != cudaSuccess)
      return e;
  }
  return e;
}

// The direct-lighting stages of one pass over global pixels
// [px0, px0 + n_px): every slot of contrib but the extra ones is filled.
cudaError_t record_direct(skw_scene *s, const Plan &P, const Workspace &W, const skw::ViewDev *d_views, int64_t px0,
                          int n_px, cudaStream_t st, const SpecHook *hook = nullptr, cudaStream_t body = nullptr) {
  skw_accel *a = s->accel;
  const int n = n_px * P.spp, nv = (int)P.views.size(), cap = P.cfg.stack_cap, ctas = P.cfg.trace_ctas_per_sm;
  cudaError_t e;
  if ((e = cudaMemsetAsync(W.contrib, 0, (size_t)n * P.slots * 12, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(W.counts, 0, 5 * sizeof(int), st)) != cudaSuccess) return e;
  if ((e = skw::launch_camera(d_views, nv, px0, n_px, P.sppx, P.sppy, W.rays, st, P.ld)) != cudaSuccess) return e;
  if ((e = skw::launch_traversal(true, cap, a->d_nodes, a->d_tris, W.rays, n, nullptr, a->scene_abs, nullptr, W.hits,
                                 a->d_status, st, ctas, W.counts + 8)) != cudaSuccess)
    return e;
  if (P.media && (e = record_media(s, P, W, d_views, px0, n, false, nullptr, nullptr, st)) != cudaSuccess) return e;
  skw::SpecQueues sq{};
  if (P.spec_levels) {
    sq.out_rays = W.qrays[0];
    sq.out_w = W.qw[0];
    sq.out_sample = W.qsample[0];
    sq.out_node = W.qnode[0];
    sq.out_count = W.counts + 3;
    sq.spec_slot = P.spec_slot;
  }
  if ((e = skw::launch_shade(s->dev, d_views, nv, n, px0, P.spp, P.slots, P.nl, W.rays, W.hits, W.contrib, W.srays,
                             W.starget, W.srgb, W.counts, W.brays, W.btarget, W.brgb, W.counts + 1, W.bnrm,
                             P.cfg.shade_block, st, P.spec_levels ? &sq : nullptr, P.ld)) != cudaSuccess)
    return e;
  const int64_t csh = (int64_t)n * (P.nl + P.npl), cbs = (int64_t)n * P.nl;
  if (csh > 0 && (e = skw::launch_traversal(false, cap, a->d_nodes, a->d_tris, W.srays, csh, W.counts, a->scene_abs,
                                            nullptr, W.occ, a->d_status, st, ctas, W.counts + 8, true)) != cudaSuccess)
    return e;
  if (cbs > 0 && (e = skw::launch_traversal(true, cap, a->d_nodes, a->d_tris, W.brays, cbs, W.counts + 1,
                                            a->scene_abs, nullptr, W.bhits, a->d_status, st, ctas, W.counts + 8, true)) != cudaSuccess)
    return e;
  if ((e = skw::launch_resolve(s->dev, (int)std::max(csh, cbs), P.nl, W.occ, W.starget, W.srgb, W.counts, W.brays,
                               W.bhits, W.btarget, W.brgb, W.counts + 1, W.bnrm, W.contrib, st)) != cudaSuccess)
    return e;
  return record_specular(s, P, W, d_views, px0, n, st, hook, body);
}

// Side streams and events of one pass workspace: a level's shadow and BSDF
// traversals run on aux[0] and aux[1] while the pass's own stream traces the
// next specular level.
struct Lanes {
  cudaStream_t aux[2] = {nullptr, nullptr};
  cudaEvent_t fork = nullptr, join[2] = {nullptr, nullptr};
  bool ready() const { return aux[0] && aux[1] && fork && join[0] && join[1]; }
};

cudaError_t lanes_events(Lanes &L) {
  cudaError_t e = cudaEventCreateWithFlags(&L.fork, cudaEventDisableTiming);
  for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&L.join[i], cudaEventDisableTiming);
  return e;
}

void lanes_release_events(Lanes &L) {
  for (cudaEvent_t ev : {L.fork, L.join[0], L.join[1]})
    if (ev) cudaEventDestroy(ev);
  L.fork = L.join[0] = L.join[1] = nullptr;
}

// Lanes of a single-camera render: the context's side streams (shared by the
// context's callers; each call orders its own work on them with its own
// events) and this call's events.  On failure the lanes stay incomplete and
// the pass runs its stages in turn.
void render_lanes(skw_ctx *ctx, Lanes &L) {
  {
    std::lock_guard<std::mutex> lock(ctx->aux_mu);
    for (int i = 0; i < 2; ++i)
      if (!ctx->aux_st[i] && cudaStreamCreateWithFlags(&ctx->aux_st[i], cudaStreamNonBlocking) != cudaSuccess) {
        ctx->aux_st[i] = nullptr;
        cudaGetLastError();
      }
    L.aux[0] = ctx->aux_st[0];
    L.aux[1] = ctx->aux_st[1];
  }
  if (lanes_events(L) != cudaSuccess) {
    lanes_release_events(L);
    cudaGetLastError();
  }
}

// The direct-lighting stages of one pass with the levels overlapped (no
// medium, no per-level hook).  The order of dependent work is the one of
// record_direct; what changes is what runs at the same time:
//   main:   camera, trace, shade(0) | trace(1)  | resolve(0), shade(1) | trace(2) ...
//   aux[0]:                          shadow(0) |                      | shadow(1) ...
//   aux[1]:                          BSDF(0)   |                      | BSDF(1) ...
// A level's shadow and BSDF traversals and the next level's traversal read
// different queues and write different outputs (each launch with its own
// ray-group counter, counts[8..10]); the main stream waits for both side
// streams before the level's resolve, which precedes the next shade that
// refills the shadow and BSDF queues.  Small levels (a few tens of
// thousands of rays each) no longer leave the GPU mostly idle in turn.
cudaError_t record_direct_pipelined(skw_scene *s, const Plan &P, const Workspace &W, const skw::ViewDev *d_views,
                                    int64_t px0, int n_px, cudaStream_t st, const Lanes &ln) {
  skw_accel *a = s->accel;
  const int n = n_px * P.spp, nv = (int)P.views.size(), cap = P.cfg.stack_cap, ctas = P.cfg.trace_ctas_per_sm;
  cudaError_t e;
  if ((e = cudaMemsetAsync(W.contrib, 0, (size_t)n * P.slots * 12, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(W.counts, 0, 5 * sizeof(int), st)) != cudaSuccess) return e;
  if ((e = skw::launch_camera(d_views, nv, px0, n_px, P.sppx, P.sppy, W.rays, st, P.ld)) != cudaSuccess) return e;
  if ((e = skw::launch_traversal(true, cap, a->d_nodes, a->d_tris, W.rays, n, nullptr, a->scene_abs, nullptr, W.hits,
                                 a->d_status, st, ctas, W.counts + 8)) != cudaSuccess)
    return e;
  skw::SpecQueues sq{};
  if (P.spec_levels) {
    sq.out_rays = W.qrays[0];
    sq.out_w = W.qw[0];
    sq.out_sample = W.qsample[0];
    sq.out_node = W.qnode[0];
    sq.out_count = W.counts + 3;
    sq.spec_slot = P.spec_slot;
  }
  if ((e = skw::launch_shade(s->dev, d_views, nv, n, px0, P.spp, P.slots, P.nl, W.rays, W.hits, W.contrib, W.srays,
                             W.starget, W.srgb, W.counts, W.brays, W.btarget, W.brgb, W.counts + 1, W.bnrm,
                             P.cfg.shade_block, st, P.spec_levels ? &sq : nullptr, P.ld)) != cudaSuccess)
    return e;
  // the shadow and BSDF traversals of a level, on the side streams
  auto side = [&](int64_t csh, int64_t cbs) -> cudaError_t {
    cudaError_t r = cudaEventRecord(ln.fork, st);
    for (int i = 0; i < 2 && r == cudaSuccess; ++i) r = cudaStreamWaitEvent(ln.aux[i], ln.fork, 0);
    if (r == cudaSuccess && csh > 0)
      r = skw::launch_traversal(false, cap, a->d_nodes, a->d_tris, W.srays, csh, W.counts, a->scene_abs, nullptr,
                                W.occ, a->d_status, ln.aux[0], ctas, W.counts + 9, true);
    if (r == cudaSuccess && cbs > 0)
      r = skw::launch_traversal(true, cap, a->d_nodes, a->d_tris, W.brays, cbs, W.counts + 1, a->scene_abs, nullptr,
                                W.bhits, a->d_status, ln.aux[1], ctas, W.counts + 10, true);
    for (int i = 0; i < 2 && r == cudaSuccess; ++i) r = cudaEventRecord(ln.join[i], ln.aux[i]);
    return r;
  };
  // ... and their resolve, on the pass's stream once both are done
  auto resolve = [&](int64_t csh, int64_t cbs, bool accumulate) -> cudaError_t {
    cudaError_t r = cudaSuccess;
    for (int i = 0; i < 2 && r == cudaSuccess; ++i) r = cudaStreamWaitEvent(st, ln.join[i], 0);
    if (r == cudaSuccess)
      r = skw::launch_resolve(s->dev, (int)std::max(csh, cbs), P.nl, W.occ, W.starget, W.srgb, W.counts, W.brays,
                              W.bhits, W.btarget, W.brgb, W.counts + 1, W.bnrm, W.contrib, st, accumulate);
    return r;
  };
  int64_t csh = (int64_t)n * (P.nl + P.npl), cbs = (int64_t)n * P.nl;
  if ((e = side(csh, cbs)) != cudaSuccess) return e;
  for (int L = 1; L <= P.spec_levels; ++L) {
    const int qi = (L - 1) & 1, qo = L & 1;
    const int64_t cl = (int64_t)n << L;
    if ((e = skw::launch_traversal(true, cap, a->d_nodes, a->d_tris, W.qrays[qi], cl, W.counts + 3 + qi, a->scene_abs,
                                   nullptr, W.qhits, a->d_status, st, ctas, W.counts + 8, true)) != cudaSuccess)
      return e;
    if ((e = resolve(csh, cbs, L > 1)) != cudaSuccess) return e;
    skw::SpecQueues q{};
    q.in_rays = W.qrays[qi];
    q.in_w = W.qw[qi];
    q.in_sample = W.qsample[qi];
    q.in_node = W.qnode[qi];
    q.in_count = W.counts + 3 + qi;
    q.spec_slot = P.spec_slot;
    if (L < P.spec_levels) {  // depth L <= max_spec_depth: children go to the next level
      q.out_rays = W.qrays[qo];
      q.out_w = W.qw[qo];
      q.out_sample = W.qsample[qo];
      q.out_node = W.qnode[qo];
      q.out_count = W.counts + 3 + qo;
      if ((e = cudaMemsetAsync(W.counts + 3 + qo, 0, sizeof(int), st)) != cudaSuccess) return e;
    }
    if ((e = cudaMemsetAsync(W.counts, 0, 2 * sizeof(int), st)) != cudaSuccess) return e;
    if ((e = skw::launch_shade_specular(s->dev, d_views, nv, cl, px0, P.spp, P.slots, P.nl, q, L, W.qhits, W.contrib,
                                        W.srays, W.starget, W.srgb, W.counts, W.brays, W.btarget, W.brgb,
                                        W.counts + 1, W.bnrm, st)) != cudaSuccess)
      return e;
    csh = cl * (P.nl + P.npl);
    cbs = cl * P.nl;
    if ((e = side(csh, cbs)) != cudaSuccess) return e;
  }
  return resolve(csh, cbs, P.spec_levels > 0);
}

// One pass: direct lighting, then the film.
cudaError_t record_pass(skw_scene *s, const Plan &P, const Workspace &W, const skw::ViewDev *d_views, int64_t px0,
                        int n_px, float *films, cudaStream_t st, const Lanes *ln) {
  cudaError_t e = ln && ln->ready() && !P.media ? record_direct_pipelined(s, P, W, d_views, px0, n_px, st, *ln)
                                                 : record_direct(s, P, W, d_views, px0, n_px, st, nullptr, ln ? ln->aux[0] : nullptr);
  if (e != cudaSuccess) return e;
  return skw::launch_film(W.contrib, px0, n_px, P.spp, P.slots, films, st, P.media ? W.tcam : nullptr, P.media_slot);
}

constexpr int kLaunchesPerPass = 8;

// Kernel launches of one pass: the direct-lighting stages, 6 per specular
// level (traversal, shade, two traversals, two resolves) and 3 for a medium.
int64_t launches_per_pass(const Plan &P) { return kLaunchesPerPass + 6 * P.spec_levels + (P.media ? 3 : 0); }

int64_t n_passes(const Plan &P) { return (P.n_px_total + P.chunk_px - 1) / P.chunk_px; }

// All passes.  With two workspaces, passes alternate between them on two
// streams (st and side), joined back into st at the end.
cudaError_t record_all(skw_scene *s, const Plan &P, const Workspace *W, int n_ws, const skw::ViewDev *d_views,
                       float *films, cudaStream_t st, cudaStream_t side, cudaEvent_t fork, cudaEvent_t join,
                       const Lanes *lanes) {
  cudaError_t e = cudaSuccess;
  if (n_ws > 1) {
    if ((e = cudaEventRecord(fork, st)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(side, fork, 0)) != cudaSuccess) return e;
  }
  int64_t k = 0;
  for (int64_t px0 = 0; px0 < P.n_px_total; px0 += P.chunk_px, ++k) {
    const int n_px = (int)std::min<int64_t>(P.chunk_px, P.n_px_total - px0);
    const int w = n_ws > 1 ? (int)(k & 1) : 0;
    if ((e = record_pass(s, P, W[w], d_views, px0, n_px, films, w ? side : st, lanes ? &lanes[w] : nullptr)) !=
        cudaSuccess)
      return e;
  }
  if (n_ws > 1) {
    if ((e = cudaEventRecord(join, side)) != cudaSuccess) return e;
    if ((e = cudaStreamWaitEvent(st, join, 0)) != cudaSuccess) return e;
  }
  return e;
}

}  // namespace

struct skw_render_batch {
  skw_scene *scene = nullptr;
  Plan plan;
  skw_render_params params{};
  std::vector<uint64_t> seeds;
  std::vector<skw_camera> cams;
  char *ws = nullptr;  // workspaces (one or two)
  size_t ws_bytes = 0;
  skw::ViewDev *d_views = nullptr;
  cudaStream_t own = nullptr, side = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr, fork = nullptr, join = nullptr;
  cudaGraphExec_t exec = nullptr;
  float *graph_films = nullptr;
  Lanes lanes[2];  // side streams of the two workspaces' levels
};

namespace {

void batch_release(skw_render_batch *b) {
  // Launches of the old graph still in flight use the workspace.
  if (b->own) cudaStreamSynchronize(b->own);
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
  b->graph_films = nullptr;
}

// (Re)builds the plan for cfg and makes sure the workspace is large enough.
int batch_configure(skw_render_batch *b, const PassConfig &cfg) {
  skw_ctx *ctx = b->scene->ctx;
  Plan P;
  int rc = plan_make(b->scene, b->cams.data(), (int)b->cams.size(), &b->params, b->seeds.data(), cfg, &P);
  if (rc != SKW_OK) return rc;
  cudaError_t e;
  if ((e = skw::prepare_traversal(P.cfg.stack_cap)) != cudaSuccess) return cuda_fail(ctx, e, "traversal occupancy");
  const int n_ws = P.cfg.overlap && n_passes(P) > 1 ? 2 : 1;
  const size_t need = workspace_bytes(P) * (size_t)n_ws;
  batch_release(b);
  if (need > b->ws_bytes) {
    if (b->ws) cudaFree(b->ws);
    b->ws = nullptr;
    b->ws_bytes = 0;
    if ((e = cudaMalloc((void **)&b->ws, need)) != cudaSuccess) return cuda_fail(ctx, e, "batch workspace");
    b->ws_bytes = need;
  }
  batch_release(b);
  b->plan = std::move(P);
  return SKW_OK;
}

int batch_capture(skw_render_batch *b, float *films) {
  skw_ctx *ctx = b->scene->ctx;
  const Plan &P = b->plan;
  const int n_ws = P.cfg.overlap && n_passes(P) > 1 ? 2 : 1;
  Workspace W[2];
  const size_t one = workspace_bytes(P);
  for (int i = 0; i < n_ws; ++i) workspace_carve(P, b->ws + one * (size_t)i, &W[i]);
  batch_release(b);
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamBeginCapture(b->own, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "graph capture");
  cudaError_t er = record_all(b->scene, P, W, n_ws, b->d_views, films, b->own, b->side, b->fork, b->join, b->lanes);
  e = cudaStreamEndCapture(b->own, &g);
  if (er != cudaSuccess || e != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    cudaGetLastError();
    return cuda_fail(ctx, er != cudaSuccess ? er : e, "graph capture");
  }
  e = cudaGraphInstantiate(&b->exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    b->exec = nullptr;
    return cuda_fail(ctx, e, "graph instantiate");
  }
  b->graph_films = films;
  return SKW_OK;
}

// Launches the graph on the batch's stream, ordered after `stream` and
// before whatever is queued on `stream` next.
int batch_launch(skw_render_batch *b, float *films, cudaStream_t stream) {
  skw_ctx *ctx = b->scene->ctx;
  if (!b->exec || b->graph_films != films) {
    int rc = batch_capture(b, films);
    if (rc != SKW_OK) return rc;
  }
  cudaError_t e;
  if ((e = cudaEventRecord(b->ev_in, stream)) != cudaSuccess) return cuda_fail(ctx, e, "batch run");
  if ((e = cudaStreamWaitEvent(b->own, b->ev_in, 0)) != cudaSuccess) return cuda_fail(ctx, e, "batch run");
  if ((e = cudaGraphLaunch(b->exec, b->own)) != cudaSuccess) return cuda_fail(ctx, e, "graph launch");
  if ((e = cudaEventRecord(b->ev_out, b->own)) != cudaSuccess) return cuda_fail(ctx, e, "batch run");
  if ((e = cudaStreamWaitEvent(stream, b->ev_out, 0)) != cudaSuccess) return cuda_fail(ctx, e, "batch run");
  ctx->launches.fetch_add(n_passes(b->plan) * launches_per_pass(b->plan));
  return SKW_OK;
}

PassConfig to_pass_config(const skw_batch_config *c) {
  PassConfig p;
  if (!c) {
    p.overlap = 1;
    return p;
  }
  p.samples_per_pass = c->samples_per_pass;
  p.stack_cap = c->stack_cap;
  p.trace_ctas_per_sm = c->trace_ctas_per_sm;
  p.shade_block = c->shade_block;
  p.overlap = c->overlap;
  return p;
}

void from_pass_config(const PassConfig &p, skw_batch_config *c) {
  c->samples_per_pass = p.samples_per_pass;
  c->stack_cap = p.stack_cap;
  c->trace_ctas_per_sm = p.trace_ctas_per_sm;
  c->shade_block = p.shade_block;
  c->overlap = p.overlap;
}

}  // namespace

extern "C" {

int skw_render_direct(skw_scene *s, const skw_camera *cam, const skw_render_params *params, float *film_rgb,
                      void *stream) {
  if (!s || !cam || !params || !film_rgb) return fail(s ? s->ctx : nullptr, SKW_ERR_ARG, "null argument");
  skw_ctx *ctx = s->ctx;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaSetDevice");
  Plan P;
  const uint64_t seed = params->seed;
  PassConfig cfg;
  int rc = plan_make(s, cam, 1, params, &seed, cfg, &P);
  if (rc != SKW_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  cudaMemPool_t pool;
  if ((e = skw::ctx_pool(ctx, &pool)) != cudaSuccess) return cuda_fail(ctx, e, "workspace pool");
  const size_t wbytes = workspace_bytes(P), vbytes = al256(sizeof(skw::ViewDev));
  char *w = nullptr;
  if ((e = cudaMallocFromPoolAsync((void **)&w, wbytes + vbytes, pool, st)) != cudaSuccess)
    return cuda_fail(ctx, e, "render workspace");
  Workspace W;
  workspace_carve(P, w, &W);
  skw::ViewDev *d_view = (skw::ViewDev *)(w + wbytes);
  e = cudaMemcpyAsync(d_view, P.views.data(), sizeof(skw::ViewDev), cudaMemcpyHostToDevice, st);
  Lanes ln;
  if (e == cudaSuccess && !P.media) render_lanes(ctx, ln);  // without side streams the stages run in turn
  if (e == cudaSuccess) e = record_all(s, P, &W, 1, d_view, film_rgb, st, nullptr, nullptr, nullptr, &ln);
  lanes_release_events(ln);
  cudaFreeAsync(w, st);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "direct-lighting render");
  ctx->launches.fetch_add(n_passes(P) * launches_per_pass(P));
  return SKW_OK;
}

int skw_render_batch_create(skw_scene *s, const skw_camera *cams, int32_t n_views, const skw_render_params *params,
                            const uint64_t *view_seeds, const skw_batch_config *cfg, skw_render_batch **out) {
  if (out) *out = nullptr;
  if (!s || !cams || !params || !out) return fail(s ? s->ctx : nullptr, SKW_ERR_ARG, "null argument");
  skw_ctx *ctx = s->ctx;
  if (n_views <= 0) return fail(ctx, SKW_ERR_ARG, "bad number of views");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaSetDevice");
  skw_render_batch *b = new (std::nothrow) skw_render_batch();
  if (!b) return fail(ctx, SKW_ERR_OOM, "host allocation");
  b->scene = s;
  b->params = *params;
  b->cams.assign(cams, cams + n_views);
  b->seeds.resize((size_t)n_views);
  for (int v = 0; v < n_views; ++v) b->seeds[(size_t)v] = view_seeds ? view_seeds[v] : params->seed + (uint64_t)v;
  int rc = batch_configure(b, to_pass_config(cfg));
  if (rc == SKW_OK) {
    if ((e = cudaMalloc((void **)&b->d_views, sizeof(skw::ViewDev) * (size_t)n_views)) != cudaSuccess ||
        (e = cudaMemcpy(b->d_views, b->plan.views.data(), sizeof(skw::ViewDev) * (size_t)n_views,
                        cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaStreamCreateWithFlags(&b->side, cudaStreamNonBlocking)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&b->ev_in, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&b->ev_out, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming)) != cudaSuccess ||
        (e = cudaEventCreateWithFlags(&b->join, cudaEventDisableTiming)) != cudaSuccess)
      rc = cuda_fail(ctx, e, "batch resources");
    for (int w = 0; w < 2 && rc == SKW_OK; ++w)
      for (int i = 0; i < 2 && rc == SKW_OK; ++i)
        if ((e = cudaStreamCreateWithFlags(&b->lanes[w].aux[i], cudaStreamNonBlocking)) != cudaSuccess ||
            (i == 0 && (e = lanes_events(b->lanes[w])) != cudaSuccess))
          rc = cuda_fail(ctx, e, "batch resources");
  }
  if (rc != SKW_OK) {
    skw_render_batch_destroy(b);
    return rc;
  }
  *out = b;
  return SKW_OK;
}

void skw_render_batch_destroy(skw_render_batch *b) {
  if (!b) return;
  if (b->own) cudaStreamSynchronize(b->own);
  if (b->side) cudaStreamSynchronize(b->side);
  batch_release(b);
  if (b->ws) cudaFree(b->ws);
  if (b->d_views) cudaFree(b->d_views);
  if (b->own) cudaStreamDestroy(b->own);
  if (b->side) cudaStreamDestroy(b->side);
  for (Lanes &L : b->lanes) {
    for (cudaStream_t &a : L.aux)
      if (a) cudaStreamDestroy(a);
    lanes_release_events(L);
  }
  for (cudaEvent_t ev : {b->ev_in, b->ev_out, b->fork, b->join})
    if (ev) cudaEventDestroy(ev);
  delete b;
}

int64_t skw_render_batch_film_floats(const skw_render_batch *b) { return b ? 3 * b->plan.n_px_total : -1; }

int64_t skw_render_batch_film_offset(const skw_render_batch *b, int32_t v) {
  if (!b || v < 0 || v >= (int32_t)b->plan.film_offset.size()) return -1;
  return b->plan.film_offset[(size_t)v];
}

int skw_render_batch_get_config(const skw_render_batch *b, skw_batch_config *out) {
  if (!b || !out) return SKW_ERR_ARG;
  from_pass_config(b->plan.cfg, out);
  return SKW_OK;
}

int skw_render_batch_run(skw_render_batch *b, float *films, void *stream) {
  if (!b || !films) return fail(b ? b->scene->ctx : nullptr, SKW_ERR_ARG, "null argument");
  cudaError_t e = cudaSetDevice(b->scene->ctx->device);
  if (e != cudaSuccess) return cuda_fail(b->scene->ctx, e, "cudaSetDevice");
  return batch_launch(b, films, (cudaStream_t)stream);
}

int skw_render_batch_autotune(skw_render_batch *b, float *scratch, void *stream, skw_batch_config *best_out,
                              float *best_ms_out, int32_t *n_candidates) {
  if (!b || !scratch) return fail(b ? b->scene->ctx : nullptr, SKW_ERR_ARG, "null argument");
  skw_ctx *ctx = b->scene->ctx;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaSetDevice");
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  if ((e = cudaEventCreate(&t0)) != cudaSuccess || (e = cudaEventCreate(&t1)) != cudaSuccess) {
    if (t0) cudaEventDestroy(t0);
    return cuda_fail(ctx, e, "autotune events");
  }
  int tried = 0;
  // Time of one run of cfg (ms), or a negative value if cfg is not usable.
  auto measure = [&](const PassConfig &cfg) -> float {
    if (batch_configure(b, cfg) != SKW_OK) return -1.0f;
    if (batch_launch(b, scratch, st) != SKW_OK) return -1.0f;  // capture + warm-up
    cudaEventRecord(t0, st);
    for (int r = 0; r < 2; ++r)
      if (batch_launch(b, scratch, st) != SKW_OK) return -1.0f;
    cudaEventRecord(t1, st);
    if (cudaEventSynchronize(t1) != cudaSuccess) return -1.0f;
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, t0, t1);
    ++tried;
    return ms / 2.0f;
  };
  PassConfig best = b->plan.cfg;
  float best_ms = measure(best);
  if (best_ms < 0) {
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    return fail(ctx, SKW_ERR_CUDA, "autotune: the starting configuration does not run");
  }
  auto consider = [&](PassConfig c) {
    const float ms = measure(c);
    if (ms > 0 && ms < best_ms) {
      best_ms = ms;
      best = c;
    }
  };
  const int64_t total = b->plan.n_px_total * b->plan.spp;
  for (int64_t q : {(int64_t)1 << 18, (int64_t)1 << 19, (int64_t)1 << 20, (int64_t)1 << 21, (int64_t)1 << 22,
                    (int64_t)1 << 23, (int64_t)1 << 24, (int64_t)1 << 25}) {
    if (q == best.samples_per_pass || q > 2 * total) continue;
    PassConfig c = best;
    c.samples_per_pass = q;
    consider(c);
  }
  {
    PassConfig c = best;
    c.overlap = best.overlap ? 0 : 1;
    consider(c);
  }
  const int max_ctas = skw::traversal_max_ctas_per_sm(best.stack_cap);
  for (int k : {max_ctas / 2, (3 * max_ctas) / 4}) {
    if (k < 1 || k >= max_ctas) continue;
    PassConfig c = best;
    c.trace_ctas_per_sm = k;
    consider(c);
  }
  for (int cap : {48, 96, 192, 416}) {
    if (cap <= best.stack_cap || cap < b->scene->accel->stack_cap) continue;
    PassConfig c = best;
    c.stack_cap = cap;
    consider(c);
    break;  // the next larger capacity only
  }
  {
    PassConfig c = best;
    c.shade_block = best.shade_block == 128 ? 64 : 128;
    consider(c);
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  int rc = batch_configure(b, best);
  if (rc != SKW_OK) return rc;
  if (best_out) from_pass_config(best, best_out);
  if (best_ms_out) *best_ms_out = best_ms;
  if (n_candidates) *n_candidates = tried;
  return SKW_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- adjoint --

extern "C" {

int64_t skw_scene_n_triangles(const skw_scene *s) { return s ? s->n_triangles : -1; }

int skw_scene_set_triangle_albedo(skw_scene *s, const float *albedo, void *stream) {
  if (!s || !albedo) return fail(s ? s->ctx : nullptr, SKW_ERR_ARG, "null argument");
  cudaError_t e = cudaSetDevice(s->ctx->device);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync((void *)s->dev.tri_albedo, albedo, (size_t)s->n_triangles * 3 * sizeof(float),
                        cudaMemcpyDefault, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(s->ctx, e, "set triangle albedo");
  return SKW_OK;
}

int skw_scene_set_emission_scale(skw_scene *s, float scale) {
  if (!s || !(scale >= 0.0f) || !std::isfinite(scale)) return fail(s ? s->ctx : nullptr, SKW_ERR_ARG, "bad scale");
  s->dev.emission_scale = scale;
  return SKW_OK;
}

int skw_render_direct_adjoint(skw_scene *s, const skw_camera *cam, const skw_render_params *params,
                              const float *d_film, float *g_albedo, double *g_emission, void *stream) {
  if (!s || !cam || !params || !d_film || !g_albedo || !g_emission)
    return fail(s ? s->ctx : nullptr, SKW_ERR_ARG, "null argument");
  skw_ctx *ctx = s->ctx;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaSetDevice");
  Plan P;
  const uint64_t seed = params->seed;
  int rc = plan_make(s, cam, 1, params, &seed, PassConfig{}, &P);
  if (rc != SKW_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  cudaMemPool_t pool;
  if ((e = skw::ctx_pool(ctx, &pool)) != cudaSuccess) return cuda_fail(ctx, e, "workspace pool");
  const int64_t sh = std::max<int64_t>(P.cap_shadow, 1), bs = std::max<int64_t>(P.cap_bsdf, 1);
  const size_t wbytes = workspace_bytes(P), vbytes = al256(sizeof(skw::ViewDev)), xbytes = al256(sh * 4) + al256(bs * 12);
  char *w = nullptr;
  if ((e = cudaMallocFromPoolAsync((void **)&w, wbytes + vbytes + xbytes, pool, st)) != cudaSuccess)
    return cuda_fail(ctx, e, "adjoint workspace");
  Workspace W;
  workspace_carve(P, w, &W);
  skw::ViewDev *d_view = (skw::ViewDev *)(w + wbytes);
  float *s_dem = (float *)(w + wbytes + vbytes), *b_dkd = (float *)(w + wbytes + vbytes + al256(sh * 4));
  float *s_dkd = W.srgb;  // 3 floats per shadow entry, like the forward pass's radiance
  skw_accel *a = s->accel;
  e = cudaMemcpyAsync(d_view, P.views.data(), sizeof(skw::ViewDev), cudaMemcpyHostToDevice, st);
  skw::SpecQueues sq0{};  // the camera level's children go to queue 0
  if (P.spec_levels) {
    sq0.out_rays = W.qrays[0];
    sq0.out_w = W.qw[0];
    sq0.out_sample = W.qsample[0];
    sq0.out_node = W.qnode[0];
    sq0.out_count = W.counts + 3;
  }
  int64_t launches = 0;
  for (int64_t px0 = 0; px0 < P.n_px_total && e == cudaSuccess; px0 += P.chunk_px) {
    const int n_px = (int)std::min<int64_t>(P.chunk_px, P.n_px_total - px0);
    const int n = n_px * P.spp, cap = P.cfg.stack_cap;
    if ((e = cudaMemsetAsync(W.counts, 0, 5 * sizeof(int), st)) != cudaSuccess) break;
    if ((e = skw::launch_camera(d_view, 1, px0, n_px, P.sppx, P.sppy, W.rays, st, P.ld)) != cudaSuccess) break;
    if ((e = skw::launch_traversal(true, cap, a->d_nodes, a->d_tris, W.rays, n, nullptr, a->scene_abs, nullptr,
                                   W.hits, a->d_status, st, 0, W.counts + 8)) != cudaSuccess)
      break;
    if (P.media && (e = record_media(s, P, W, d_view, px0, n, true, d_film, g_emission, st)) != cudaSuccess) break;
    if ((e = skw::launch_shade_adjoint(s->dev, d_view, 1, n, px0, P.spp, P.nl, d_film, g_albedo, g_emission, W.rays,
                                       W.hits, W.srays, W.starget, s_dkd, s_dem, W.counts, W.brays, W.btarget, b_dkd,
                                       W.brgb, W.counts + 1, W.bnrm, P.media ? W.tcam : nullptr, st, P.ld,
                                       P.spec_levels ? &sq0 : nullptr)) != cudaSuccess)
      break;
    const int64_t csh = (int64_t)n * (P.nl + P.npl), cbs = (int64_t)n * P.nl;
    if (csh > 0 && (e = skw::launch_traversal(false, cap, a->d_nodes, a->d_tris, W.srays, csh, W.counts,
                                              a->scene_abs, nullptr, W.occ, a->d_status, st, 0, W.counts + 8, true)) != cudaSuccess)
      break;
    if (cbs > 0 && (e = skw::launch_traversal(true, cap, a->d_nodes, a->d_tris, W.brays, cbs, W.counts + 1,
                                              a->scene_abs, nullptr, W.bhits, a->d_status, st, 0, W.counts + 8, true)) != cudaSuccess)
      break;
    if ((e = skw::launch_resolve_adjoint(s->dev, (int)std::max(csh, cbs), P.nl, W.occ, W.starget, s_dkd, s_dem,
                                         W.counts, W.brays, W.bhits, W.btarget, b_dkd, W.brgb, W.counts + 1, W.bnrm,
                                         g_albedo, g_emission, st)) != cudaSuccess)
      break;
    launches += 7;
    // The specular levels, replayed as in record_specular with the adjoint
    // shading and resolves (the entries' weights scale dL/dI).
    for (int L = 1; L <= P.spec_levels && e == cudaSuccess; ++L) {
      const int qi = (L - 1) & 1, qo = L & 1;
      const int64_t cl = (int64_t)n << L;
      skw::SpecQueues q{};
      q.in_rays = W.qrays[qi];
      q.in_w = W.qw[qi];
      q.in_sample = W.qsample[qi];
      q.in_node = W.qnode[qi];
      q.in_count = W.counts + 3 + qi;
      if (L < P.spec_levels) {
        q.out_rays = W.qrays[qo];
        q.out_w = W.qw[qo];
        q.out_sample = W.qsample[qo];
        q.out_node = W.qnode[qo];
        q.out_count = W.counts + 3 + qo;
        if ((e = cudaMemsetAsync(W.counts + 3 + qo, 0, sizeof(int), st)) != cudaSuccess) break;
      }
      if ((e = cudaMemsetAsync(W.counts, 0, 2 * sizeof(int), st)) != cudaSuccess) break;
      if ((e = skw::launch_traversal(true, cap, a->d_nodes, a->d_tris, W.qrays[qi], cl, W.counts + 3 + qi,
                                     a->scene_abs, nullptr, W.qhits, a->d_status, st, 0, W.counts + 8, true)) != cudaSuccess)
        break;
      // the medium along the level's rays: the entries' weights take the
      // segments' transmittance, the in-scattering its emission derivative
      if (P.media &&
          (e = record_media_level(s, P, W, d_view, px0, qi, cl, true, d_film, g_emission, st, nullptr)) != cudaSuccess)
        break;
      if ((e = skw::launch_shade_specular_adjoint(s->dev, d_view, 1, cl, px0, P.spp, P.nl, d_film, g_albedo,
                                                  g_emission, q, L, W.qhits, W.srays, W.starget, s_dkd, s_dem,
                                                  W.counts, W.brays, W.btarget, b_dkd, W.brgb, W.counts + 1,
                                                  W.bnrm, st, P.media ? W.tcam : nullptr)) != cudaSuccess)
        break;
      const int64_t lsh = cl * (P.nl + P.npl), lbs = cl * P.nl;
      if (lsh > 0 && (e = skw::launch_traversal(false, cap, a->d_nodes, a->d_tris, W.srays, lsh, W.counts,
                                                a->scene_abs, nullptr, W.occ, a->d_status, st, 0, W.counts + 8, true)) != cudaSuccess)
        break;
      if (lbs > 0 && (e = skw::launch_traversal(true, cap, a->d_nodes, a->d_tris, W.brays, lbs, W.counts + 1,
                                                a->scene_abs, nullptr, W.bhits, a->d_status, st, 0, W.counts + 8, true)) != cudaSuccess)
        break;
      if ((e = skw::launch_resolve_adjoint(s->dev, (int)std::max(lsh, lbs), P.nl, W.occ, W.starget, s_dkd, s_dem,
                                           W.counts, W.brays, W.bhits, W.btarget, b_dkd, W.brgb, W.counts + 1,
                                           W.bnrm, g_albedo, g_emission, st, true)) != cudaSuccess)
        break;
      launches += 6;
    }
  }
  cudaFreeAsync(w, st);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "direct-lighting adjoint");
  ctx->launches.fetch_add(launches);
  return SKW_OK;
}

}  // extern "C"

// ------------------------------------------------------ photon-map render --

extern "C" {

int skw_render_photon(skw_scene *s, const skw_photon_map *pm, const skw_camera *cam, const skw_render_params *params,
                      const skw_photon_render_params *pp, float *film_rgb, void *stream) {
  if (!s || !pm || !cam || !params || !pp || !film_rgb) return fail(s ? s->ctx : nullptr, SKW_ERR_ARG, "null argument");
  skw_ctx *ctx = s->ctx;
  if (pp->gather_samples < 0 || pp->gather_samples > 1024) return fail(ctx, SKW_ERR_ARG, "gather_samples out of range");
  if (pp->caustic_lookup < 0 || pp->caustic_lookup > 4096) return fail(ctx, SKW_ERR_ARG, "caustic_lookup out of range");
  const bool caustic = pm->maps[0].n > 0 && pp->caustic_lookup > 0;
  if (caustic && !(pp->max_caustic_dist > 0.0))
    return fail(ctx, SKW_ERR_ARG, "max_caustic_dist must be positive");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaSetDevice");
  // the sampler rounds sequence lengths up to squares (Sampler.cpp:39-57, StratifiedSampler.cpp:33-37)
  int gs = 0;
  if (pp->gather_samples > 0 && params->sampler == SKW_SAMPLER_LD) {  // LDSampler: powers of two
    gs = 1;
    while (gs < pp->gather_samples) gs <<= 1;
  } else if (pp->gather_samples > 0) {
    const int r = (int)std::ceil(std::sqrt((double)pp->gather_samples));
    gs = r * r;
  }
  const bool gather = gs > 0 && pm->n_irr > 0;
  PassConfig cfg;
  cfg.samples_per_pass = (int64_t)1 << 19;
  cfg.extra_slots = (gather ? 2 * gs : 0) + (caustic ? 1 : 0);
  // PhotonLTEIntegrator has no medium march (_MediaRadianceAndTranmsittance
  // returns transmittance 1, PhotonLTEIntegrator.cpp:638-648); its direct
  // lighting still attenuates light samples through the medium.
  cfg.media = false;
  Plan P;
  const uint64_t seed = params->seed;
  int rc = plan_make(s, cam, 1, params, &seed, cfg, &P);
  if (rc != SKW_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  cudaMemPool_t pool;
  if ((e = skw::ctx_pool(ctx, &pool)) != cudaSuccess) return cuda_fail(ctx, e, "workspace pool");
  const size_t wbytes = workspace_bytes(P), vbytes = al256(sizeof(skw::ViewDev)),
               gbytes = gather ? skw::gather_bytes(P.cap_samples, gs) : 0,
               cbytes = caustic ? skw::caustic_bytes(P.cap_samples, pp->caustic_lookup) : 0;
  char *w = nullptr;
  if ((e = cudaMallocFromPoolAsync((void **)&w, wbytes + vbytes + gbytes + cbytes, pool, st)) != cudaSuccess)
    return cuda_fail(ctx, e, "photon render workspace");
  Workspace W;
  workspace_carve(P, w, &W);
  skw::ViewDev *d_view = (skw::ViewDev *)(w + wbytes);
  void *gws = w + wbytes + vbytes;
  void *cws = w + wbytes + vbytes + gbytes;
  const skw::PhotonMapData &cm = pm->maps[0];
  skw::CausticMap CM{cm.d_nodes, cm.d_nids, cm.d_dirid, cm.d_weight, (int32_t)cm.n, (double)cm.paths,
                     pp->caustic_lookup, pp->max_caustic_dist, pm->d_dirs};
  skw::GatherMaps M{};
  const skw::PhotonMapData &im = pm->maps[2];
  M.ind_nodes = im.d_nodes;
  M.ind_nids = im.d_nids;
  M.ind_dirid = im.d_dirid;
  M.n_ind = (int32_t)im.n;
  // max lookup distance of the 32 indirect photons (PhotonLTEIntegrator.cpp:450-453)
  M.ind_lookup_dist = im.n > 0 ? std::sqrt(pm->scene_area / (double)im.n * 32 * 0.31830988618379067154) : 0.0;
  M.irr_nodes = pm->d_irr_nodes;
  M.irr_nids = pm->d_irr_nids;
  M.irr_ext = pm->d_irr_ext;
  M.irr_int = pm->d_irr_int;
  M.n_irr = (int32_t)pm->n_irr;
  M.max_irr_dist = pm->max_irr_dist;
  M.dirs = pm->d_dirs;
  for (int k = 0; k < 3; ++k) {
    M.lo[k] = s->accel->info.bounds[k];
    M.hi[k] = s->accel->info.bounds[3 + k];
  }
  skw_accel *a = s->accel;
  skw::TraceFn trace = [a](const void *rays, int64_t n, const int *n_dev, void *hits, cudaStream_t stq, int *work) {
    return skw::launch_traversal(true, a->stack_cap, a->d_nodes, a->d_tris, rays, n, n_dev, a->scene_abs, nullptr,
                                 hits, a->d_status, stq, 0, work, true);
  };
  e = cudaMemcpyAsync(d_view, P.views.data(), sizeof(skw::ViewDev), cudaMemcpyHostToDevice, st);
  int64_t launches = 0;
  const int base_slot = 1 + 2 * P.nl + P.npl;
  // The specular levels' entries get the same caustic and gather terms,
  // weighted, in their sample's specular slot (PhotonLTEIntegrator::
  // _SurfaceRadiance at every depth, PhotonLTEIntegrator.cpp:320-385).  A
  // level's length is read back and its entries run in chunks of the pass's
  // sample count (the gather and caustic workspaces' capacity).
  int64_t px_cur = 0;
  int32_t *h_count = nullptr;
  if (e == cudaSuccess && P.spec_levels && (gather || caustic)) e = cudaMallocHost((void **)&h_count, sizeof(int32_t));
  SpecHook hook = [&](const SpecLevel &L) -> cudaError_t {
    cudaError_t he = cudaMemcpyAsync(h_count, L.count, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    if (he == cudaSuccess) he = cudaStreamSynchronize(st);
    if (he != cudaSuccess) return he;
    const int64_t cnt = std::min<int64_t>(*h_count, L.capacity);
    for (int64_t off = 0; off < cnt && he == cudaSuccess; off += P.cap_samples) {
      const int m = (int)std::min<int64_t>(P.cap_samples, cnt - off);
      skw::SpecSource sp;
      sp.in_sample = L.sample + off;
      sp.in_w = L.w + 3 * off;
      sp.in_node = L.node + off;
      sp.slot = P.spec_slot;
      const void *lr = (const char *)L.rays + 32 * off, *lh = (const char *)L.hits + 16 * off;
      if (gather)
        he = skw::launch_gather(s->dev, M, d_view, 1, m, px_cur, P.spp, P.slots, base_slot, gs, lr, lh, gws,
                                W.contrib, trace, pm->d_status, st, &sp);
      if (he == cudaSuccess && caustic)
        he = skw::launch_caustic(s->dev, CM, d_view, 1, m, px_cur, P.spp, P.slots, P.spec_slot, lr, lh, cws,
                                 W.contrib, pm->d_status, st, &sp);
      launches += (gather ? 6 : 0) + (caustic ? 3 : 0);
    }
    return he;
  };
  for (int64_t px0 = 0; px0 < P.n_px_total && e == cudaSuccess; px0 += P.chunk_px) {
    const int n_px = (int)std::min<int64_t>(P.chunk_px, P.n_px_total - px0);
    const int n = n_px * P.spp;
    px_cur = px0;
    if ((e = record_direct(s, P, W, d_view, px0, n_px, st, P.spec_levels && (gather || caustic) ? &hook : nullptr)) !=
        cudaSuccess)
      break;
    if (gather && (e = skw::launch_gather(s->dev, M, d_view, 1, n, px0, P.spp, P.slots, base_slot, gs, W.rays, W.hits,
                                          gws, W.contrib, trace, pm->d_status, st)) != cudaSuccess)
      break;
    // _LookupCausticRadiance (PhotonLTEIntegrator.cpp:342) into the slot after the gather slots
    if (caustic && (e = skw::launch_caustic(s->dev, CM, d_view, 1, n, px0, P.spp, P.slots,
                                            base_slot + (gather ? 2 * gs : 0), W.rays, W.hits, cws, W.contrib,
                                            pm->d_status, st)) != cudaSuccess)
      break;
    if ((e = skw::launch_film(W.contrib, px0, n_px, P.spp, P.slots, film_rgb, st)) != cudaSuccess) break;
    launches += launches_per_pass(P) + (gather ? 6 : 0) + (caustic ? 3 : 0);
  }
  cudaFreeAsync(w, st);
  if (h_count) {
    cudaStreamSynchronize(st);
    cudaFreeHost(h_count);
  }
  if (e != cudaSuccess) return cuda_fail(ctx, e, "photon-map render");
  ctx->launches.fetch_add(launches);
  return SKW_OK;
}

}  // extern "C"

extern "C" {

int skw_scene_hit_geometry(skw_scene *s, const skw_ray *rays, const skw_hit *hits, int64_t n,
                           skw_hit_geometry *out, void *stream) {
  if (!s) return SKW_ERR_ARG;
  if (n < 0 || n > (int64_t)INT32_MAX || (n > 0 && (!rays || !hits || !out)))
    return fail(s->ctx, SKW_ERR_ARG, "bad hit-geometry buffers");
  static_assert(sizeof(skw_hit_geometry) == 12 * sizeof(double), "skw_hit_geometry layout");
  cudaError_t e = cudaSetDevice(s->ctx->device);
  if (e == cudaSuccess) e = skw::launch_hit_geometry(s->dev, rays, hits, n, (double *)out, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(s->ctx, e, "hit geometry");
  s->ctx->launches.fetch_add(n > 0 ? 1 : 0);
  return SKW_OK;
}

int skw_scene_intersection(skw_scene *s, const skw_ray_differential *rays, const skw_hit_d *hits, int64_t n,
                           skw_intersection *out, void *stream) {
  if (!s) return SKW_ERR_ARG;
  if (n < 0 || n > (int64_t)INT32_MAX || (n > 0 && (!rays || !hits || !out)))
    return fail(s->ctx, SKW_ERR_ARG, "bad intersection buffers");
  static_assert(sizeof(skw_ray_differential) == 21 * sizeof(double), "skw_ray_differential layout");
  static_assert(sizeof(skw_intersection) == 36 * sizeof(double), "skw_intersection layout");
  static_assert(sizeof(skw_hit_d) == 16, "skw_hit_d layout");
  cudaError_t e = cudaSetDevice(s->ctx->device);
  if (e == cudaSuccess) e = skw::launch_intersection(s->dev, rays, hits, n, (double *)out, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(s->ctx, e, "intersection");
  s->ctx->launches.fetch_add(n > 0 ? 1 : 0);
  return SKW_OK;
}

double skw_next_min_t(const skw_intersection *isect, const double *direction) {
  if (!isect || !direction) return 0.0;
  const double div = direction[0] * isect->cross[0] + direction[1] * isect->cross[1] + direction[2] * isect->cross[2];
  if (div == 0.0) return 0.0;
  return std::max(0.0, isect->dot * (1.0 / div) + 1e-14);
}

int skw_scene_next_rays(skw_scene *s, const skw_ray *rays, const skw_hit *hits, const float *directions, int64_t n,
                        skw_ray *out, void *stream) {
  if (!s) return SKW_ERR_ARG;
  if (n < 0 || n > (int64_t)INT32_MAX || (n > 0 && (!rays || !hits || !directions || !out)))
    return fail(s->ctx, SKW_ERR_ARG, "bad outgoing-ray buffers");
  cudaError_t e = cudaSetDevice(s->ctx->device);
  if (e == cudaSuccess) e = skw::launch_next_rays(s->dev, rays, hits, directions, n, out, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(s->ctx, e, "outgoing rays");
  s->ctx->launches.fetch_add(n > 0 ? 1 : 0);
  return SKW_OK;
}

int skw_scene_set_max_specular_depth(skw_scene *s, int32_t depth) {
  if (!s) return SKW_ERR_ARG;
  if (depth < 0 || depth > kMaxSpecDepth)
    return fail(s->ctx, SKW_ERR_ARG, "max specular depth must be in [0, 11]");
  s->dev.max_spec_depth = depth;
  return SKW_OK;
}

int skw_scene_set_medium(skw_scene *s, const skw_medium *m) {
  if (!s) return SKW_ERR_ARG;
  skw::MediumDev &M = s->dev.medium;
  if (!m) {
    M = skw::MediumDev{};
    return SKW_OK;
  }
  bool ok = m->step > 0.0f && std::isfinite(m->step) && m->g > -1.0f && m->g < 1.0f;
  for (int k = 0; k < 3; ++k)
    ok = ok && m->lo[k] <= m->hi[k] && m->sigma_a[k] >= 0.0f && m->sigma_s[k] >= 0.0f && m->emission[k] >= 0.0f &&
         std::isfinite(m->sigma_a[k] + m->sigma_s[k] + m->emission[k] + m->lo[k] + m->hi[k]);
  if (!ok) return fail(s->ctx, SKW_ERR_ARG, "bad medium");
  M.on = 1;
  double diag2 = 0.0;
  for (int k = 0; k < 3; ++k) {
    M.lo[k] = m->lo[k];
    M.hi[k] = m->hi[k];
    M.sigma_s[k] = m->sigma_s[k];
    M.sigma_t[k] = m->sigma_a[k] + m->sigma_s[k];  // HomogeneousVolumeRegion.cpp:26
    M.emission[k] = m->emission[k];
    diag2 += (double)(m->hi[k] - m->lo[k]) * (m->hi[k] - m->lo[k]);
  }
  M.g = m->g;
  M.step = m->step;
  // Every step is at least `step` long (step = step / luminance(T) and
  // luminance(T) <= 1), so a ray crosses the box in at most diag / step + 1.
  const double steps = std::ceil(std::sqrt(diag2) / m->step) + 2.0;
  if (steps > (double)((int64_t)1 << 24)) return fail(s->ctx, SKW_ERR_ARG, "medium step too small for its box");
  M.max_steps = (int32_t)steps;
  return SKW_OK;
}

}  // extern "C"
