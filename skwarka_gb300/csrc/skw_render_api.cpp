// C ABI (include/skw.h): render scenes and the direct-lighting render.
#include "../../include/skw.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "kernels.h"
#include "render_scene.h"
#include "skw_internal.h"

using skw::cuda_fail;
using skw::fail;

struct skw_scene {
  skw_ctx *ctx = nullptr;
  skw_accel *accel = nullptr;
  std::vector<void *> buffers;  // device allocations owned by the scene
  skw::SceneDev dev{};
};

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
  std::vector<float> vpos, vnrm, albedo;
  std::vector<int32_t> tri_vidx, prim_tri_offset((size_t)std::max(n_prims, 1)), prim_material((size_t)std::max(n_prims, 1)),
      prim_light((size_t)std::max(n_prims, 1), -1), prim_has_normals((size_t)std::max(n_prims, 1), 0);
  bool any_albedo = false, any_normals = false;
  for (int32_t p = 0; p < n_prims; ++p) any_albedo |= prims[p].triangle_albedo != nullptr;
  for (int32_t p = 0; p < n_prims; ++p) any_normals |= prims[p].vertex_normals != nullptr;
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
    double inv[9];
    const bool has_inv = prims[p].mesh_to_world && inverse3(prims[p].mesh_to_world, inv);
    for (int64_t v = 0; v < m.n_vertices; ++v) {
      float w[3];
      xform_point(prims[p].mesh_to_world, m.vertices + 3 * v, w);
      vpos.insert(vpos.end(), w, w + 3);
      if (any_normals) {
        float nn[3] = {0, 0, 1};
        if (prims[p].vertex_normals) xform_normal(has_inv ? inv : nullptr, prims[p].vertex_normals + 3 * v, nn);
        vnrm.insert(vnrm.end(), nn, nn + 3);
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
    for (int64_t t = 0; t < m.n_triangles; ++t) {
      const int32_t *ix = m.triangles + 3 * t;
      bool bad = false;
      for (int k = 0; k < 3; ++k)
        if (ix[k] < 0 || (int64_t)ix[k] >= m.n_vertices) bad = true;
      if (bad || ix[0] == ix[1] || ix[0] == ix[2] || ix[1] == ix[2]) continue;  // TriangleMesh.cpp:176-182
      for (int k = 0; k < 3; ++k) tri_vidx.push_back(voff + ix[k]);
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
    }
    if (light) {
      L.tri_count = (int32_t)areas.size();
      L.area = (float)area_sum;
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
    } else if (m.kind == SKW_MATERIAL_METAL) {
      d.kind = skw::kMetal;
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
  cudaError_t e = cudaSetDevice(ctx->device);
  skw::SceneDev &D = s->dev;
  if (e == cudaSuccess) e = upload(s, vpos, &D.vpos);
  if (e == cudaSuccess) e = upload(s, vnrm, &D.vnrm);
  if (e == cudaSuccess) e = upload(s, tri_vidx, &D.tri_vidx);
  if (e == cudaSuccess) e = upload(s, albedo, &D.tri_albedo);
  if (e == cudaSuccess) e = upload(s, prim_tri_offset, &D.prim_tri_offset);
  if (e == cudaSuccess) e = upload(s, prim_material, &D.prim_material);
  if (e == cudaSuccess) e = upload(s, prim_light, &D.prim_light);
  if (e == cudaSuccess) e = upload(s, prim_has_normals, &D.prim_has_normals);
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

int skw_render_direct(skw_scene *s, const skw_camera *cam, const skw_render_params *params, float *film_rgb,
                      void *stream) {
  if (!s || !cam || !params || !film_rgb) return fail(s ? s->ctx : nullptr, SKW_ERR_ARG, "null argument");
  skw_ctx *ctx = s->ctx;
  if (cam->width <= 0 || cam->height <= 0 || params->spp_x <= 0 || params->spp_y <= 0 || params->light_samples < 0 ||
      params->light_samples > 64 || !(cam->x_view_angle > 0.0) || !(cam->x_view_angle < 3.14159265358979))
    return fail(ctx, SKW_ERR_ARG, "bad camera or render parameters");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaSetDevice");
  skw::CameraDev cd{};
  std::memcpy(cd.c2w, cam->camera_to_world, sizeof(cd.c2w));
  cd.x_tan = std::tan(cam->x_view_angle / 2.0);  // PerspectiveCamera.cpp:19-33
  cd.y_tan = cd.x_tan * (double)cam->height / cam->width;
  cd.width = cam->width;
  cd.height = cam->height;
  const int spp = params->spp_x * params->spp_y;
  const int nl = params->light_samples;
  const int npl = s->dev.n_point_lights;
  const int slots = 1 + 2 * nl + npl;
  const int64_t n_px_total = (int64_t)cam->width * cam->height;
  // Pixels per chunk: at most 2^21 samples in flight.
  const int64_t chunk_px = std::max<int64_t>(1, std::min<int64_t>(n_px_total, ((int64_t)1 << 21) / spp));
  const int64_t cap_samples = chunk_px * spp;
  const int64_t cap_shadow = cap_samples * (nl + npl), cap_bsdf = cap_samples * nl;
  if (cap_shadow > INT32_MAX || cap_samples * slots * 3 > ((int64_t)1 << 40))
    return fail(ctx, SKW_ERR_ARG, "render too large");
  auto al = [](int64_t x) { return (size_t)((x + 255) & ~(int64_t)255); };
  const size_t b_rays = al(cap_samples * 32), b_hits = al(cap_samples * 16), b_contrib = al(cap_samples * slots * 12),
               b_srays = al(std::max<int64_t>(cap_shadow, 1) * 32), b_starget = al(std::max<int64_t>(cap_shadow, 1) * 4),
               b_srgb = al(std::max<int64_t>(cap_shadow, 1) * 12), b_occ = al(std::max<int64_t>(cap_shadow, 1)),
               b_brays = al(std::max<int64_t>(cap_bsdf, 1) * 32), b_btarget = al(std::max<int64_t>(cap_bsdf, 1) * 4),
               b_brgb = al(std::max<int64_t>(cap_bsdf, 1) * 16), b_bhits = al(std::max<int64_t>(cap_bsdf, 1) * 16),
               b_cnt = 256;
  const size_t total = b_rays + b_hits + b_contrib + b_srays + b_starget + b_srgb + b_occ + b_brays + b_btarget +
                       b_brgb + b_bhits + b_cnt;
  cudaStream_t st = (cudaStream_t)stream;
  cudaMemPool_t pool;
  if ((e = skw::ctx_pool(ctx, &pool)) != cudaSuccess) return cuda_fail(ctx, e, "workspace pool");
  char *w = nullptr;
  if ((e = cudaMallocFromPoolAsync((void **)&w, total, pool, st)) != cudaSuccess)
    return cuda_fail(ctx, e, "render workspace");
  char *p = w;
  auto take = [&](size_t b) {
    char *r = p;
    p += b;
    return r;
  };
  void *rays = take(b_rays), *hits = take(b_hits);
  float *contrib = (float *)take(b_contrib);
  void *srays = take(b_srays);
  int *starget = (int *)take(b_starget);
  float *srgb = (float *)take(b_srgb);
  uint8_t *occ = (uint8_t *)take(b_occ);
  void *brays = take(b_brays);
  int *btarget = (int *)take(b_btarget);
  float *brgb = (float *)take(b_brgb);
  void *bhits = take(b_bhits);
  int *counts = (int *)take(b_cnt);  // [0] shadow queue length, [1] BSDF queue length
  skw_accel *a = s->accel;
  int64_t launches = 0;
  for (int64_t px0 = 0; px0 < n_px_total && e == cudaSuccess; px0 += chunk_px) {
    const int n_px = (int)std::min<int64_t>(chunk_px, n_px_total - px0);
    const int n = n_px * spp;
    if ((e = cudaMemsetAsync(contrib, 0, (size_t)n * slots * 12, st)) != cudaSuccess) break;
    if ((e = cudaMemsetAsync(counts, 0, 2 * sizeof(int), st)) != cudaSuccess) break;
    if ((e = skw::launch_camera(cd, (int)px0, n_px, params->spp_x, params->spp_y, params->seed, rays, st)) != cudaSuccess)
      break;
    if ((e = skw::launch_traversal(true, a->stack_cap, a->d_nodes, a->d_tris, rays, n, nullptr, a->scene_abs, nullptr,
                                   hits, a->d_status, st)) != cudaSuccess)
      break;
    if ((e = skw::launch_shade(s->dev, n, px0 * spp, slots, nl, params->seed, rays, hits, contrib, srays, starget, srgb,
                               counts, brays, btarget, brgb, counts + 1, st)) != cudaSuccess)
      break;
    const int64_t csh = (int64_t)n * (nl + npl), cbs = (int64_t)n * nl;
    if (csh > 0 && (e = skw::launch_traversal(false, a->stack_cap, a->d_nodes, a->d_tris, srays, csh, counts,
                                              a->scene_abs, nullptr, occ, a->d_status, st)) != cudaSuccess)
      break;
    if (cbs > 0 && (e = skw::launch_traversal(true, a->stack_cap, a->d_nodes, a->d_tris, brays, cbs, counts + 1,
                                              a->scene_abs, nullptr, bhits, a->d_status, st)) != cudaSuccess)
      break;
    if ((e = skw::launch_resolve(s->dev, (int)std::max(csh, cbs), nl, occ, starget, srgb, counts, brays, bhits,
                                 btarget, brgb, counts + 1, contrib, st)) != cudaSuccess)
      break;
    if ((e = skw::launch_film(contrib, (int)px0, n_px, spp, slots, film_rgb, st)) != cudaSuccess) break;
    launches += 8;
  }
  cudaFreeAsync(w, st);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "direct-lighting render");
  ctx->launches.fetch_add(launches);
  return SKW_OK;
}

}  // extern "C"
