// C-ABI driver over the reference renderer's own classes, linked with the
// reference sources into oracle/_ref/libskw_ref.so by oracle/build_ref.py.
//
// Test infrastructure only: the parity tests and the CPU baseline call it to
// get the reference's answers (and its timings) on the same inputs that the
// CUDA path receives.  Nothing in the product links or loads it.
//
// Every entry point mirrors one reference call:
//   skw_ref_accel_*      TriangleAccelerator ctor / Intersect / IntersectTest
//                        (Raytracer/Core/TriangleAccelerator.cpp:22-147, 295-352, 464-468)
//   skw_ref_kdtree_*     KDTree<Photon> ctor + GetNearestPoints / GetNearestPoint
//                        with PhotonFilter (Raytracer/Core/KDTree.h:428-576,
//                        PhotonInternalTypes.h:113-137)
// Internal members are read through `#define private public`, which is why
// the standard headers are included first.
#include <algorithm>
#include <atomic>
#include <cstdint>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <queue>
#include <random>
#include <sstream>
#include <string>
#include <thread>
#include <vector>
#include <tbb/tbb.h>

#define private public
#define protected public
#include <Raytracer/Core/TriangleAccelerator.h>
#include <Raytracer/Core/TriangleMesh.h>
#include <Raytracer/Core/Primitive.h>
#include <Raytracer/Core/KDTree.h>
#include <Raytracer/LTEIntegrators/PhotonLTEIntegrator.h>
#include <Raytracer/LTEIntegrators/PhotonLTEIntegrator/PhotonInternalTypes.h>
#include <Math/CompressedDirection.h>
#include <Raytracer/Core/Scene.h>
#include <Raytracer/Core/LightSources.h>
#include <Raytracer/Core/Texture.h>
#include <Raytracer/Core/SpectrumRoutines.h>
#include <Raytracer/Textures/ConstantTexture.h>
#include <Raytracer/Materials/MatteMaterial.h>
#include <Raytracer/Materials/PlasticMaterial.h>
#include <Raytracer/Materials/MetalMaterial.h>
#include <Raytracer/LightSources/DiffuseAreaLightSource.h>
#include <Raytracer/LightSources/PointLight.h>
#include <Raytracer/Cameras/PerspectiveCamera.h>
#include <Raytracer/Films/ImageFilm.h>
#include <Raytracer/FilmFilters/BoxFilter.h>
#include <Raytracer/Samplers/StratifiedSampler.h>
#include <Raytracer/LTEIntegrators/DirectLightingLTEIntegrator.h>
#include <Raytracer/Renderers/SamplerBasedRenderer.h>
#undef private
#undef protected
#include <chrono>

namespace {

// Runs fn(begin, end) over [0, n) on `threads` workers (0 = all cores).
void parallel_ranges(int64_t n, int threads, const std::function<void(int64_t, int64_t)> &fn) {
  unsigned nt = threads > 0 ? (unsigned)threads : tbb::shim_num_workers();
  if (nt <= 1 || n < 1024) {
    fn(0, n);
    return;
  }
  std::atomic<int64_t> next(0);
  const int64_t chunk = 256;
  tbb::shim_run_workers(nt, [&](unsigned) {
    for (;;) {
      int64_t s = next.fetch_add(chunk);
      if (s >= n) break;
      fn(s, std::min(n, s + chunk));
    }
  });
}

struct RefAccel {
  std::vector<intrusive_ptr<const Primitive>> prims;
  std::unique_ptr<TriangleAccelerator> accel;
};

Transform make_transform(const double *m) {
  if (!m) return Transform();
  double v[4][4];
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) v[r][c] = m[r * 4 + c];
  return Transform(v);
}

}  // namespace

extern "C" {

int skw_ref_version(void) { return 1; }

// Builds one primitive per entry; entries sharing a mesh id share one
// TriangleMesh object (instancing).  verts: float xyz per vertex; tris: int32
// triples.  xforms: optional row-major 4x4 mesh-to-world per primitive.
void *skw_ref_accel_create(int n_prims, const int32_t *mesh_of_prim, int n_meshes, const float *const *verts,
                           const int64_t *n_verts, const int32_t *const *tris, const int64_t *n_tris,
                           const double *xforms) {
  auto *ra = new RefAccel();
  std::vector<intrusive_ptr<const TriangleMesh>> meshes;
  for (int m = 0; m < n_meshes; ++m) {
    std::vector<Point3D_f> v((size_t)n_verts[m]);
    for (int64_t i = 0; i < n_verts[m]; ++i)
      v[(size_t)i] = Point3D_f(verts[m][3 * i], verts[m][3 * i + 1], verts[m][3 * i + 2]);
    std::vector<MeshTriangle> t((size_t)n_tris[m]);
    for (int64_t i = 0; i < n_tris[m]; ++i)
      t[(size_t)i] = MeshTriangle(tris[m][3 * i], tris[m][3 * i + 1], tris[m][3 * i + 2]);
    meshes.push_back(intrusive_ptr<const TriangleMesh>(new TriangleMesh(v, t, false, false)));
  }
  for (int p = 0; p < n_prims; ++p) {
    Transform tr = make_transform(xforms ? xforms + 16 * p : nullptr);
    ra->prims.push_back(intrusive_ptr<const Primitive>(
        new Primitive(meshes[(size_t)mesh_of_prim[p]], tr, intrusive_ptr<const Material>(), NULL, NULL)));
  }
  ra->accel.reset(new TriangleAccelerator(ra->prims));
  return ra;
}

void skw_ref_accel_destroy(void *a) { delete (RefAccel *)a; }

// rays: 8 floats per ray (ox oy oz dx dy dz tmin tmax), widened exactly to
// double.  Outputs the reference's (primitive index, mesh triangle index, t);
// -1 and +inf on a miss.  Runs TriangleAccelerator::Intersect, which also
// computes the differential geometry of the hit, as the renderer does.
void skw_ref_intersect(void *a, const float *rays, int64_t n, int32_t *prim, int32_t *tri, double *t,
                       int threads) {
  const RefAccel *ra = (const RefAccel *)a;
  parallel_ranges(n, threads, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      const float *r = rays + 8 * i;
      Ray ray(Point3D_d(r[0], r[1], r[2]), Vector3D_d(r[3], r[4], r[5]), r[6], r[7]);
      RayDifferential rd(ray);
      Intersection isect;
      double th;
      if (ra->accel->Intersect(rd, isect, &th)) {
        size_t pi = 0;
        for (; pi < ra->prims.size(); ++pi)
          if (ra->prims[pi].get() == isect.mp_primitive) break;
        prim[i] = (int32_t)pi;
        tri[i] = (int32_t)isect.m_triangle_index;
        t[i] = th;
      } else {
        prim[i] = -1;
        tri[i] = -1;
        t[i] = std::numeric_limits<double>::infinity();
      }
    }
  });
}

void skw_ref_intersect_test(void *a, const float *rays, int64_t n, uint8_t *occluded, int threads) {
  const RefAccel *ra = (const RefAccel *)a;
  parallel_ranges(n, threads, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      const float *r = rays + 8 * i;
      Ray ray(Point3D_d(r[0], r[1], r[2]), Vector3D_d(r[3], r[4], r[5]), r[6], r[7]);
      occluded[i] = ra->accel->IntersectTest(ray) ? 1 : 0;
    }
  });
}

// Tree export, pre-order with children visited left, middle, right.
// node_bbox: 6 floats (min xyz, max xyz).  node_info: 8 int32 per node:
// flags (reference Node::m_flags & 3), child L/M/R pre-order indices (-1 if
// absent), triangles [begin, end), instances [begin, end).
// tri_prim / tri_idx: m_primitive_indices / m_triangle_indices in the
// accelerator's final triangle order (-1 for a shared-mesh triangle).
int64_t skw_ref_accel_num_nodes(void *a) {
  const RefAccel *ra = (const RefAccel *)a;
  int64_t count = 0;
  std::vector<const TriangleAccelerator::Node *> st{ra->accel->mp_root};
  while (!st.empty()) {
    const TriangleAccelerator::Node *nd = st.back();
    st.pop_back();
    ++count;
    if (!nd->IsLeaf())
      for (int c = 2; c >= 0; --c)
        if (nd->m_children[c]) st.push_back(nd->m_children[c]);
  }
  return count;
}

int64_t skw_ref_accel_num_triangles(void *a) { return (int64_t)((const RefAccel *)a)->accel->m_triangles.size(); }

void skw_ref_accel_export(void *a, float *node_bbox, int32_t *node_info, int32_t *tri_prim, int32_t *tri_idx,
                          float *tris_out) {
  const RefAccel *ra = (const RefAccel *)a;
  const TriangleAccelerator &acc = *ra->accel;
  std::vector<const TriangleAccelerator::Node *> order;
  std::map<const TriangleAccelerator::Node *, int32_t> index;
  std::vector<const TriangleAccelerator::Node *> st{acc.mp_root};
  while (!st.empty()) {
    const TriangleAccelerator::Node *nd = st.back();
    st.pop_back();
    index[nd] = (int32_t)order.size();
    order.push_back(nd);
    if (!nd->IsLeaf())
      for (int c = 2; c >= 0; --c)
        if (nd->m_children[c]) st.push_back(nd->m_children[c]);
  }
  for (size_t i = 0; i < order.size(); ++i) {
    const TriangleAccelerator::Node *nd = order[i];
    for (int k = 0; k < 3; ++k) {
      node_bbox[6 * i + k] = nd->m_bbox.m_min[k];
      node_bbox[6 * i + 3 + k] = nd->m_bbox.m_max[k];
    }
    int32_t *info = node_info + 8 * i;
    info[0] = nd->m_flags & 3;
    for (int c = 0; c < 3; ++c)
      info[1 + c] = (!nd->IsLeaf() && nd->m_children[c]) ? index[nd->m_children[c]] : -1;
    info[4] = (int32_t)nd->m_triangles_begin;
    info[5] = (int32_t)nd->m_triangles_end;
    info[6] = (int32_t)nd->m_instances_begin;
    info[7] = (int32_t)nd->m_instances_end;
  }
  for (size_t i = 0; i < acc.m_triangles.size(); ++i) {
    tri_prim[i] = acc.m_primitive_indices[i] == std::numeric_limits<size_t>::max() ? -1 : (int32_t)acc.m_primitive_indices[i];
    tri_idx[i] = (int32_t)acc.m_triangle_indices[i];
    if (tris_out)
      for (int v = 0; v < 3; ++v)
        for (int k = 0; k < 3; ++k) tris_out[9 * i + 3 * v + k] = acc.m_triangles[i][v][k];
  }
}

// ---------------------------------------------------------------- photons --

typedef PhotonLTEIntegrator::Photon RefPhoton;
typedef KDTree<RefPhoton> RefPhotonTree;

struct RefKD {
  std::unique_ptr<RefPhotonTree> tree;
};

// Builds KDTree<Photon> over photons with the given float positions and
// packed 16-bit normals / incident directions.  perm_out[i] = input index of
// the photon at tree position i; node_words: 2 uint32 per node (split
// coordinate bits, right-child/flags word) exactly as the reference stores them.
void *skw_ref_kdtree_create(const float *pos, const uint16_t *normal_ids, const uint16_t *dir_ids, int64_t n,
                            int32_t *perm_out, uint32_t *node_words) {
  std::vector<RefPhoton> pts((size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    RefPhoton p;
    p.m_point = Point3D_f(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    float tag;
    uint32_t u = (uint32_t)i;
    std::memcpy(&tag, &u, 4);
    p.m_weight = Spectrum_f(tag, 0.f, 0.f);
    p.m_normal = CompressedDirection::FromID(normal_ids ? normal_ids[i] : 0);
    p.m_incident_direction = CompressedDirection::FromID(dir_ids ? dir_ids[i] : 0);
    pts[(size_t)i] = p;
  }
  auto *kd = new RefKD();
  kd->tree.reset(new RefPhotonTree(std::move(pts)));
  const auto &P = kd->tree->m_points;
  const auto &N = kd->tree->m_nodes;
  for (size_t i = 0; i < P.size(); ++i) {
    float tag = P[i].m_weight[0];
    uint32_t u;
    std::memcpy(&u, &tag, 4);
    if (perm_out) perm_out[i] = (int32_t)u;
    if (node_words) {
      std::memcpy(&node_words[2 * i], &N[i].m_split_coordinate, 4);
      node_words[2 * i + 1] = N[i].m_right_child;
    }
  }
  return kd;
}

void skw_ref_kdtree_destroy(void *kd) { delete (RefKD *)kd; }

// Filtered k-NN (GetNearestPoints with PhotonFilter when cos_threshold >= 0,
// the unfiltered overload otherwise).  Indices are tree positions.  Each
// query's k slots hold the reference's heap order; unused slots are -1.
void skw_ref_knn(void *kdp, const double *q, const double *qn, int64_t nq, int32_t k, double max_dist,
                 double cos_threshold, int32_t *out_idx, double *out_d2, int32_t *out_count, int threads) {
  const RefKD *kd = (const RefKD *)kdp;
  const RefPhoton *base = kd->tree->m_points.empty() ? nullptr : &kd->tree->m_points[0];
  parallel_ranges(nq, threads, [&](int64_t b, int64_t e) {
    std::vector<RefPhotonTree::NearestPoint> buf((size_t)std::max(k, 1));
    for (int64_t i = b; i < e; ++i) {
      Point3D_d p(q[3 * i], q[3 * i + 1], q[3 * i + 2]);
      size_t found;
      if (cos_threshold >= 0) {
        Vector3D_d nrm(qn[3 * i], qn[3 * i + 1], qn[3 * i + 2]);
        PhotonLTEIntegrator::PhotonFilter filter(p, nrm, cos_threshold);
        found = kd->tree->GetNearestPoints(p, (size_t)k, &buf[0], filter, max_dist);
      } else {
        found = kd->tree->GetNearestPoints(p, (size_t)k, &buf[0], max_dist);
      }
      out_count[i] = (int32_t)found;
      for (int32_t j = 0; j < k; ++j) {
        if ((size_t)j < found) {
          out_idx[i * k + j] = (int32_t)(buf[(size_t)j].mp_point - base);
          out_d2[i * k + j] = buf[(size_t)j].m_distance_sqr;
        } else {
          out_idx[i * k + j] = -1;
          out_d2[i * k + j] = 0.0;
        }
      }
    }
  });
}

// GetNearestPoint (unfiltered): tree position of the nearest photon, or -1.
void skw_ref_nearest(void *kdp, const double *q, int64_t nq, double max_dist, int32_t *out_idx, int threads) {
  const RefKD *kd = (const RefKD *)kdp;
  const RefPhoton *base = kd->tree->m_points.empty() ? nullptr : &kd->tree->m_points[0];
  parallel_ranges(nq, threads, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      const RefPhoton *r = kd->tree->GetNearestPoint(Point3D_d(q[3 * i], q[3 * i + 1], q[3 * i + 2]), max_dist);
      out_idx[i] = r ? (int32_t)(r - base) : -1;
    }
  });
}

// CompressedDirection table entry i as doubles (for codec parity).
void skw_ref_compressed_direction_table(double *out) {
  for (int i = 0; i < (1 << 16); ++i) {
    Vector3D_d v = CompressedDirection::FromID((unsigned short)i).ToVector3D<double>();
    out[3 * i] = v[0];
    out[3 * i + 1] = v[1];
    out[3 * i + 2] = v[2];
  }
}

uint16_t skw_ref_compress_direction(double x, double y, double z) {
  return CompressedDirection(Vector3D_d(x, y, z)).GetID();
}

// ------------------------------------------------------------- rendering --

// Per-triangle constant reflectance, looked up by the hit's triangle index.
class TriangleAlbedoTexture : public Texture<SpectrumCoef_d> {
 public:
  explicit TriangleAlbedoTexture(std::vector<SpectrumCoef_d> v) : m_v(std::move(v)) {}
  SpectrumCoef_d Evaluate(const DifferentialGeometry &, size_t i_triangle_index) const override {
    return m_v[i_triangle_index];
  }

 private:
  std::vector<SpectrumCoef_d> m_v;
};

// Same layouts as the product's skw_material / skw_render_primitive.
struct RefMaterialIn {
  int32_t kind;
  float kd[3], ks[3];
  float roughness, sigma;
  float eta[3], k[3];
};
struct RefPrimIn {
  int32_t mesh;
  const double *mesh_to_world;
  int32_t material;
  const float *vertex_normals;
  const float *triangle_albedo;
  float emission[3];
};

// Renders the direct-lighting image with the reference's SamplerBasedRenderer,
// StratifiedSampler, DirectLightingLTEIntegrator, PerspectiveCamera and an
// ImageFilm with a 0.5-wide BoxFilter.  film_out: height x width x 3.
int skw_ref_render_direct(int n_meshes, const float *const *verts, const int64_t *n_verts, const int32_t *const *tris,
                          const int64_t *n_tris, int n_prims, const RefPrimIn *prims, int n_materials,
                          const RefMaterialIn *materials, int n_point_lights, const float *point_lights,
                          const double *camera_to_world, double x_view_angle, int width, int height, int spp_x,
                          int spp_y, int light_samples, float *film_out, double *seconds_out) {
  std::vector<intrusive_ptr<const Primitive>> prim_list;
  LightSources lights;
  for (int p = 0; p < n_prims; ++p) {
    const RefPrimIn &P = prims[p];
    const int m = P.mesh;
    std::vector<Point3D_f> v((size_t)n_verts[m]);
    for (int64_t i = 0; i < n_verts[m]; ++i)
      v[(size_t)i] = Point3D_f(verts[m][3 * i], verts[m][3 * i + 1], verts[m][3 * i + 2]);
    std::vector<MeshTriangle> t((size_t)n_tris[m]);
    for (int64_t i = 0; i < n_tris[m]; ++i) t[(size_t)i] = MeshTriangle(tris[m][3 * i], tris[m][3 * i + 1], tris[m][3 * i + 2]);
    intrusive_ptr<TriangleMesh> mesh;
    if (P.vertex_normals) {
      std::vector<Vector3D_f> nrm((size_t)n_verts[m]);
      for (int64_t i = 0; i < n_verts[m]; ++i)
        nrm[(size_t)i] = Vector3D_f(P.vertex_normals[3 * i], P.vertex_normals[3 * i + 1], P.vertex_normals[3 * i + 2]);
      mesh.reset(new TriangleMesh(v, t, nrm, std::vector<Vector3D_f>(), true, false));
    } else {
      mesh.reset(new TriangleMesh(v, t, false, false));
    }
    const RefMaterialIn &M = materials[P.material];
    intrusive_ptr<const Texture<SpectrumCoef_d>> kd;
    if (P.triangle_albedo) {
      std::vector<SpectrumCoef_d> a((size_t)n_tris[m]);
      for (int64_t i = 0; i < n_tris[m]; ++i)
        a[(size_t)i] = SpectrumCoef_d(P.triangle_albedo[3 * i], P.triangle_albedo[3 * i + 1], P.triangle_albedo[3 * i + 2]);
      kd.reset(new TriangleAlbedoTexture(a));
    } else {
      kd.reset(new ConstantTexture<SpectrumCoef_d>(SpectrumCoef_d(M.kd[0], M.kd[1], M.kd[2])));
    }
    intrusive_ptr<const Material> mat;
    if (M.kind == 0) {
      mat.reset(new MatteMaterial(kd, intrusive_ptr<const Texture<double>>(new ConstantTexture<double>(M.sigma))));
    } else if (M.kind == 1) {
      mat.reset(new PlasticMaterial(kd, intrusive_ptr<const Texture<SpectrumCoef_d>>(new ConstantTexture<SpectrumCoef_d>(
                                            SpectrumCoef_d(M.ks[0], M.ks[1], M.ks[2]))),
                                    intrusive_ptr<const Texture<double>>(new ConstantTexture<double>(M.roughness))));
    } else {
      mat.reset(new MetalMaterial(
          intrusive_ptr<const Texture<SpectrumCoef_d>>(new ConstantTexture<SpectrumCoef_d>(SpectrumCoef_d(M.eta[0], M.eta[1], M.eta[2]))),
          intrusive_ptr<const Texture<SpectrumCoef_d>>(new ConstantTexture<SpectrumCoef_d>(SpectrumCoef_d(M.k[0], M.k[1], M.k[2]))),
          intrusive_ptr<const Texture<double>>(new ConstantTexture<double>(M.roughness))));
    }
    intrusive_ptr<const AreaLightSource> light;
    if (P.emission[0] > 0 || P.emission[1] > 0 || P.emission[2] > 0) {
      light.reset(new DiffuseAreaLightSource(Spectrum_d(P.emission[0], P.emission[1], P.emission[2]), mesh));
      lights.m_area_light_sources.push_back(light);
    }
    prim_list.push_back(intrusive_ptr<const Primitive>(
        new Primitive(mesh, make_transform(P.mesh_to_world), mat, light, NULL)));
  }
  for (int i = 0; i < n_point_lights; ++i) {
    const float *L = point_lights + 6 * i;
    lights.m_delta_light_sources.push_back(intrusive_ptr<const DeltaLightSource>(
        new PointLight(Point3D_d(L[0], L[1], L[2]), Spectrum_d(L[3], L[4], L[5]))));
  }
  intrusive_ptr<const Scene> scene(new Scene(prim_list, NULL, lights));
  intrusive_ptr<FilmFilter> filter(new BoxFilter(0.5, 0.5));
  intrusive_ptr<ImageFilm> film(new ImageFilm((size_t)width, (size_t)height, filter));
  intrusive_ptr<const Camera> camera(new PerspectiveCamera(make_transform(camera_to_world), film, 0.0, 1.0, x_view_angle));
  Point2D_i begin, end;
  film->GetSamplingExtent(begin, end);
  intrusive_ptr<Sampler> sampler(new StratifiedSampler(begin, end, (size_t)spp_x, (size_t)spp_y));
  DirectLightingLTEIntegratorParams params;
  params.m_direct_light_samples_num = (size_t)light_samples;
  params.m_max_specular_depth = 6;
  params.m_media_step_size = 0.01;
  intrusive_ptr<LTEIntegrator> integrator(new DirectLightingLTEIntegrator(scene, params));
  SamplerBasedRenderer renderer(integrator, sampler);
  auto t0 = std::chrono::steady_clock::now();
  renderer.Render(camera, false);
  if (seconds_out) *seconds_out = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  for (int y = 0; y < height; ++y)
    for (int x = 0; x < width; ++x) {
      Spectrum_d c;
      float *o = film_out + 3 * ((int64_t)y * width + x);
      if (film->GetPixel(Point2D_i(x, y), c, true)) {
        o[0] = (float)c[0];
        o[1] = (float)c[1];
        o[2] = (float)c[2];
      } else {
        o[0] = o[1] = o[2] = 0.0f;
      }
    }
  return 0;
}

// Row Y of the reference's spectrum-to-XYZ matrix (its luminance weights).
void skw_ref_luminance_weights(double *out) {
  for (int k = 0; k < 3; ++k) {
    double rgb[3] = {0, 0, 0};
    rgb[k] = 1.0;
    out[k] = SpectrumRoutines::Luminance(Spectrum_d(rgb[0], rgb[1], rgb[2]));
  }
}

}  // extern "C"
