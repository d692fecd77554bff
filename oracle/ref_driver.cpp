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
#include <Raytracer/Materials/TransparentMaterial.h>
#include <Raytracer/Materials/SubstrateMaterial.h>
#include <Raytracer/Materials/UberMaterial.h>
#include <Raytracer/Materials/MixMaterial.h>
#include <Raytracer/LightSources/DiffuseAreaLightSource.h>
#include <Raytracer/LightSources/PointLight.h>
#include <Raytracer/Cameras/PerspectiveCamera.h>
#include <Raytracer/Films/ImageFilm.h>
#include <Raytracer/FilmFilters/BoxFilter.h>
#include <Raytracer/Samplers/StratifiedSampler.h>
#include <Raytracer/Samplers/LDSampler.h>
#include <Raytracer/LTEIntegrators/DirectLightingLTEIntegrator.h>
#include <Raytracer/Renderers/SamplerBasedRenderer.h>
#include <Raytracer/VolumeRegions/HomogeneousVolumeRegion.h>
#include <Raytracer/PhaseFunctions/HGPhaseFunction.h>
#include <Raytracer/BxDFs/MERLMeasured.h>
#include <Raytracer/Materials/MERLMeasuredMaterial.h>
#include <Raytracer/Core/Color.h>
#include <Raytracer/Core/CoreUtils.h>
#undef private
#undef protected
#include <chrono>
#include <sstream>

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

// skw_ref_accel_create with optional per-mesh shading normals (float xyz per
// vertex; null = none): a mesh with normals uses them for shading
// (TriangleMesh(vertices, triangles, normals, tangents, true, false)), one
// without has use_shading_normals = false, as the render scenes build them.
void *skw_ref_accel_create_normals(int n_prims, const int32_t *mesh_of_prim, int n_meshes, const float *const *verts,
                                   const int64_t *n_verts, const int32_t *const *tris, const int64_t *n_tris,
                                   const float *const *normals, const double *xforms) {
  auto *ra = new RefAccel();
  std::vector<intrusive_ptr<const TriangleMesh>> meshes;
  for (int m = 0; m < n_meshes; ++m) {
    std::vector<Point3D_f> v((size_t)n_verts[m]);
    for (int64_t i = 0; i < n_verts[m]; ++i)
      v[(size_t)i] = Point3D_f(verts[m][3 * i], verts[m][3 * i + 1], verts[m][3 * i + 2]);
    std::vector<MeshTriangle> t((size_t)n_tris[m]);
    for (int64_t i = 0; i < n_tris[m]; ++i)
      t[(size_t)i] = MeshTriangle(tris[m][3 * i], tris[m][3 * i + 1], tris[m][3 * i + 2]);
    if (normals && normals[m]) {
      std::vector<Vector3D_f> nv((size_t)n_verts[m]);
      for (int64_t i = 0; i < n_verts[m]; ++i)
        nv[(size_t)i] = Vector3D_f(normals[m][3 * i], normals[m][3 * i + 1], normals[m][3 * i + 2]);
      meshes.push_back(intrusive_ptr<const TriangleMesh>(
          new TriangleMesh(v, t, nv, std::vector<Vector3D_f>(), true, false)));
    } else {
      meshes.push_back(intrusive_ptr<const TriangleMesh>(new TriangleMesh(v, t, false, false)));
    }
  }
  for (int p = 0; p < n_prims; ++p) {
    Transform tr = make_transform(xforms ? xforms + 16 * p : nullptr);
    ra->prims.push_back(intrusive_ptr<const Primitive>(
        new Primitive(meshes[(size_t)mesh_of_prim[p]], tr, intrusive_ptr<const Material>(), NULL, NULL)));
  }
  ra->accel.reset(new TriangleAccelerator(ra->prims));
  return ra;
}

// Double rays (8 doubles: ox oy oz dx dy dz tmin tmax) through
// TriangleAccelerator::Intersect: (primitive, mesh triangle, t); -1, -1,
// +inf on a miss.
void skw_ref_intersect_d(void *a, const double *rays, int64_t n, int32_t *prim, int32_t *tri, double *t,
                         int threads) {
  const RefAccel *ra = (const RefAccel *)a;
  parallel_ranges(n, threads, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      const double *r = rays + 8 * i;
      Ray ray(Point3D_d(r[0], r[1], r[2]), Vector3D_d(r[3], r[4], r[5]), r[6], r[7]);
      Intersection isect;
      double th;
      if (ra->accel->Intersect(RayDifferential(ray), isect, &th)) {
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

void skw_ref_intersect_test_d(void *a, const double *rays, int64_t n, uint8_t *occluded, int threads) {
  const RefAccel *ra = (const RefAccel *)a;
  parallel_ranges(n, threads, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      const double *r = rays + 8 * i;
      occluded[i] = ra->accel->IntersectTest(Ray(Point3D_d(r[0], r[1], r[2]), Vector3D_d(r[3], r[4], r[5]), r[6], r[7]))
                        ? 1
                        : 0;
    }
  });
}

// The whole Intersection of TriangleAccelerator::Intersect for ray
// differentials: rays 8 doubles as above; diffs (may be null = no
// differentials) 12 doubles per ray: origin_dx, direction_dx, origin_dy,
// direction_dy.  out: 40 doubles per ray -- point, geometric normal, shading
// normal (3 each), uv (2), point_dx, point_dy, normal_dx, normal_dy (3 each),
// duv_dx, duv_dy (2 each), tangent (3), m_cross (3), m_dot, t, primitive,
// mesh triangle (as doubles), 3 unused; NaN and primitive -1 on a miss.
// Also GetNextMinT (CoreUtils.h:139-149) of each hit for the direction
// next_dirs[3 i ...] (may be null) into next_tmin[i].
void skw_ref_intersection(void *a, const double *rays, const double *diffs, int64_t n, double *out,
                          const double *next_dirs, double *next_tmin, int threads) {
  const RefAccel *ra = (const RefAccel *)a;
  parallel_ranges(n, threads, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      const double *r = rays + 8 * i;
      RayDifferential rd(Ray(Point3D_d(r[0], r[1], r[2]), Vector3D_d(r[3], r[4], r[5]), r[6], r[7]));
      if (diffs) {
        const double *d = diffs + 12 * i;
        rd.m_has_differentials = true;
        rd.m_origin_dx = Point3D_d(d[0], d[1], d[2]);
        rd.m_direction_dx = Vector3D_d(d[3], d[4], d[5]);
        rd.m_origin_dy = Point3D_d(d[6], d[7], d[8]);
        rd.m_direction_dy = Vector3D_d(d[9], d[10], d[11]);
      }
      double *o = out + 40 * i;
      Intersection is;
      double th;
      if (!ra->accel->Intersect(rd, is, &th)) {
        for (int k = 0; k < 40; ++k) o[k] = std::numeric_limits<double>::quiet_NaN();
        o[35] = o[36] = -1.0;
        if (next_tmin) next_tmin[i] = std::numeric_limits<double>::quiet_NaN();
        continue;
      }
      const DifferentialGeometry &g = is.m_dg;
      const double v[35] = {g.m_point[0], g.m_point[1], g.m_point[2], g.m_geometric_normal[0],
                            g.m_geometric_normal[1], g.m_geometric_normal[2], g.m_shading_normal[0],
                            g.m_shading_normal[1], g.m_shading_normal[2], g.m_uv[0], g.m_uv[1], g.m_point_dx[0],
                            g.m_point_dx[1], g.m_point_dx[2], g.m_point_dy[0], g.m_point_dy[1], g.m_point_dy[2],
                            g.m_normal_dx[0], g.m_normal_dx[1], g.m_normal_dx[2], g.m_normal_dy[0], g.m_normal_dy[1],
                            g.m_normal_dy[2], g.m_duv_dx[0], g.m_duv_dx[1], g.m_duv_dy[0], g.m_duv_dy[1],
                            g.m_tangent[0], g.m_tangent[1], g.m_tangent[2], is.m_cross[0], is.m_cross[1],
                            is.m_cross[2], is.m_dot, th};
      for (int k = 0; k < 35; ++k) o[k] = v[k];
      size_t pi = 0;
      for (; pi < ra->prims.size(); ++pi)
        if (ra->prims[pi].get() == is.mp_primitive) break;
      o[35] = (double)pi;
      o[36] = (double)is.m_triangle_index;
      o[37] = o[38] = o[39] = 0.0;
      if (next_dirs && next_tmin) {
        const double *nd = next_dirs + 3 * i;
        next_tmin[i] = CoreUtils::GetNextMinT(is, Vector3D_d(nd[0], nd[1], nd[2]));
      }
    }
  });
}

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

// Instances of the accelerator in its final (partitioned) order: primitive
// index, the world-to-mesh matrix the traversal applies to rays (the
// instance Transform's inverse matrix, row-major) and the triangle count of
// the instanced subtree; plus whether the meshes' addresses ascend with
// their creation order (the reference orders shared meshes by address).
int64_t skw_ref_accel_num_instances(void *a) { return (int64_t)((RefAccel *)a)->accel->m_instance_nodes.size(); }

void skw_ref_accel_export_instances(void *a, int32_t *prim, double *world_to_mesh, int32_t *sub_tris) {
  const TriangleAccelerator &acc = *((RefAccel *)a)->accel;
  for (size_t i = 0; i < acc.m_instance_nodes.size(); ++i) {
    prim[i] = (int32_t)acc.m_instance_primitive_indices[i];
    const Matrix4x4_d &m = acc.m_instance_to_world_transformations[i].m_inverted_matrix;
    for (int r = 0; r < 4; ++r)
      for (int c = 0; c < 4; ++c) world_to_mesh[16 * i + 4 * r + c] = m.m_values[r][c];
    sub_tris[i] = (int32_t)(acc.m_instance_nodes[i]->m_triangles_end - acc.m_instance_nodes[i]->m_triangles_begin);
  }
}

// rank[m] = position of mesh m (meshes numbered in order of first use by
// the primitives) in the reference's address order of meshes.
void skw_ref_accel_mesh_rank(void *a, int32_t *rank) {
  const RefAccel *ra = (const RefAccel *)a;
  std::vector<const TriangleMesh *> seen;
  for (const auto &p : ra->prims) {
    const TriangleMesh *m = p->GetTriangleMesh_RawPtr();
    if (std::find(seen.begin(), seen.end(), m) == seen.end()) seen.push_back(m);
  }
  std::vector<const TriangleMesh *> sorted = seen;
  std::sort(sorted.begin(), sorted.end());
  for (size_t i = 0; i < seen.size(); ++i)
    rank[i] = (int32_t)(std::find(sorted.begin(), sorted.end(), seen[i]) - sorted.begin());
}

int skw_ref_accel_meshes_ascending(void *a) {
  const RefAccel *ra = (const RefAccel *)a;
  const TriangleMesh *prev = nullptr;
  std::vector<const TriangleMesh *> seen;
  for (const auto &p : ra->prims) {
    const TriangleMesh *m = p->GetTriangleMesh_RawPtr();
    if (std::find(seen.begin(), seen.end(), m) != seen.end()) continue;
    if (prev && m < prev) return 0;
    seen.push_back(m);
    prev = m;
  }
  return 1;
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
  const void *measured;  // kind 3: a MERLMeasuredData (skw_ref_merl_create)
  float refractive_index;  // kinds 4, 6: TransparentMaterial, UberMaterial
  float kr[3];             // kind 6: UberMaterial
  float opacity[3];        // kind 6: UberMaterial
  int32_t mix[2];          // kind 7: MixMaterial
  float mix_scale[3];      // kind 7: MixMaterial
  float v_roughness;       // kind 5: > 0 the two-roughness SubstrateMaterial
};
struct RefPrimIn {
  int32_t mesh;
  const double *mesh_to_world;
  int32_t material;
  const float *vertex_normals;
  const float *triangle_albedo;
  float emission[3];
  const float *vertex_tangents;  // TriangleMesh tangents (mesh space) or NULL
  const float *triangle_uvs;     // 6 floats per triangle (MeshTriangle::m_uvs) or NULL
};

static intrusive_ptr<const Texture<SpectrumCoef_d>> const_rgb(const float *v) {
  return intrusive_ptr<const Texture<SpectrumCoef_d>>(new ConstantTexture<SpectrumCoef_d>(SpectrumCoef_d(v[0], v[1], v[2])));
}
static intrusive_ptr<const Texture<double>> const_d(double v) {
  return intrusive_ptr<const Texture<double>>(new ConstantTexture<double>(v));
}

// The reference material for materials[i]; kd: its diffuse texture (the
// per-triangle albedo where the primitive has one).
static intrusive_ptr<const Material> make_material(const RefMaterialIn *materials, int i,
                                                   intrusive_ptr<const Texture<SpectrumCoef_d>> kd) {
  const RefMaterialIn &M = materials[i];
  intrusive_ptr<const Material> mat;
  if (M.kind == 0) {
    mat.reset(new MatteMaterial(kd, const_d(M.sigma)));
  } else if (M.kind == 1) {
    mat.reset(new PlasticMaterial(kd, const_rgb(M.ks), const_d(M.roughness)));
  } else if (M.kind == 3) {
    mat.reset(new MERLMeasuredMaterial(intrusive_ptr<const MERLMeasuredData>((const MERLMeasuredData *)M.measured)));
  } else if (M.kind == 4) {
    mat.reset(new TransparentMaterial(const_rgb(M.kd), const_rgb(M.ks), (double)M.refractive_index));
  } else if (M.kind == 5) {
    if (M.v_roughness > 0.0f)
      mat.reset(new SubstrateMaterial(kd, const_rgb(M.ks), const_d(M.roughness), const_d(M.v_roughness)));
    else
      mat.reset(new SubstrateMaterial(kd, const_rgb(M.ks), const_d(M.roughness)));
  } else if (M.kind == 6) {
    mat.reset(new UberMaterial(kd, const_rgb(M.ks), const_rgb(M.kr), const_d(M.roughness), const_rgb(M.opacity),
                               (double)M.refractive_index));
  } else if (M.kind == 7) {
    auto sub = [&](int j) {
      return make_material(materials, j, const_rgb(materials[j].kd));
    };
    mat.reset(new MixMaterial(sub(M.mix[0]), M.mix[1] >= 0 ? sub(M.mix[1]) : intrusive_ptr<const Material>(),
                              const_rgb(M.mix_scale)));
  } else {
    mat.reset(new MetalMaterial(const_rgb(M.eta), const_rgb(M.k), const_d(M.roughness)));
  }
  return mat;
}

// The reference Scene for the product's scene description (meshes,
// primitives with materials / emission / shading normals / per-triangle
// albedo, point lights).
static intrusive_ptr<const Scene> make_scene(int n_meshes, const float *const *verts, const int64_t *n_verts,
                                             const int32_t *const *tris, const int64_t *n_tris, int n_prims,
                                             const RefPrimIn *prims, const RefMaterialIn *materials,
                                             int n_point_lights, const float *point_lights,
                                             const double *medium = nullptr) {
  (void)n_meshes;
  std::vector<intrusive_ptr<const Primitive>> prim_list;
  LightSources lights;
  for (int p = 0; p < n_prims; ++p) {
    const RefPrimIn &P = prims[p];
    const int m = P.mesh;
    std::vector<Point3D_f> v((size_t)n_verts[m]);
    for (int64_t i = 0; i < n_verts[m]; ++i)
      v[(size_t)i] = Point3D_f(verts[m][3 * i], verts[m][3 * i + 1], verts[m][3 * i + 2]);
    std::vector<MeshTriangle> t((size_t)n_tris[m]);
    for (int64_t i = 0; i < n_tris[m]; ++i) {
      t[(size_t)i] = MeshTriangle(tris[m][3 * i], tris[m][3 * i + 1], tris[m][3 * i + 2]);
      if (P.triangle_uvs)
        for (int k = 0; k < 3; ++k)
          t[(size_t)i].m_uvs[k] = Point2D_f(P.triangle_uvs[6 * i + 2 * k], P.triangle_uvs[6 * i + 2 * k + 1]);
    }
    intrusive_ptr<TriangleMesh> mesh;
    std::vector<Vector3D_f> tan;
    if (P.vertex_tangents) {
      tan.resize((size_t)n_verts[m]);
      for (int64_t i = 0; i < n_verts[m]; ++i)
        tan[(size_t)i] = Vector3D_f(P.vertex_tangents[3 * i], P.vertex_tangents[3 * i + 1], P.vertex_tangents[3 * i + 2]);
    }
    if (P.vertex_normals) {
      std::vector<Vector3D_f> nrm((size_t)n_verts[m]);
      for (int64_t i = 0; i < n_verts[m]; ++i)
        nrm[(size_t)i] = Vector3D_f(P.vertex_normals[3 * i], P.vertex_normals[3 * i + 1], P.vertex_normals[3 * i + 2]);
      mesh.reset(new TriangleMesh(v, t, nrm, tan, true, false));
    } else if (!tan.empty()) {
      mesh.reset(new TriangleMesh(v, t, std::vector<Vector3D_f>(), tan, false, false));
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
    intrusive_ptr<const Material> mat = make_material(materials, P.material, kd);
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
  // medium: bounds lo[3], hi[3], emission[3], absorption[3], scattering[3], HG g
  intrusive_ptr<const VolumeRegion> volume;
  if (medium) {
    BBox3D_d b(Point3D_d(medium[0], medium[1], medium[2]), Point3D_d(medium[3], medium[4], medium[5]));
    Spectrum_d em(medium[6], medium[7], medium[8]);
    SpectrumCoef_d ab(medium[9], medium[10], medium[11]), sc(medium[12], medium[13], medium[14]);
    volume.reset(new HomogeneousVolumeRegion(b, em, ab, sc, intrusive_ptr<const PhaseFunction>(new HGPhaseFunction(medium[15]))));
  }
  return intrusive_ptr<const Scene>(new Scene(prim_list, volume, lights));
}

// Renders `integrator` with the reference's SamplerBasedRenderer,
// StratifiedSampler (ld = 0) or LDSampler with spp_x * spp_y samples per
// pixel and its default ConsecutiveImagePixelsOrder (ld = 1),
// PerspectiveCamera and an ImageFilm with a 0.5-wide BoxFilter into film_out
// (height x width x 3).
static double render_film(intrusive_ptr<LTEIntegrator> integrator, const double *camera_to_world, double x_view_angle,
                          int width, int height, int spp_x, int spp_y, float *film_out, int ld = 0) {
  intrusive_ptr<FilmFilter> filter(new BoxFilter(0.5, 0.5));
  intrusive_ptr<ImageFilm> film(new ImageFilm((size_t)width, (size_t)height, filter));
  intrusive_ptr<const Camera> camera(new PerspectiveCamera(make_transform(camera_to_world), film, 0.0, 1.0, x_view_angle));
  Point2D_i begin, end;
  film->GetSamplingExtent(begin, end);
  intrusive_ptr<Sampler> sampler;
  if (ld)
    sampler.reset(new LDSampler(begin, end, (size_t)spp_x * (size_t)spp_y));
  else
    sampler.reset(new StratifiedSampler(begin, end, (size_t)spp_x, (size_t)spp_y));
  SamplerBasedRenderer renderer(integrator, sampler);
  auto t0 = std::chrono::steady_clock::now();
  renderer.Render(camera, false);
  const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
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
  return sec;
}

// Renders the direct-lighting image (DirectLightingLTEIntegrator), with an
// optional homogeneous medium (17 doubles: bounds lo, hi, emission,
// absorption, scattering, HG g, march step; NULL = none).
int skw_ref_render_direct(int n_meshes, const float *const *verts, const int64_t *n_verts, const int32_t *const *tris,
                          const int64_t *n_tris, int n_prims, const RefPrimIn *prims, int n_materials,
                          const RefMaterialIn *materials, int n_point_lights, const float *point_lights,
                          const double *camera_to_world, double x_view_angle, int width, int height, int spp_x,
                          int spp_y, int light_samples, float *film_out, double *seconds_out, const double *medium,
                          int ld) {
  (void)n_materials;
  intrusive_ptr<const Scene> scene = make_scene(n_meshes, verts, n_verts, tris, n_tris, n_prims, prims, materials,
                                                n_point_lights, point_lights, medium);
  DirectLightingLTEIntegratorParams params;
  params.m_direct_light_samples_num = (size_t)light_samples;
  params.m_max_specular_depth = 6;
  params.m_media_step_size = medium ? medium[16] : 0.01;  // medium[16]: the march step
  intrusive_ptr<LTEIntegrator> integrator(new DirectLightingLTEIntegrator(scene, params));
  const double sec = render_film(integrator, camera_to_world, x_view_angle, width, height, spp_x, spp_y, film_out, ld);
  if (seconds_out) *seconds_out = sec;
  return 0;
}

// Photon-mapping render (PhotonLTEIntegrator): ShootPhotons(n_paths) then
// the sampler-based render with final gathering.  info_out: caustic, direct,
// indirect, irradiance photon counts; seconds_out: shooting (incl. the maps)
// and rendering.
int skw_ref_render_photon(int n_meshes, const float *const *verts, const int64_t *n_verts, const int32_t *const *tris,
                          const int64_t *n_tris, int n_prims, const RefPrimIn *prims, const RefMaterialIn *materials,
                          int n_point_lights, const float *point_lights, const double *camera_to_world,
                          double x_view_angle, int width, int height, int spp_x, int spp_y, int light_samples,
                          int64_t n_paths, int gather_samples, int caustic_lookup, double max_caustic_dist,
                          float *film_out, int64_t *info_out, double *seconds_out) {
  intrusive_ptr<const Scene> scene =
      make_scene(n_meshes, verts, n_verts, tris, n_tris, n_prims, prims, materials, n_point_lights, point_lights);
  PhotonLTEIntegratorParams params;
  params.m_direct_light_samples_num = (size_t)light_samples;
  params.m_caustic_lookup_photons_num = (size_t)caustic_lookup;
  params.m_max_caustic_lookup_dist = max_caustic_dist;
  params.m_gather_samples_num = (size_t)gather_samples;
  params.m_max_specular_depth = 6;
  params.m_media_step_size = 0.01;
  intrusive_ptr<PhotonLTEIntegrator> integrator(new PhotonLTEIntegrator(scene, params));
  auto t0 = std::chrono::steady_clock::now();
  integrator->ShootPhotons((size_t)n_paths, false);
  const double shoot = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (info_out) {
    auto &maps = integrator->mp_photon_maps;
    info_out[0] = maps->GetCausticMap() ? (int64_t)maps->GetCausticMap()->GetNumberOfPoints() : 0;
    info_out[1] = maps->GetDirectMap() ? (int64_t)maps->GetDirectMap()->GetNumberOfPoints() : 0;
    info_out[2] = maps->GetIndirectMap() ? (int64_t)maps->GetIndirectMap()->GetNumberOfPoints() : 0;
    info_out[3] = integrator->mp_irradiance_map ? (int64_t)integrator->mp_irradiance_map->GetNumberOfPoints() : 0;
  }
  double render = 0.0;
  if (width > 0 && height > 0)
    render = render_film(integrator, camera_to_world, x_view_angle, width, height, spp_x, spp_y, film_out);
  if (seconds_out) {
    seconds_out[0] = shoot;
    seconds_out[1] = render;
  }
  return 0;
}

// PhotonLTEIntegrator::ShootPhotons(n_paths) alone: the photon positions of
// the caustic, direct and indirect maps (3 floats each, at most cap[m] per
// map m, in the maps' kd-tree order) and each map's size in n_out[m].
int skw_ref_shoot_photons(int n_meshes, const float *const *verts, const int64_t *n_verts, const int32_t *const *tris,
                          const int64_t *n_tris, int n_prims, const RefPrimIn *prims, const RefMaterialIn *materials,
                          int n_point_lights, const float *point_lights, int64_t n_paths, float *const *pos_out,
                          const int64_t *cap, int64_t *n_out) {
  intrusive_ptr<const Scene> scene =
      make_scene(n_meshes, verts, n_verts, tris, n_tris, n_prims, prims, materials, n_point_lights, point_lights);
  PhotonLTEIntegratorParams params;
  params.m_max_specular_depth = 6;
  params.m_media_step_size = 0.01;
  intrusive_ptr<PhotonLTEIntegrator> integrator(new PhotonLTEIntegrator(scene, params));
  integrator->ShootPhotons((size_t)n_paths, false);
  auto &maps = integrator->mp_photon_maps;
  shared_ptr<const KDTree<PhotonLTEIntegrator::Photon>> m[3] = {maps->GetCausticMap(), maps->GetDirectMap(),
                                                                maps->GetIndirectMap()};
  for (int k = 0; k < 3; ++k) {
    n_out[k] = m[k] ? (int64_t)m[k]->GetNumberOfPoints() : 0;
    for (int64_t i = 0; m[k] && i < std::min(n_out[k], cap[k]); ++i)
      for (int c = 0; c < 3; ++c) pos_out[k][3 * i + c] = m[k]->m_points[(size_t)i].m_point[c];
  }
  return 0;
}

// _ConstructIrradiancePhotonMap on given photon maps (28-byte records:
// position, weight, incident id, normal id), each with its number of paths,
// and the scene's total area: the irradiance photons in the reference's
// kd-tree order (position, external and internal irradiance, normal id) and
// m_max_irradiance_lookup_dist.  n_irr_out: their count (the arrays must
// hold n_indirect / 10 + 1 entries).
struct RefPhotonIn {
  float p[3];
  float w[3];
  uint16_t dir, nrm;
};
int skw_ref_photon_irradiance(const RefPhotonIn *const *photons, const int64_t *n, const int64_t *paths,
                              double scene_area, int64_t *n_irr_out, float *pos, float *ext, float *intr,
                              uint16_t *nrm, double *max_dist_out) {
  // A one-triangle scene: the integrator needs one, and the area is set below.
  std::vector<Point3D_f> v = {Point3D_f(0, 0, 0), Point3D_f(1, 0, 0), Point3D_f(0, 1, 0)};
  std::vector<MeshTriangle> t = {MeshTriangle(0, 1, 2)};
  intrusive_ptr<TriangleMesh> mesh(new TriangleMesh(v, t, false, false));
  std::vector<intrusive_ptr<const Primitive>> prim_list = {intrusive_ptr<const Primitive>(
      new Primitive(mesh, Transform(), intrusive_ptr<const Material>(), intrusive_ptr<const AreaLightSource>(), NULL))};
  LightSources lights;
  intrusive_ptr<const Scene> scene(new Scene(prim_list, NULL, lights));
  PhotonLTEIntegratorParams params;
  params.m_direct_light_samples_num = 1;
  params.m_caustic_lookup_photons_num = 50;
  params.m_max_caustic_lookup_dist = 0.1;
  params.m_gather_samples_num = 4;
  params.m_max_specular_depth = 6;
  params.m_media_step_size = 0.01;
  PhotonLTEIntegrator integ(scene, params);
  integ.m_scene_total_area = scene_area;
  integ.mp_photon_maps.reset(new PhotonLTEIntegrator::PhotonMaps());
  for (int m = 0; m < 3; ++m) {
    std::vector<RefPhoton> ph((size_t)n[m]);
    for (int64_t i = 0; i < n[m]; ++i) {
      const RefPhotonIn &r = photons[m][i];
      ph[(size_t)i] = RefPhoton(Point3D_f(r.p[0], r.p[1], r.p[2]), Spectrum_f(r.w[0], r.w[1], r.w[2]),
                                CompressedDirection::FromID(r.dir), CompressedDirection::FromID(r.nrm));
    }
    if (m == 0) integ.mp_photon_maps->AddCausticPhotons(ph, (size_t)paths[m]);
    if (m == 1) integ.mp_photon_maps->AddDirectPhotons(ph, (size_t)paths[m]);
    if (m == 2) integ.mp_photon_maps->AddIndirectPhotons(ph, (size_t)paths[m]);
  }
  integ.mp_photon_maps->GetCausticMap();
  integ.mp_photon_maps->GetDirectMap();
  integ.mp_photon_maps->GetIndirectMap();
  integ._ConstructIrradiancePhotonMap();
  int64_t k = 0;
  if (integ.mp_irradiance_map) {
    const auto &P = integ.mp_irradiance_map->GetAllPoints();
    for (const auto &ip : P) {
      for (int c = 0; c < 3; ++c) {
        pos[3 * k + c] = ip.m_point[c];
        ext[3 * k + c] = ip.m_external_irradiance[c];
        intr[3 * k + c] = ip.m_internal_irradiance[c];
      }
      nrm[k] = ip.m_normal.GetID();
      ++k;
    }
  }
  *n_irr_out = k;
  *max_dist_out = integ.m_max_irradiance_lookup_dist;
  return 0;
}

// Photon-mapping render with given photon maps instead of shooting: the
// maps (28-byte records, each with its number of paths) are added as
// ShootPhotons' merging filter adds them, the kd-trees and the irradiance
// map are built as at the end of ShootPhotons (PhotonLTEIntegrator.cpp:
// 271-277), then the sampler-based render runs.  info_out: the four map
// sizes; seconds_out: the render time.
int skw_ref_render_photon_maps(int n_meshes, const float *const *verts, const int64_t *n_verts,
                               const int32_t *const *tris, const int64_t *n_tris, int n_prims, const RefPrimIn *prims,
                               const RefMaterialIn *materials, int n_point_lights, const float *point_lights,
                               const RefPhotonIn *const *photons, const int64_t *n_photons, const int64_t *paths,
                               const double *camera_to_world, double x_view_angle, int width, int height, int spp_x,
                               int spp_y, int light_samples, int gather_samples, int caustic_lookup,
                               double max_caustic_dist, float *film_out, int64_t *info_out, double *seconds_out) {
  intrusive_ptr<const Scene> scene =
      make_scene(n_meshes, verts, n_verts, tris, n_tris, n_prims, prims, materials, n_point_lights, point_lights);
  PhotonLTEIntegratorParams params;
  params.m_direct_light_samples_num = (size_t)light_samples;
  params.m_caustic_lookup_photons_num = (size_t)caustic_lookup;
  params.m_max_caustic_lookup_dist = max_caustic_dist;
  params.m_gather_samples_num = (size_t)gather_samples;
  params.m_max_specular_depth = 6;
  params.m_media_step_size = 0.01;
  intrusive_ptr<PhotonLTEIntegrator> integrator(new PhotonLTEIntegrator(scene, params));
  integrator->mp_photon_maps.reset(new PhotonLTEIntegrator::PhotonMaps());
  for (int m = 0; m < 3; ++m) {
    std::vector<RefPhoton> ph((size_t)n_photons[m]);
    for (int64_t i = 0; i < n_photons[m]; ++i) {
      const RefPhotonIn &r = photons[m][i];
      ph[(size_t)i] = RefPhoton(Point3D_f(r.p[0], r.p[1], r.p[2]), Spectrum_f(r.w[0], r.w[1], r.w[2]),
                                CompressedDirection::FromID(r.dir), CompressedDirection::FromID(r.nrm));
    }
    if (m == 0) integrator->mp_photon_maps->AddCausticPhotons(ph, (size_t)paths[m]);
    if (m == 1) integrator->mp_photon_maps->AddDirectPhotons(ph, (size_t)paths[m]);
    if (m == 2) integrator->mp_photon_maps->AddIndirectPhotons(ph, (size_t)paths[m]);
  }
  integrator->mp_photon_maps->GetCausticMap();
  integrator->mp_photon_maps->GetDirectMap();
  integrator->mp_photon_maps->GetIndirectMap();
  integrator->_ConstructIrradiancePhotonMap();
  if (info_out) {
    auto &maps = integrator->mp_photon_maps;
    info_out[0] = maps->GetCausticMap() ? (int64_t)maps->GetCausticMap()->GetNumberOfPoints() : 0;
    info_out[1] = maps->GetDirectMap() ? (int64_t)maps->GetDirectMap()->GetNumberOfPoints() : 0;
    info_out[2] = maps->GetIndirectMap() ? (int64_t)maps->GetIndirectMap()->GetNumberOfPoints() : 0;
    info_out[3] = integrator->mp_irradiance_map ? (int64_t)integrator->mp_irradiance_map->GetNumberOfPoints() : 0;
  }
  const double render = render_film(integrator, camera_to_world, x_view_angle, width, height, spp_x, spp_y, film_out);
  if (seconds_out) seconds_out[0] = render;
  return 0;
}

// ------------------------------------------------------------- measured BRDF

// MERLMeasuredData from a file image in the MERL binary format (3 int32
// dims, then 3 channels of doubles).
void *skw_ref_merl_create(const char *bytes, int64_t n_bytes) {
  std::string buf(bytes, (size_t)n_bytes);
  std::istringstream is(buf, std::ios::binary);
  auto *d = new MERLMeasuredData(is);
  d->IncRef();
  return d;
}

void skw_ref_merl_destroy(void *d) {
  if (((MERLMeasuredData *)d)->DecRef() == 0) delete (MERLMeasuredData *)d;
}

// The converted table (half RGB per entry, the reference's m_brdf_data) and
// the sampling segmentations: per incident theta bin, the 45 x 24 column
// CDFs, the 24 row CDFs, the 45 X and 24 Y grid lines (1,173 floats).
void skw_ref_merl_export(void *dp, uint16_t *table, float *seg) {
  const MERLMeasuredData *d = (const MERLMeasuredData *)dp;
  for (size_t i = 0; i < d->m_brdf_data.size(); ++i)
    for (int c = 0; c < 3; ++c) {
      const HalfFloat h = d->m_brdf_data[i][c];
      std::memcpy(&table[3 * i + c], &h, 2);
    }
  float *o = seg;
  for (const auto &sg : d->m_segmentations) {
    for (size_t i = 0; i < MERLMeasuredData::SEGMENTATION_EXITANT_THETA_RES; ++i)
      for (size_t j = 0; j < MERLMeasuredData::SEGMENTATION_EXITANT_PHI_RES; ++j) *o++ = sg.m_CDF_cols[i][j];
    for (float v : sg.m_CDF_rows) *o++ = v;
    for (float v : sg.m_grid_X) *o++ = v;
    for (float v : sg.m_grid_Y) *o++ = v;
  }
}

// MERLMeasured BxDF (local frame): Evaluate / PDF for n direction pairs
// (3 doubles each); Sample for n incident directions and 2D samples.
void skw_ref_merl_eval(void *dp, const double *wi, const double *wo, int64_t n, double *f, double *pdf) {
  MERLMeasured bx((const MERLMeasuredData *)dp);
  for (int64_t i = 0; i < n; ++i) {
    const Vector3D_d a(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]), b(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
    const SpectrumCoef_d v = bx.Evaluate(a, b);
    for (int c = 0; c < 3; ++c) f[3 * i + c] = v[c];
    pdf[i] = bx.PDF(a, b);
  }
}

void skw_ref_merl_sample(void *dp, const double *wi, const double *u, int64_t n, double *wo, double *f, double *pdf) {
  MERLMeasured bx((const MERLMeasuredData *)dp);
  for (int64_t i = 0; i < n; ++i) {
    const Vector3D_d a(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]);
    Vector3D_d e;
    double p = 0.0;
    const SpectrumCoef_d v = bx.Sample(a, e, Point2D_d(u[2 * i], u[2 * i + 1]), p);
    for (int c = 0; c < 3; ++c) {
      wo[3 * i + c] = e[c];
      f[3 * i + c] = v[c];
    }
    pdf[i] = p;
  }
}

// The loader's colour conversion: RGB -> XYZ (sRGB primaries, E white) ->
// spectrum coefficients, for n RGB triples.
void skw_ref_merl_convert(const double *rgb, int64_t n, double *out) {
  for (int64_t i = 0; i < n; ++i) {
    RGBColor_d c(rgb[3 * i], rgb[3 * i + 1], rgb[3 * i + 2]);
    XYZColor_d xyz = global_sRGB_E_ColorSystem.RGB_To_XYZ(c);
    SpectrumCoef_d s = SpectrumRoutines::XYZToSpectrumCoef(xyz);
    for (int k = 0; k < 3; ++k) out[3 * i + k] = s[k];
  }
}

// The two stages of that conversion separately (stage 0: RGB -> XYZ,
// stage 1: XYZ -> spectrum coefficients).
void skw_ref_color_stage(int stage, const double *in, int64_t n, double *out) {
  for (int64_t i = 0; i < n; ++i) {
    if (stage == 0) {
      XYZColor_d x = global_sRGB_E_ColorSystem.RGB_To_XYZ(RGBColor_d(in[3 * i], in[3 * i + 1], in[3 * i + 2]));
      for (int k = 0; k < 3; ++k) out[3 * i + k] = x[k];
    } else {
      SpectrumCoef_d s = SpectrumRoutines::XYZToSpectrumCoef(XYZColor_d(in[3 * i], in[3 * i + 1], in[3 * i + 2]));
      for (int k = 0; k < 3; ++k) out[3 * i + k] = s[k];
    }
  }
}

// The PBRT importer's colour parameters (PbrtImport::ParamSet,
// CADImport/SceneImporters/PbrtSceneImporter/PbrtParamSet.cpp:99-129) for n
// float RGB triples: kind 0 a reflectance (AddRGBSpectrumCoef: a grey
// triple as is, else sRGB with the E white point, then XYZ ->
// coefficients), kind 1 an emission (AddRGBSpectrum: sRGB with the D65
// white point, then XYZ -> spectrum); kind 2 that emission's XYZ.
void skw_ref_pbrt_rgb(int kind, const float *rgb, int64_t n, double *out) {
  for (int64_t i = 0; i < n; ++i) {
    const float r = rgb[3 * i], g = rgb[3 * i + 1], b = rgb[3 * i + 2];
    if (kind == 0) {
      SpectrumCoef_d s = (r == g && r == b)
                             ? SpectrumCoef_d(r)
                             : SpectrumRoutines::XYZToSpectrumCoef(global_sRGB_E_ColorSystem.RGB_To_XYZ(RGBColor_d(r, g, b)));
      for (int k = 0; k < 3; ++k) out[3 * i + k] = s[k];
    } else if (kind == 1) {
      Spectrum_d s = SpectrumRoutines::XYZToSpectrum(global_sRGB_D65_ColorSystem.RGB_To_XYZ(RGBColor_d(r, g, b)));
      for (int k = 0; k < 3; ++k) out[3 * i + k] = s[k];
    } else {  // kind 2: the first stage of kind 1 alone (RGB -> XYZ, D65)
      XYZColor_d x = global_sRGB_D65_ColorSystem.RGB_To_XYZ(RGBColor_d(r, g, b));
      for (int k = 0; k < 3; ++k) out[3 * i + k] = x[k];
    }
  }
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
