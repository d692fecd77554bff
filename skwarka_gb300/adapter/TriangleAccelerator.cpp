// TriangleAccelerator over the GB300 library (see TriangleAccelerator.h).
//
// Construction hands the primitives' meshes and transforms to
// skw_accel_create in the reference's order (it keys meshes by address,
// TriangleAccelerator.cpp:25-38 of the reference), so the device tree is
// the reference's node for node.  Queries convert the reference's Ray to
// skw_ray_d, run the double-ray traversal, and complete each hit's
// Intersection with the reference's own code path: the ray taken to mesh
// space, TriangleMesh::ComputeDifferentialGeometry, the geometry taken back
// to world space and the m_cross / m_dot that CoreUtils::GetNextMinT reads
// (the steps of TriangleAccelerator::Intersect, TriangleAccelerator.cpp:
// 303-347 of the reference, which have to happen in that order for the
// result to be bit-identical).
#include "TriangleAccelerator.h"
#include "TriangleMesh.h"

#include <algorithm>
#include <cmath>
#include <map>
#include <stdexcept>
#include <string>

#include <skw.h>

namespace {

void check(int rc, skw_ctx *ctx, const char *what) {
  if (rc != SKW_OK)
    throw std::runtime_error(std::string("TriangleAccelerator (GPU): ") + what + ": " +
                             (ctx ? skw_last_error(ctx) : "no context"));
}

skw_ray_d to_skw(const Ray &r) {
  skw_ray_d o;
  o.ox = r.m_origin[0];
  o.oy = r.m_origin[1];
  o.oz = r.m_origin[2];
  o.dx = r.m_direction[0];
  o.dy = r.m_direction[1];
  o.dz = r.m_direction[2];
  o.tmin = r.m_min_t;
  o.tmax = r.m_max_t;
  return o;
}

}  // namespace

TriangleAccelerator::TriangleAccelerator(std::vector<intrusive_ptr<const Primitive>> i_primitives)
    : m_primitives(i_primitives), mp_ctx(NULL), mp_accel(NULL) {
  // meshes in address order; primitives grouped by mesh in that order, each
  // group in primitive order (the reference's std::map over mesh pointers)
  std::map<const TriangleMesh *, std::vector<size_t>> by_mesh;
  for (size_t i = 0; i < m_primitives.size(); ++i) by_mesh[m_primitives[i]->GetTriangleMesh_RawPtr()].push_back(i);
  std::vector<std::vector<float>> verts;
  std::vector<std::vector<int32_t>> tris;
  std::vector<skw_mesh> meshes;
  std::vector<skw_primitive> prims;
  std::vector<std::vector<double>> xforms;
  for (const auto &kv : by_mesh) {
    const TriangleMesh *m = kv.first;
    std::vector<float> v(3 * m->GetNumberOfVertices());
    for (size_t i = 0; i < m->GetNumberOfVertices(); ++i) {
      const Point3D_f p = m->GetVertex(i);
      v[3 * i] = p[0];
      v[3 * i + 1] = p[1];
      v[3 * i + 2] = p[2];
    }
    std::vector<int32_t> t(3 * m->GetNumberOfTriangles());
    for (size_t i = 0; i < m->GetNumberOfTriangles(); ++i) {
      const MeshTriangle mt = m->GetTriangle(i);
      for (int k = 0; k < 3; ++k) t[3 * i + k] = (int32_t)mt.m_vertices[k];
    }
    verts.push_back(std::move(v));
    tris.push_back(std::move(t));
    for (size_t p : kv.second) {
      m_order.push_back(p);
      const Matrix4x4_d mat = m_primitives[p]->GetMeshToWorldTransform().GetMatrix();
      std::vector<double> x(16);
      for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) x[4 * r + c] = mat.m_values[r][c];
      xforms.push_back(std::move(x));
    }
  }
  size_t mi = 0;
  for (const auto &kv : by_mesh) {
    meshes.push_back(skw_mesh{verts[mi].data(), (int64_t)verts[mi].size() / 3, tris[mi].data(),
                              (int64_t)tris[mi].size() / 3});
    for (size_t k = 0; k < kv.second.size(); ++k) prims.push_back(skw_primitive{(int32_t)mi, NULL});
    ++mi;
  }
  for (size_t i = 0; i < prims.size(); ++i) prims[i].mesh_to_world = xforms[i].data();
  check(skw_ctx_create(0, &mp_ctx), NULL, "no CUDA device");
  check(skw_accel_create(mp_ctx, meshes.data(), (int32_t)meshes.size(), prims.data(), (int32_t)prims.size(),
                         &mp_accel),
        mp_ctx, "build");
  skw_accel_info info;
  check(skw_accel_get_info(mp_accel, &info), mp_ctx, "info");
  // the root's float box, as GetWorldBounds returns it
  m_bounds = BBox3D_d(Point3D_d(info.bounds[0], info.bounds[1], info.bounds[2]),
                      Point3D_d(info.bounds[3], info.bounds[4], info.bounds[5]));
}

TriangleAccelerator::~TriangleAccelerator() {
  skw_accel_destroy(mp_accel);
  skw_ctx_destroy(mp_ctx);
}

BBox3D_d TriangleAccelerator::GetWorldBounds() const { return m_bounds; }

void TriangleAccelerator::_Complete(const RayDifferential &i_ray, size_t i_primitive, size_t i_triangle,
                                    Intersection &o_intersection) const {
  const intrusive_ptr<const Primitive> &p_primitive = m_primitives[i_primitive];
  o_intersection.mp_primitive = p_primitive.get();
  o_intersection.m_triangle_index = i_triangle;
  const TriangleMesh *p_mesh = p_primitive->GetTriangleMesh_RawPtr();
  const Transform mesh_to_world = p_primitive->GetMeshToWorldTransform();
  const Transform world_to_mesh = mesh_to_world.Inverted();
  // the ray and its differentials in mesh space
  RayDifferential mesh_ray(i_ray);
  world_to_mesh(i_ray.m_base_ray, mesh_ray.m_base_ray);
  world_to_mesh(i_ray.m_origin_dx, mesh_ray.m_origin_dx);
  world_to_mesh(i_ray.m_origin_dy, mesh_ray.m_origin_dy);
  world_to_mesh(i_ray.m_direction_dx, mesh_ray.m_direction_dx);
  world_to_mesh(i_ray.m_direction_dy, mesh_ray.m_direction_dy);
  DifferentialGeometry dg;
  p_mesh->ComputeDifferentialGeometry(i_triangle, mesh_ray, dg);
  // back to world space: points and the tangent by the transform, normals by
  // its normal transform
  DifferentialGeometry &w = o_intersection.m_dg;
  w = dg;
  mesh_to_world(dg.m_point, w.m_point);
  mesh_to_world(dg.m_point_dx, w.m_point_dx);
  mesh_to_world(dg.m_point_dy, w.m_point_dy);
  mesh_to_world(dg.m_tangent, w.m_tangent);
  w.m_geometric_normal = mesh_to_world.TransformNormal(dg.m_geometric_normal);
  w.m_shading_normal = mesh_to_world.TransformNormal(dg.m_shading_normal);
  w.m_normal_dx = mesh_to_world.TransformNormal(dg.m_normal_dx);
  w.m_normal_dy = mesh_to_world.TransformNormal(dg.m_normal_dy);
  // GetNextMinT's inputs, from the mesh-space triangle and the world point
  // taken back to mesh space
  const MeshTriangle tri = p_mesh->GetTriangle(i_triangle);
  const Point3D_d v0 = Convert<double>(p_mesh->GetVertex(tri.m_vertices[0]));
  const Point3D_d v1 = Convert<double>(p_mesh->GetVertex(tri.m_vertices[1]));
  const Point3D_d v2 = Convert<double>(p_mesh->GetVertex(tri.m_vertices[2]));
  const Vector3D_d e1(v1 - v0), e2(v2 - v0);
  o_intersection.m_cross = e1 ^ e2;
  o_intersection.m_dot = (Vector3D_d(v0 - world_to_mesh(w.m_point)) ^ e1) * e2;
}

void TriangleAccelerator::Intersect(const RayDifferential *i_rays, size_t i_n, Intersection *o_intersections,
                                    double *o_t, bool *o_hit) const {
  if (i_n == 0) return;
  std::vector<skw_ray_d> rays(i_n);
  for (size_t i = 0; i < i_n; ++i) rays[i] = to_skw(i_rays[i].m_base_ray);
  std::vector<skw_hit_d> hits(i_n);
  {
    std::lock_guard<std::mutex> lock(m_mutex);
    check(skw_intersect_d_host(mp_accel, rays.data(), (int64_t)i_n, hits.data()), mp_ctx, "Intersect");
  }
  for (size_t i = 0; i < i_n; ++i) {
    o_hit[i] = hits[i].prim >= 0;
    if (!o_hit[i]) {
      if (o_t) o_t[i] = hits[i].t;  // +inf, as the reference reports a miss
      continue;
    }
    if (o_t) o_t[i] = hits[i].t;
    _Complete(i_rays[i], m_order[(size_t)hits[i].prim], (size_t)hits[i].tri, o_intersections[i]);
  }
}

bool TriangleAccelerator::Intersect(const RayDifferential &i_ray, Intersection &o_intersection, double *o_t) const {
  bool hit = false;
  double t = 0.0;
  Intersect(&i_ray, 1, &o_intersection, &t, &hit);
  if (o_t) *o_t = t;
  return hit;
}

void TriangleAccelerator::IntersectTest(const Ray *i_rays, size_t i_n, bool *o_hit) const {
  if (i_n == 0) return;
  std::vector<skw_ray_d> rays(i_n);
  for (size_t i = 0; i < i_n; ++i) rays[i] = to_skw(i_rays[i]);
  std::vector<uint8_t> occ(i_n);
  {
    std::lock_guard<std::mutex> lock(m_mutex);
    check(skw_intersect_test_d_host(mp_accel, rays.data(), (int64_t)i_n, occ.data()), mp_ctx, "IntersectTest");
  }
  for (size_t i = 0; i < i_n; ++i) o_hit[i] = occ[i] != 0;
}

bool TriangleAccelerator::IntersectTest(const Ray &i_ray) const {
  bool hit = false;
  IntersectTest(&i_ray, 1, &hit);
  return hit;
}
