// Drop-in replacement for Skwarka's Raytracer/Core/TriangleAccelerator.h
// that runs the ray queries on the GPU through the C ABI of this library
// (include/skw.h).
//
// It declares the class the reference declares (TriangleAccelerator.h:
// 35-65 of the reference: the constructor over primitives, Intersect,
// IntersectTest, GetWorldBounds; not copyable), so the reference's Scene
// (Scene.h:99 holds one by value) and every caller of Scene::Intersect /
// IntersectTest compile and run unchanged when this header and
// TriangleAccelerator.cpp replace the reference's two files in its build
// and the build links libskw.so.  Answers are the reference's bit for bit:
// the traversal runs the double-ray entry points (skw_intersect_d*, the
// reference's exact t and hit ids), and the Intersection is completed on
// the host with the reference's own TriangleMesh code, as its Intersect
// completes it.  Batched forms of both queries serve callers that can
// collect many rays.
//
// Threading: all queries are const and may come from many threads (the
// reference's class is thread-safe); they are serialised on a mutex, since
// one library context serves one host thread at a time.
#ifndef TRIANGLE_ACCELERATOR_H
#define TRIANGLE_ACCELERATOR_H

#include <Common/Common.h>
#include <Math/Geometry.h>
#include "Primitive.h"
#include "Intersection.h"

#include <mutex>
#include <vector>

struct skw_ctx;
struct skw_accel;

class TriangleAccelerator
  {
  public:
    // Builds the ternary bbox kd-tree over the primitives (instances for
    // meshes shared by several primitives) and uploads it to GPU 0.
    TriangleAccelerator(std::vector<intrusive_ptr<const Primitive>> i_primitives);
    ~TriangleAccelerator();

    // The reference's queries, one ray each.
    bool Intersect(const RayDifferential &i_ray, Intersection &o_intersection, double *o_t = NULL) const;
    bool IntersectTest(const Ray &i_ray) const;
    BBox3D_d GetWorldBounds() const;

    // The same for n rays in one GPU call: o_hit[i] tells whether ray i hit
    // (o_intersections[i] and o_t[i], if o_t is not NULL, are then set).
    void Intersect(const RayDifferential *i_rays, size_t i_n, Intersection *o_intersections, double *o_t,
                   bool *o_hit) const;
    void IntersectTest(const Ray *i_rays, size_t i_n, bool *o_hit) const;

  private:
    TriangleAccelerator();
    TriangleAccelerator(TriangleAccelerator &);
    TriangleAccelerator &operator=(TriangleAccelerator &);

    // Fills the Intersection of a hit on (primitive, mesh triangle).
    void _Complete(const RayDifferential &i_ray, size_t i_primitive, size_t i_triangle,
                   Intersection &o_intersection) const;

  private:
    std::vector<intrusive_ptr<const Primitive>> m_primitives;
    // The library's primitive order (meshes by address, as the reference
    // builds its tree) and back.
    std::vector<size_t> m_order;
    skw_ctx *mp_ctx;
    skw_accel *mp_accel;
    BBox3D_d m_bounds;
    mutable std::mutex m_mutex;
  };

#endif // TRIANGLE_ACCELERATOR_H
