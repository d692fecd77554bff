/*
 * skw.hpp -- C++ host interface over the C ABI of skw.h.
 *
 * Owning wrappers with the reference's class and method names, in batched
 * form: the reference answers one ray / one query per call from many host
 * threads; these take whole batches (host vectors, or device buffers on a
 * stream).  Header only; link with libskw.  Errors throw skw::Error (the
 * status code and skw_last_error's message).
 *
 *   skw::TriangleAccelerator  TriangleAccelerator(primitives)
 *                             (Raytracer/Core/TriangleAccelerator.h:35-57):
 *                             Intersect / IntersectTest
 *   skw::PhotonKDTree         KDTree<Photon> (Raytracer/Core/KDTree.h:63-119):
 *                             GetNearestPoints with PhotonFilter
 *   skw::Scene                Scene + DirectLightingLTEIntegrator +
 *                             SamplerBasedRenderer::Render
 *                             (Renderers/SamplerBasedRenderer.cpp:200-239)
 *   skw::PhotonMap            PhotonLTEIntegrator::ShootPhotons and its
 *                             render with final gathering
 *                             (LTEIntegrators/PhotonLTEIntegrator/)
 */
#ifndef SKW_HPP
#define SKW_HPP

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "skw.h"

namespace skw {

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string &msg) : std::runtime_error(msg), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

inline void check(int rc, const skw_ctx *ctx, const char *what) {
  if (rc != SKW_OK) throw Error(rc, std::string(what) + ": " + (ctx ? skw_last_error(ctx) : "invalid argument"));
}

// Owns one handle; moves, never copies.
template <typename T, void (*Destroy)(T *)>
class Handle {
 public:
  Handle() = default;
  explicit Handle(T *h) : h_(h) {}
  Handle(Handle &&o) noexcept : h_(std::exchange(o.h_, nullptr)) {}
  Handle &operator=(Handle &&o) noexcept {
    if (this != &o) {
      reset();
      h_ = std::exchange(o.h_, nullptr);
    }
    return *this;
  }
  Handle(const Handle &) = delete;
  Handle &operator=(const Handle &) = delete;
  ~Handle() { reset(); }
  T *get() const { return h_; }
  void reset() {
    if (h_) Destroy(h_);
    h_ = nullptr;
  }

 private:
  T *h_ = nullptr;
};

// A CUDA device and the library's state on it (workspace pool, launch count).
class Context {
 public:
  explicit Context(int device = 0) {
    skw_ctx *c = nullptr;
    check(skw_ctx_create(device, &c), nullptr, "skw_ctx_create");
    h_ = Handle<skw_ctx, skw_ctx_destroy>(c);
  }
  skw_ctx *get() const { return h_.get(); }
  int64_t LaunchCount() const { return skw_launch_count(h_.get()); }

 private:
  Handle<skw_ctx, skw_ctx_destroy> h_;
};

// A mesh in mesh space: float xyz per vertex, vertex-index triples.
struct Mesh {
  std::vector<float> vertices;
  std::vector<int32_t> triangles;
};

namespace detail {
inline std::vector<skw_mesh> mesh_views(const std::vector<Mesh> &meshes) {
  std::vector<skw_mesh> v;
  v.reserve(meshes.size());
  for (const Mesh &m : meshes)
    v.push_back({m.vertices.data(), (int64_t)(m.vertices.size() / 3), m.triangles.data(),
                 (int64_t)(m.triangles.size() / 3)});
  return v;
}
}  // namespace detail

// TriangleAccelerator over primitives (a mesh and a row-major 4x4
// mesh-to-world matrix each, NULL = identity): the reference's kd-tree,
// built on the host node for node, traversed on the GPU.  A hit's prim is
// the index of the reference's Intersection::mp_primitive in `prims`, its
// tri the Intersection's m_triangle_index.
class TriangleAccelerator {
 public:
  TriangleAccelerator(Context &ctx, const std::vector<Mesh> &meshes, const std::vector<skw_primitive> &prims)
      : ctx_(ctx.get()) {
    const std::vector<skw_mesh> mv = detail::mesh_views(meshes);
    skw_accel *a = nullptr;
    check(skw_accel_create(ctx_, mv.data(), (int32_t)mv.size(), prims.data(), (int32_t)prims.size(), &a), ctx_,
          "skw_accel_create");
    h_ = Handle<skw_accel, skw_accel_destroy>(a);
  }

  // Closest hits of a host batch (TriangleAccelerator::Intersect).
  std::vector<skw_hit> Intersect(const std::vector<skw_ray> &rays) const {
    std::vector<skw_hit> hits(rays.size());
    check(skw_intersect_host(h_.get(), rays.data(), (int64_t)rays.size(), hits.data()), ctx_, "skw_intersect_host");
    return hits;
  }
  // Occlusion of a host batch within each ray's [tmin, tmax] (IntersectTest).
  std::vector<uint8_t> IntersectTest(const std::vector<skw_ray> &rays) const {
    std::vector<uint8_t> occ(rays.size());
    check(skw_intersect_test_host(h_.get(), rays.data(), (int64_t)rays.size(), occ.data()), ctx_,
          "skw_intersect_test_host");
    return occ;
  }
  // Device buffers, ordered on `stream` (a cudaStream_t, NULL = default).
  void Intersect(const skw_ray *d_rays, int64_t n, skw_hit *d_hits, void *stream) const {
    check(skw_intersect(h_.get(), d_rays, n, d_hits, stream), ctx_, "skw_intersect");
  }
  void IntersectTest(const skw_ray *d_rays, int64_t n, uint8_t *d_occluded, void *stream) const {
    check(skw_intersect_test(h_.get(), d_rays, n, d_occluded, stream), ctx_, "skw_intersect_test");
  }
  skw_accel_info Info() const {
    skw_accel_info i{};
    check(skw_accel_get_info(h_.get(), &i), ctx_, "skw_accel_get_info");
    return i;
  }
  skw_accel *get() const { return h_.get(); }

 private:
  skw_ctx *ctx_;
  Handle<skw_accel, skw_accel_destroy> h_;
};

// KDTree<Photon>: positions (xyz floats) and CompressedDirection ids of the
// photons' normals.  Lookup results index the tree order; Permutation()
// maps a tree position back to the input index.
class PhotonKDTree {
 public:
  PhotonKDTree(Context &ctx, const std::vector<float> &positions, const std::vector<uint16_t> &normal_ids)
      : ctx_(ctx.get()) {
    skw_kdtree *t = nullptr;
    check(skw_kdtree_create(ctx_, positions.data(), normal_ids.empty() ? nullptr : normal_ids.data(),
                            (int64_t)(positions.size() / 3), &t),
          ctx_, "skw_kdtree_create");
    h_ = Handle<skw_kdtree, skw_kdtree_destroy>(t);
  }

  struct Neighbours {
    int32_t k = 0;
    std::vector<int32_t> idx;    // k per query, the reference's heap order, -1 past count
    std::vector<double> d2;      // squared distances of idx
    std::vector<int32_t> count;  // points found per query
  };
  // GetNearestPoints(point, k, out, PhotonFilter(point, normal, cos), max_dist)
  // for every query (q, qn: xyz doubles); cos_threshold < 0: no filter.
  Neighbours GetNearestPoints(const std::vector<double> &q, const std::vector<double> &qn, int32_t k,
                              double max_dist, double cos_threshold) const {
    const int64_t nq = (int64_t)(q.size() / 3);
    Neighbours r;
    r.k = k;
    r.idx.resize((size_t)(nq * k));
    r.d2.resize((size_t)(nq * k));
    r.count.resize((size_t)nq);
    check(skw_knn_host(h_.get(), q.data(), qn.empty() ? nullptr : qn.data(), nq, k, max_dist, cos_threshold,
                       r.idx.data(), r.d2.data(), r.count.data()),
          ctx_, "skw_knn_host");
    return r;
  }
  std::vector<int32_t> Permutation() const {
    int64_t n = 0;
    check(skw_kdtree_size(h_.get(), &n), ctx_, "skw_kdtree_size");
    std::vector<int32_t> p((size_t)n);
    check(skw_kdtree_permutation(h_.get(), p.data()), ctx_, "skw_kdtree_permutation");
    return p;
  }
  skw_kdtree *get() const { return h_.get(); }

 private:
  skw_ctx *ctx_;
  Handle<skw_kdtree, skw_kdtree_destroy> h_;
};

// Scene with materials and lights, rendered by the direct-lighting
// integrator into a device film (height x width RGB floats).
class Scene {
 public:
  Scene(Context &ctx, const std::vector<Mesh> &meshes, const std::vector<skw_render_primitive> &prims,
        const std::vector<skw_material> &materials, const std::vector<skw_point_light> &point_lights)
      : ctx_(ctx.get()) {
    const std::vector<skw_mesh> mv = detail::mesh_views(meshes);
    skw_scene *s = nullptr;
    check(skw_scene_create(ctx_, mv.data(), (int32_t)mv.size(), prims.data(), (int32_t)prims.size(),
                           materials.data(), (int32_t)materials.size(), point_lights.data(),
                           (int32_t)point_lights.size(), &s),
          ctx_, "skw_scene_create");
    h_ = Handle<skw_scene, skw_scene_destroy>(s);
  }
  void SetMaxSpecularDepth(int32_t depth) {
    check(skw_scene_set_max_specular_depth(h_.get(), depth), ctx_, "skw_scene_set_max_specular_depth");
  }
  void SetMedium(const skw_medium *medium) { check(skw_scene_set_medium(h_.get(), medium), ctx_, "skw_scene_set_medium"); }
  void RenderDirect(const skw_camera &camera, const skw_render_params &params, float *d_film, void *stream) {
    check(skw_render_direct(h_.get(), &camera, &params, d_film, stream), ctx_, "skw_render_direct");
  }
  // The scene's accelerator (owned by the scene) and the differential
  // geometry of its closest hits (TriangleMesh::ComputeDifferentialGeometry);
  // device buffers.
  skw_accel *Accelerator() const { return skw_scene_accel(h_.get()); }
  void HitGeometry(const skw_ray *d_rays, const skw_hit *d_hits, int64_t n, skw_hit_geometry *d_out,
                   void *stream) const {
    check(skw_scene_hit_geometry(h_.get(), d_rays, d_hits, n, d_out, stream), ctx_, "skw_scene_hit_geometry");
  }
  skw_scene *get() const { return h_.get(); }
  skw_ctx *context() const { return ctx_; }

 private:
  skw_ctx *ctx_;
  Handle<skw_scene, skw_scene_destroy> h_;
};

// Photon maps of a scene: shot on the GPU (ShootPhotons) and rendered with
// caustic radiance and final gathering.
class PhotonMap {
 public:
  static PhotonMap Shoot(Scene &scene, const skw_photon_params &params) {
    skw_photon_map *m = nullptr;
    check(skw_photon_shoot(scene.get(), &params, &m), scene.context(), "skw_photon_shoot");
    return PhotonMap(scene.context(), m);
  }
  skw_photon_map_info Info() const {
    skw_photon_map_info i{};
    check(skw_photon_map_get_info(h_.get(), &i), ctx_, "skw_photon_map_get_info");
    return i;
  }
  void Render(Scene &scene, const skw_camera &camera, const skw_render_params &params,
              const skw_photon_render_params &photon_params, float *d_film, void *stream) const {
    check(skw_render_photon(scene.get(), h_.get(), &camera, &params, &photon_params, d_film, stream), ctx_,
          "skw_render_photon");
  }
  skw_photon_map *get() const { return h_.get(); }

 private:
  PhotonMap(skw_ctx *ctx, skw_photon_map *m) : ctx_(ctx), h_(m) {}
  skw_ctx *ctx_;
  Handle<skw_photon_map, skw_photon_map_destroy> h_;
};

}  // namespace skw

#endif  // SKW_HPP
