// Launch wrappers exported by the .cu translation units to the host layer.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>
#include <functional>

namespace skw {

// Smallest compiled traversal stack capacity that covers a tree of the given
// depth (root = 0): 2 * depth + 1 entries suffice for the ternary tree.
int traversal_stack_capacity(int max_depth);

// closest = true: hits is skw_hit[n] (int4); false: out is uint8_t[n].
// status: device word; bit 0 is set if a stack ever overflowed.
// scene_abs: the largest absolute coordinate of any vertex in the tree (it
// bounds the slab-test rounding error).
// out_index (may be null): result of ray j goes to slot out_index[j].
// n_dev (may be null): device int holding the number of rays to trace (at
// most n), for queues filled on the device.  out_index (may be null): the
// result of ray j goes to slot out_index[j].
// ctas_per_sm > 0 caps the persistent grid at that many CTAs per SM (0: as
// many as fit).  prepare_traversal computes the occupancy of a capacity's
// kernels ahead of a stream capture.
// surface: the rays leave surfaces with tmin from next_min_t (an upper bound
// of the reference's GetNextMinT); a triangle whose t cannot be told apart
// from tmin in float is then skipped (it lies on the ray's own plane
// crossing) instead of being decided in double.
cudaError_t launch_traversal(bool closest, int stack_cap, const void *nodes, const void *tris, const void *rays,
                             int64_t n, const int *n_dev, float scene_abs, const int32_t *out_index, void *out,
                             unsigned *status, cudaStream_t stream, int ctas_per_sm = 0, int *work = nullptr,
                             bool surface = false);
// work (may be null): a device int of the caller's, not used by any launch
// that may run at the same time; it is zeroed on `stream` and the warps
// then take groups of 32 rays from it as they finish (no idle tail).  Null:
// each warp traces a fixed share of the rays.
cudaError_t prepare_traversal(int stack_cap);
// Resident CTAs per SM of the closest-hit kernel at this capacity.
int traversal_max_ctas_per_sm(int stack_cap);
// An accelerator with instances registers its device tables (DevInst[],
// LeafExt[]) under its node array; traversal launches on that node array
// then run the exact instance-aware kernel.
void register_instances(const void *nodes, const void *inst, const void *ext);
void unregister_instances(const void *nodes);
// Every traversal launch on the accelerator whose device node array is
// `nodes` adds its ray count to *traced (a device counter).
void register_ray_counter(const void *nodes, unsigned long long *traced);
// Double rays (skw_ray_d, 64 bytes each): closest = true writes skw_hit_d
// (double t, prim, tri; t = +inf, ids -1 on a miss), false uint8_t per ray.
cudaError_t launch_traversal_d(bool closest, int stack_cap, const void *nodes, const void *tris, const void *rays,
                               int64_t n, float scene_abs, void *out, unsigned *status, cudaStream_t stream,
                               int *work);



// Photon kd-tree lookups (knn.cu).  nodes: KdNode[n]; nids: uint16 normal
// id per node; dirs: direction_table_device() (3 doubles per 16-bit
// direction id, then the same as 3 floats per id); q / qn: 3 doubles
// per query (qn may be null when cos_t < 0, which disables the filter).
// Outputs per query: k slots of tree positions and squared distances in the
// reference's heap order (-1 / 0 when unused) and the found count;
// out_visited (optional) counts visited nodes.  A non-zero knn_scratch_bytes(nq, k) (k > 128) means a scratch buffer of that
// many bytes is required.  status bit 1: stack overflow.
size_t knn_scratch_bytes(int64_t nq, int k);
// Exclusive scan of n 64-bit values in place (three launches); sums holds
// ceil(n / 256) values of scratch.
cudaError_t scan64(uint64_t *v, int64_t n, uint64_t *sums, cudaStream_t st);
cudaError_t launch_knn(const void *nodes, const uint16_t *nids, const double *dirs, int n, const double *q,
                       const double *qn, int64_t nq, int k, double max_dist, double cos_t, int32_t *out_idx,
                       double *out_d2, int32_t *out_count, int32_t *out_visited, void *scratch, unsigned *status,
                       cudaStream_t stream, const int *nq_dev = nullptr, const int32_t *order = nullptr);
// Spatial-bin order of n queries (3 doubles each; count_dev, if not null,
// caps n on the device) in the box [lo, hi]: order[t] = the query the t-th
// lookup thread takes (launch_knn / launch_nearest order), grouped by 64^3
// Morton cells.  keys: n uint32; bins: bin_order_bins() ints.
int64_t bin_order_bins();
cudaError_t launch_bin_order(const double *q, int64_t n, const int *count_dev, const float lo[3], const float hi[3],
                             uint32_t *keys, int *bins, int32_t *order, cudaStream_t st);
// The same cells as launch_bin_order, sorted stably (a radix sort of the
// cell keys): the queries of a cell keep their order.  scratch:
// sort_order_bytes(n).
size_t sort_order_bytes(int64_t n);
cudaError_t launch_sort_order(const double *q, int64_t n, const float lo[3], const float hi[3], void *scratch,
                              int32_t *order, cudaStream_t st);
// k-NN with its heaps in the library's static device scratch (no
// allocation): nq * k must be <= knn_noalloc_capacity() entries, else
// cudaErrorInvalidValue.  Overlapping calls race on that scratch.
int64_t knn_noalloc_capacity();
cudaError_t launch_knn_noalloc(const void *nodes, const uint16_t *nids, const double *dirs, int n, const double *q,
                               const double *qn, int64_t nq, int k, double max_dist, double cos_t,
                               int32_t *out_idx, double *out_d2, int32_t *out_count, unsigned *status,
                               cudaStream_t stream);
// Nearest accepted point per query (-1 if none within max_dist).
// nq_dev (launch_knn, launch_nearest; may be null): device int holding the
// number of queries to run (at most nq), for queues filled on the device.
// order (may be null): thread t answers query order[t] (a permutation of
// the queries that groups nearby ones into warps); results stay indexed by
// query.
cudaError_t launch_nearest(const void *nodes, const uint16_t *nids, const double *dirs, int n, const double *q,
                           const double *qn, int64_t nq, double max_dist, double cos_t, int32_t *out_idx,
                           unsigned *status, cudaStream_t stream, const int *nq_dev = nullptr,
                           const int32_t *order = nullptr);

// Direct-lighting render stages (render.cu); see render_scene.h.
// A pass covers global pixels [px_begin, px_begin + n_px) of the views'
// concatenated films, every pixel with spp samples.
struct SceneDev;
struct ViewDev;
// Point, normals, barycentrics and t of closest hits (12 doubles each).
cudaError_t launch_hit_geometry(const SceneDev &S, const void *rays, const void *hits, int64_t n, double *out,
                                cudaStream_t s);
// The whole Intersection (36 doubles each, skw_intersection) of double ray
// differentials (21 doubles each, skw_ray_differential) and their
// skw_hit_d hits.
cudaError_t launch_intersection(const SceneDev &S, const void *rays, const void *hits, int64_t n, double *out,
                                cudaStream_t s);
// Outgoing rays of closest hits (float rays, skw_hit) in directions dirs.
cudaError_t launch_next_rays(const SceneDev &S, const void *rays, const void *hits, const float *dirs, int64_t n,
                             void *out, cudaStream_t s);
// ld: LDSampler image points (sppx = samples per pixel, a power of two; sppy = 1)
cudaError_t launch_camera(const ViewDev *views, int n_views, int64_t px_begin, int n_px, int sppx, int sppy,
                          void *rays, cudaStream_t s, int ld = 0);
// Queues of one specular level (render.cu, SpecArgs): the input level's
// rays / weights / camera samples / tree nodes / count and the next level's.
struct SpecQueues {
  const void *in_rays;
  const float *in_w;
  const int *in_sample, *in_node, *in_count;
  void *out_rays;
  float *out_w;
  int *out_sample, *out_node, *out_count;
  int spec_slot;
};
// spec (may be null): queue the specular children of the camera hits into
// spec->out_* (the scene's max_spec_depth >= 0 and some material is
// specular).
cudaError_t launch_shade(const SceneDev &S, const ViewDev *views, int n_views, int n, int64_t px_begin, int spp,
                         int slots, int n_light_samples, const void *rays, const void *hits, float *contrib,
                         void *srays, int *starget, float *srgb, int *scount, void *brays, int *btarget, float *brgb,
                         int *bcount, float *bnrm, int block, cudaStream_t s, const SpecQueues *spec = nullptr,
                         int ld = 0);
// One specular level: shades entries [0, min(*spec.in_count, capacity)) of
// spec.in_* (hits: their closest hits) at specular depth `depth`, adding
// weight x (emission + direct lighting) into each entry's sample slot
// spec.spec_slot through the shadow / BSDF queues, and queues the children.
cudaError_t launch_shade_specular(const SceneDev &S, const ViewDev *views, int n_views, int64_t capacity,
                                  int64_t px_begin, int spp, int slots, int n_light_samples, const SpecQueues &spec,
                                  int depth, const void *hits, float *contrib, void *srays, int *starget, float *srgb,
                                  int *scount, void *brays, int *btarget, float *brgb, int *bcount, float *bnrm,
                                  cudaStream_t s);
// bnrm: per BSDF-queue entry, the shading normal turned to the viewer (the
// light-choice density of the light a BSDF ray hits depends on it).
// accumulate: add into the target slots (specular levels) instead of storing.
cudaError_t launch_resolve(const SceneDev &S, int capacity, int n_light_samples, const uint8_t *occ,
                           const int *starget, const float *srgb, const int *scount, const void *brays,
                           const void *bhits, const int *btarget, const float *brgb, const int *bcount,
                           const float *bnrm, float *contrib, cudaStream_t s, bool accumulate = false);
// tcam (may be null): per-sample transmittance of the camera ray's medium
// segment; with it, slot media_slot is the medium's radiance and the others
// are scaled by the transmittance.
cudaError_t launch_film(const float *contrib, int64_t px_begin, int n_px, int spp, int slots, float *film,
                        cudaStream_t s, const float *tcam = nullptr, int media_slot = 0);
// Homogeneous medium along the camera rays (render.cu, k_media): writes tcam
// and the medium emission slot, queues one light sample per march step
// (mrays / mtarget / mval; adjoint: mdem = dI . d(value)/d(emission scale)).
// status bit 2: a ray needed more than the medium's max_steps.
cudaError_t launch_media(bool adjoint, const SceneDev &S, const ViewDev *views, int n_views, int n, int64_t px_begin,
                         int spp, int slots, int media_slot, const float *dfilm, const void *rays, const void *hits,
                         float *contrib, float *tcam, void *mrays, int *mtarget, float *mval, float *mdem,
                         int *mcount, unsigned *status, cudaStream_t s);
// A chunk of a specular level counted on the device: entries
// [*off_dev, *off_dev + n) of the level, clipped to min(*count_dev,
// capacity).  All null / 0: the n entries the pointers start at.
struct MediaChunk {
  const int *off_dev = nullptr;
  const int *count_dev = nullptr;
  int64_t capacity = 0;
};
// The medium along n entries of a specular level (rays, hits, in_sample,
// in_w, in_node point at the first, or at the level's start for a
// device-counted chunk): in_w is multiplied by each segment's
// transmittance, emission and queued light samples target the entry's
// sample's slot spec_slot (mtarget holds full slot indices: resolve with
// slots = 1, media_slot = 0).  adjoint: mdem receives each queued light
// sample's emission-scale derivative (dfilm = dL/dI, scaled by the sample's
// camera-segment transmittance tcam) and nothing is added to contrib.
cudaError_t launch_media_specular(bool adjoint, const SceneDev &S, const ViewDev *views, int n_views, int n,
                                  int64_t px_begin, int spp, int slots, int spec_slot, const void *rays,
                                  const void *hits, const int *in_sample, float *in_w, const int *in_node,
                                  const MediaChunk &chunk, const float *dfilm, const float *tcam, float *contrib,
                                  void *mrays, int *mtarget, float *mval, float *mdem, int *mcount,
                                  unsigned *status, cudaStream_t s);
// Ends one iteration of a graph's device-counted chunk loop: *off += chunk,
// and the loop's conditional set to whether *off < min(*count, capacity).
cudaError_t launch_media_advance(cudaGraphConditionalHandle h, int *off, const int *count, int chunk,
                                 int64_t capacity, cudaStream_t s);
cudaError_t launch_resolve_media(bool adjoint, int64_t capacity, const uint8_t *occ, const int *mtarget,
                                 const float *mval, const float *mdem, const int *mcount, int slots, int media_slot,
                                 float *contrib, double *g_emission, cudaStream_t s);
// Adjoint of one pass (render.cu): replays the pass's rays and accumulates
// dL/d(triangle albedo) (3 floats per global triangle) and dL/d(emission
// scale) from dfilm = dL/dI (3 floats per global pixel).
cudaError_t launch_shade_adjoint(const SceneDev &S, const ViewDev *views, int n_views, int n, int64_t px_begin, int spp,
                                 int n_light_samples, const float *dfilm, float *g_albedo, double *g_emission,
                                 const void *rays, const void *hits, void *srays, int *stri, float *s_dkd,
                                 float *s_dem, int *scount, void *brays, int *btri, float *b_dkd, float *brgb,
                                 int *bcount, float *bnrm, const float *tcam, cudaStream_t s, int ld = 0,
                                 const SpecQueues *spec = nullptr);
// Adjoint of one specular level (the entries' weights multiply dL/dI).
cudaError_t launch_shade_specular_adjoint(const SceneDev &S, const ViewDev *views, int n_views, int64_t capacity,
                                          int64_t px_begin, int spp, int n_light_samples, const float *dfilm,
                                          float *g_albedo, double *g_emission, const SpecQueues &spec, int depth,
                                          const void *hits, void *srays, int *stri, float *s_dkd, float *s_dem,
                                          int *scount, void *brays, int *btri, float *b_dkd, float *brgb,
                                          int *bcount, float *bnrm, cudaStream_t s,
                                          const float *tcam = nullptr);
cudaError_t launch_resolve_adjoint(const SceneDev &S, int capacity, int n_light_samples, const uint8_t *occ,
                                   const int *stri, const float *s_dkd, const float *s_dem, const int *scount,
                                   const void *brays, const void *bhits, const int *btri, const float *b_dkd,
                                   const float *brgb, const int *bcount, const float *bnrm, float *g_albedo,
                                   double *g_emission, cudaStream_t s, bool capped = false);

// Photon mapping (photon.cu).  trace(rays, n, n_dev, hits, stream) runs the
// closest-hit traversal of the scene's accelerator.
struct PhotonRec;
struct PhotonShootArgs;
using TraceFn = std::function<cudaError_t(const void *, int64_t, const int *, void *, cudaStream_t, int *)>;
// Workspace bytes of one shooting chunk of n_paths paths with `slots`
// indirect-photon slots per path.
size_t photon_chunk_bytes(int64_t n_paths, int slots);
// Shoots paths [path0, path0 + n_paths): writes the chunk's direct photons
// (at most n_paths), indirect photons (at most n_paths * A.slots)
// and caustic photons (at most n_paths) in path order, and their counts to
// d_totals[0], d_totals[1], d_totals[2].
cudaError_t photon_shoot_chunk(const SceneDev &S, const PhotonShootArgs &A, const TraceFn &trace, int64_t path0,
                               int n_paths, void *ws, PhotonRec *out_direct, PhotonRec *out_indirect,
                               PhotonRec *out_caustic, int *d_totals, cudaStream_t st);
// Irradiance estimate of nq points from one map's k-NN output (see
// k_irradiance_sum); first = this is the first map added.
cudaError_t launch_irradiance_sum(const void *nodes, const float *weight, const uint16_t *dirid, const double *dirs,
                                  const double *q, const double *qn, const int32_t *idx, const int32_t *count,
                                  int64_t nq, int k, double paths, double max_lookup_dist, bool first, float *ext,
                                  float *intr, cudaStream_t st);

// Caustic radiance of a render pass (photon.cu): the filtered k-NN in the
// caustic map at each camera hit and the Simpson-kernel estimate, written to
// slot `slot` of contrib.  cws: caustic_bytes(n, k) bytes of workspace.
struct CausticMap;
// Entries of a specular level as the shading points of the caustic and
// gather stages: entry e belongs to camera sample in_sample[e], carries the
// RGB weight in_w[3e..] and tree node in_node[e] (its random stream), and
// its weighted terms are added (atomics) into that sample's slot `slot`.
// Null: the shading points are the pass's camera hits, one per sample.
struct SpecSource {
  const int *in_sample = nullptr;
  const float *in_w = nullptr;
  const int *in_node = nullptr;
  int slot = 0;
};
size_t caustic_bytes(int64_t n, int k);
cudaError_t launch_caustic(const SceneDev &S, const CausticMap &C, const ViewDev *views, int n_views, int n,
                           int64_t px_begin, int spp, int slots, int slot, const void *rays, const void *hits,
                           void *cws, float *contrib, unsigned *status, cudaStream_t st,
                           const SpecSource *sp = nullptr);

// Final gather of a render pass (photon.cu): adds each camera hit's gathered
// indirect radiance to its slots [base_slot, base_slot + 2 gs) of contrib.
// gws: gather_bytes(n, gs) bytes of workspace.
struct GatherMaps;
size_t gather_bytes(int64_t n, int gs);
cudaError_t launch_gather(const SceneDev &S, const GatherMaps &M, const ViewDev *views, int n_views, int n,
                          int64_t px_begin, int spp, int slots, int base_slot, int gs, const void *rays,
                          const void *hits, void *gws, float *contrib, const TraceFn &trace, unsigned *status,
                          cudaStream_t st, const SpecSource *sp = nullptr);

}  // namespace skw
