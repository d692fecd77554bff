/*
 * skw.h -- C ABI of the GB300 ray-query and light-transport library.
 *
 * Plain pointers, sizes and status codes only; no C++ or torch types.  Every
 * entry point names the reference interface it stands in for (paths are in
 * the Skwarka source tree).  All functions return SKW_OK (0) on success or a
 * nonzero skw_status; skw_last_error() gives a one-line message for the last
 * failure on a context.
 *
 * Threading: a context and the handles made from it may be used from one
 * host thread at a time.  Work is stream-ordered on the caller's CUDA stream
 * (a cudaStream_t passed as void*, NULL = the legacy default stream).
 *
 * Memory: "device" buffers are caller-owned device (or managed) memory on
 * the context's device; "_host" variants take caller-owned host memory and
 * do the copies themselves.  Handles own their device memory and free it in
 * *_destroy.
 */
#ifndef SKW_H
#define SKW_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum skw_status {
  SKW_OK = 0,
  SKW_ERR_ARG = 1,            /* invalid argument (null pointer, bad size, bad index) */
  SKW_ERR_CUDA = 2,           /* a CUDA runtime call failed */
  SKW_ERR_OOM = 3,            /* device or host allocation failed */
  SKW_ERR_BUDGET = 4,         /* a device loop hit its iteration budget */
  SKW_ERR_STACK_OVERFLOW = 5, /* traversal stack capacity exceeded */
  SKW_ERR_UNSUPPORTED = 6,    /* valid input outside what this build implements */
  SKW_ERR_NO_DEVICE = 7       /* no usable CUDA device */
} skw_status;

typedef struct skw_ctx skw_ctx;
typedef struct skw_accel skw_accel;
typedef struct skw_kdtree skw_kdtree;
typedef struct skw_scene skw_scene;

/* ------------------------------------------------------------ context -- */

/* Binds a context to a CUDA device (the one the caller's streams use). */
int skw_ctx_create(int device, skw_ctx **out);
void skw_ctx_destroy(skw_ctx *ctx);
/* Message of the last failure on this context ("" if none). */
const char *skw_last_error(const skw_ctx *ctx);
/* Library version (major * 10000 + minor * 100 + patch). */
int skw_version(void);

/* ------------------------------------------------- triangle accelerator -- */

/* A triangle mesh: float xyz per vertex, int32 vertex-index triples.
 * Mirrors TriangleMesh(vertices, triangles) (Raytracer/Core/TriangleMesh.h:82):
 * triangles with an out-of-range or repeated vertex index are dropped the
 * same way (TriangleMesh.cpp:176-182), shifting later mesh triangle indices. */
typedef struct skw_mesh {
  const float *vertices;
  int64_t n_vertices;
  const int32_t *triangles;
  int64_t n_triangles;
} skw_mesh;

/* A primitive: a mesh placed by a row-major 4x4 mesh-to-world matrix (NULL =
 * identity).  Mirrors Primitive(mesh, transform, ...) (Raytracer/Core/Primitive.h:48). */
typedef struct skw_primitive {
  int32_t mesh;
  const double *mesh_to_world;
} skw_primitive;

/* Ray: origin, direction (normalised), [tmin, tmax].  32 bytes.  Stands in
 * for Ray (Math/Ray.h:57-59) with float components widened exactly. */
typedef struct skw_ray {
  float ox, oy, oz;
  float dx, dy, dz;
  float tmin, tmax;
} skw_ray;

/* Closest-hit result.  prim = primitive index, tri = triangle index within
 * that primitive's mesh (the reference's Intersection::mp_primitive and
 * m_triangle_index), t = ray parameter; prim = tri = -1 and t = +inf on a
 * miss.  flags: SKW_HIT_* bits.  16 bytes. */
typedef struct skw_hit {
  float t;
  int32_t prim;
  int32_t tri;
  uint32_t flags;
} skw_hit;

/* The hit was decided by the exact double-precision re-test (a grazing hit,
 * a hit near a triangle edge, or a near-tie in t between two triangles). */
#define SKW_HIT_FP64_DECIDED 1u
/* Two candidate triangles had double-precision t within 1e-12 relative. */
#define SKW_HIT_NEAR_TIE 2u
/* The hit was decided in float but its t was recomputed exactly (grazing
 * incidence, where the float t's error bound exceeds 5e-6 relative). */
#define SKW_HIT_T_REFINED 4u

typedef struct skw_accel_info {
  int64_t n_triangles;
  int64_t n_nodes;
  int64_t n_leaves;
  int32_t max_depth;   /* deepest node (root = 0) */
  int32_t stack_need;  /* traversal stack entries that suffice: 2*max_depth+1 */
  float bounds[6];     /* world bounds: min xyz, max xyz (GetWorldBounds) */
  double build_ms;     /* build time (wall clock) */
  int64_t device_bytes;
  int32_t built_on_device; /* 1: the tree was built on the GPU */
} skw_accel_info;

/* Host-only build of the ternary bbox kd-tree over all primitives (the same
 * splits, partitions and leaf rule as TriangleAccelerator::TriangleAccelerator,
 * Raytracer/Core/TriangleAccelerator.cpp:22-147, 505-729), flattened into the
 * device layout.  Needs no GPU.  threads <= 0 uses all hardware threads.
 * A mesh used by several primitives is instanced as the reference does it
 * (TriangleAccelerator.cpp:54-102): one subtree over its mesh-space
 * triangles, and per primitive an instance (its world box, its primitive's
 * world-to-mesh matrix) placed in the tree like a triangle; queries on such
 * an accelerator run an exact double-precision traversal that takes rays
 * into each instance's mesh space (TriangleAccelerator.cpp:213-233).
 * On failure a message is written to err (if errlen > 0). */
typedef struct skw_flat_tree skw_flat_tree;
int skw_flat_tree_build(const skw_mesh *meshes, int32_t n_meshes, const skw_primitive *prims, int32_t n_prims,
                        int threads, skw_flat_tree **out, char *err, size_t errlen);
void skw_flat_tree_destroy(skw_flat_tree *tree);
/* skw_flat_tree_build with the tree built on the context's GPU: node for
 * node the same tree (the split search's float and double arithmetic and
 * the partition's element order reproduced exactly).  Accelerators with
 * instancing, or of fewer than min_device_triangles triangles, are built on
 * the host; *on_device (optional) is 1 when the GPU built it.  Errors are
 * the context's (skw_last_error). */
int skw_flat_tree_build_device(skw_ctx *ctx, const skw_mesh *meshes, int32_t n_meshes, const skw_primitive *prims,
                               int32_t n_prims, int64_t min_device_triangles, skw_flat_tree **out,
                               int32_t *on_device);
/* n_nodes, n_triangles, max_depth (root = 0) of a flat tree. */
int skw_flat_tree_sizes(const skw_flat_tree *tree, int64_t *n_nodes, int64_t *n_triangles, int32_t *max_depth);
/* Copies out nodes (8 x 32-bit words each, see skw_accel_export), triangle
 * slots (9 floats: v0 v1 v2 in world space) and their (primitive, mesh
 * triangle) ids.  Any pointer may be NULL. */
int skw_flat_tree_export(const skw_flat_tree *tree, uint32_t *nodes, float *tris, int32_t *tri_prim,
                         int32_t *tri_index);

/* Instances of a flat tree, in the tree's final order: per instance its
 * primitive, the node index of its mesh's subtree root and its
 * world-to-mesh matrix (16 doubles, row-major: the inverse of the
 * primitive's mesh-to-world matrix as Matrix4x4::Inverted computes it,
 * Math/Matrix4x4.h:240-316); and the subtree roots (one per shared mesh, in
 * mesh order; the tree's own root is node 0).  Any output may be NULL.
 * A leaf holding instances has bit 7 set in its word 7, and its word 6
 * indexes a table read by skw_flat_tree_leaf_ranges: its triangle-slot
 * range (first, count) and instance range (first, count). */
int skw_flat_tree_instances(const skw_flat_tree *tree, int64_t *n_instances, int32_t *prim, uint32_t *subtree_root,
                            double *world_to_mesh, int64_t *n_subtrees, uint32_t *subtree_roots);
int skw_flat_tree_leaf_ranges(const skw_flat_tree *tree, uint32_t leaf_word6, uint32_t *out4);

/* Uploads a flat tree to the context's device (the tree stays owned by the
 * caller).  Together with skw_flat_tree_build this is
 * TriangleAccelerator::TriangleAccelerator. */
int skw_accel_create_from_flat(skw_ctx *ctx, const skw_flat_tree *tree, skw_accel **out);

/* skw_flat_tree_build_device (trees of 16,384 triangles or more on the GPU)
 * + skw_accel_create_from_flat. */
int skw_accel_create(skw_ctx *ctx, const skw_mesh *meshes, int32_t n_meshes, const skw_primitive *prims,
                     int32_t n_prims, skw_accel **out);
void skw_accel_destroy(skw_accel *accel);
int skw_accel_get_info(const skw_accel *accel, skw_accel_info *info);
/* Rays traced so far by every query, render and photon launch on this
 * accelerator (queue lengths as the device saw them); waits for the device.
 * A statistic of this library: the reference keeps none. */
int skw_accel_rays_traced(const skw_accel *accel, uint64_t *out);

/* Copies out the flattened tree for inspection: nodes as 8 x 32-bit words
 * (min xyz, max xyz as float bits; word 6: first child / first triangle;
 * word 7: type and child mask / triangle count), and per triangle slot its
 * (primitive, mesh triangle) ids.  Any pointer may be NULL. */
int skw_accel_export(const skw_accel *accel, uint32_t *nodes, int32_t *tri_prim, int32_t *tri_index);

/* Closest hit for n rays, device buffers.  Stands in for
 * TriangleAccelerator::Intersect / Scene::Intersect
 * (Raytracer/Core/TriangleAccelerator.cpp:295-352, Scene.h:77-85) without the
 * differential-geometry step (skw_scene_hit_geometry does that part).  Each
 * call takes a 256-byte work counter from the context's stream-ordered
 * pool (allocated and freed on `stream`), so calls on different streams
 * may run at the same time. */
int skw_intersect(skw_accel *accel, const skw_ray *rays, int64_t n, skw_hit *hits, void *stream);

/* Any hit in [tmin, tmax] for n rays, device buffers; occluded[i] = 0 or 1.
 * Stands in for TriangleAccelerator::IntersectTest / Scene::IntersectTest
 * (Raytracer/Core/TriangleAccelerator.cpp:354-468, Scene.h:140-148). */
int skw_intersect_test(skw_accel *accel, const skw_ray *rays, int64_t n, uint8_t *occluded, void *stream);

/* Same as above with host buffers (pinned or pageable), waiting for
 * completion.  Page-locked buffers (cudaHostAlloc, cudaHostRegister) on a
 * device with a coherent link to the host (NVLink-C2C:
 * skw_ctx_host_buffers_in_place) are read and written in place by the
 * traversal; otherwise the rays are copied in and the results out in 2M-ray
 * chunks on two streams, overlapped with the traversals. */
int skw_intersect_host(skw_accel *accel, const skw_ray *rays, int64_t n, skw_hit *hits);
int skw_intersect_test_host(skw_accel *accel, const skw_ray *rays, int64_t n, uint8_t *occluded);

/* A ray in double precision, the reference's Ray (Math/Ray.h:57-59): origin,
 * direction (normalised), [tmin, tmax].  64 bytes. */
typedef struct skw_ray_d {
  double ox, oy, oz;
  double dx, dy, dz;
  double tmin, tmax;
} skw_ray_d;

/* Closest hit of a double ray: t is the reference's exact double t (the
 * o_t of TriangleAccelerator::Intersect); t = +inf and prim = tri = -1 on a
 * miss.  16 bytes. */
typedef struct skw_hit_d {
  double t;
  int32_t prim;
  int32_t tri;
} skw_hit_d;

/* Closest / any hit of double rays, device buffers: Scene::Intersect /
 * IntersectTest on the reference's own ray type (TriangleAccelerator.cpp:
 * 154-352, 354-468).  Nodes are culled in float with bounds that cover the
 * rounding of the ray to float, so a node is skipped only if the reference
 * skips it; every triangle of a reached leaf is tested with the reference's
 * double Moller-Trumbore on the double ray, so the hit ids and t are the
 * reference's, bit for bit.  Slower than the float entry points (every
 * triangle test runs in double). */
int skw_intersect_d(skw_accel *accel, const skw_ray_d *rays, int64_t n, skw_hit_d *hits, void *stream);
int skw_intersect_test_d(skw_accel *accel, const skw_ray_d *rays, int64_t n, uint8_t *occluded, void *stream);
/* The same with host buffers; waits for completion. */
int skw_intersect_d_host(skw_accel *accel, const skw_ray_d *rays, int64_t n, skw_hit_d *hits);
int skw_intersect_test_d_host(skw_accel *accel, const skw_ray_d *rays, int64_t n, uint8_t *occluded);

/* Kernel launches made by this library since the context was created. */
int64_t skw_launch_count(const skw_ctx *ctx);
/* 1 when the context's device reaches host memory over a coherent link
 * (native atomics across it, as NVLink-C2C on a Grace system): the
 * host-buffer queries then work on page-locked buffers in place; else 0. */
int skw_ctx_host_buffers_in_place(const skw_ctx *ctx);

/* ---------------------------------------------------- photon kd-tree -- */

/* 16-bit direction codec of the reference's CompressedDirection
 * (Math/CompressedDirection.h:107-133, CompressedDirection.cpp:21-41):
 * encode a unit vector, and the decoded unit vector of every id (3 doubles
 * per id, 65536 ids). */
uint16_t skw_compress_direction(double x, double y, double z);
int skw_direction_table(double *out);

/* Host-only build of the photon kd-tree (KDTree<T>::KDTree / _Build,
 * Raytracer/Core/KDTree.h:396-473): perm[i] = input index of the point at
 * tree position i; node_words: 2 words per node, the reference's
 * (split coordinate as float bits, right-child/flags word).  Needs no GPU.
 * Either output may be NULL. */
int skw_kdtree_build_host(const float *positions, int64_t n, int threads, int32_t *perm, uint32_t *node_words);
/* The same tree built on the GPU (level by level over per-axis sorted
 * lists), same outputs as skw_kdtree_build_host.  *median_tie = the number
 * of nodes whose median ties on its split axis: below such a node the
 * reference's tree is std::nth_element's choice among the equal points, so
 * those subtrees and the paths to them are remade on the host from the
 * input order (skw_kdtree_repair_host); above 256 of them the whole tree is
 * built on the host.  Host buffers. */
/* The host half of skw_kdtree_build_device: perm / node_words (in/out) hold
 * a tree equal to the reference's except below the tie nodes at tree
 * positions ties[0..n_ties) (all of them); remakes the paths from the root
 * to those nodes and their subtrees as KDTree::_Build makes them, leaving
 * every other subtree as it is.  Needs no GPU. */
int skw_kdtree_repair_host(const float *positions, int64_t n, const int32_t *ties, int64_t n_ties, int32_t *perm,
                           uint32_t *node_words);
int skw_kdtree_build_device(skw_ctx *ctx, const float *positions, int64_t n, int32_t *perm, uint32_t *node_words,
                            int32_t *median_tie);

/* Builds the tree -- on the GPU for 16,384 or more photons when no node's
 * median ties on its split axis, else on the host; the same tree either way
 * -- and keeps it on the device.  positions: float xyz per
 * photon; normal_ids: the photons' 16-bit surface-normal ids (NULL = all 0),
 * used by the filtered lookups.  Lookup results index the TREE order
 * (skw_kdtree_permutation maps them back to input order), as the
 * reference's pointers index its permuted point array. */
int skw_kdtree_create(skw_ctx *ctx, const float *positions, const uint16_t *normal_ids, int64_t n,
                      skw_kdtree **out);
void skw_kdtree_destroy(skw_kdtree *tree);
int skw_kdtree_size(const skw_kdtree *tree, int64_t *n);
int skw_kdtree_permutation(const skw_kdtree *tree, int32_t *perm);

/* k nearest photons within max_dist for nq queries, device buffers.
 * Stands in for KDTree::GetNearestPoints (Raytracer/Core/KDTree.h:506-533)
 * with PhotonFilter (LTEIntegrators/PhotonLTEIntegrator/PhotonInternalTypes.h:
 * 113-137) when cos_threshold >= 0 (query normals qn required), unfiltered
 * when cos_threshold < 0 (qn may be NULL).  q, qn: 3 doubles per query.
 * Per query: out_count = points found (<= k); out_idx / out_d2: k slots in
 * the reference's heap order, -1 / 0 past out_count.  The index sets and
 * their order equal the reference's bit for bit.  Batches of 65,536 or
 * more queries are walked in spatial order (the queries sorted by a 64^3
 * cell of the tree's bounding box, stably, so a cell keeps the caller's
 * order): each result still lands in its own query's slots, the same as in
 * any order.  Workspace from the context's stream-ordered pool: the sort's
 * (18 bytes per query) for such batches, and the heaps' for k > 128
 * (up to 4096). */
int skw_knn(skw_kdtree *tree, const double *q, const double *qn, int64_t nq, int32_t k, double max_dist,
            double cos_threshold, int32_t *out_idx, double *out_d2, int32_t *out_count, void *stream);
/* skw_knn without any allocation, for callers that cannot allocate device
 * memory at query time: a renderer that reserves its whole device budget up
 * front and forbids allocations inside a frame, or a host callback that must
 * not block or synchronise the device the way cudaMalloc / cudaFree can.
 * This entry point has no counterpart in the reference (which allocates its
 * per-thread heaps from a host memory pool).
 *
 * The heaps live in one static device array of 1,048,576 entries (16 MiB)
 * that every GPU loading this library holds until the process exits; a call
 * needs nq * k <= 1,048,576 and returns SKW_ERR_ARG (with a message) beyond
 * that.  Results are identical to skw_knn.  The first call on a device looks
 * the array's device address up (cudaGetSymbolAddress), which can load the
 * library's device code; make that first call before any stream capture.
 * The address is looked up again when the device's current context has
 * changed since (a cudaDeviceReset destroys the array's module; every
 * handle made before a reset is invalid anyway).
 * All calls share the array, and it keeps the previous call's contents:
 * every heap slot is written before it is read, so nothing needs clearing,
 * but calls that overlap on the GPU (different streams or contexts) race on
 * it and must be serialised by the caller.  Device buffers only. */
int skw_knn_noalloc(skw_kdtree *tree, const double *q, const double *qn, int64_t nq, int32_t k, double max_dist,
                    double cos_threshold, int32_t *out_idx, double *out_d2, int32_t *out_count, void *stream);

/* Same with host buffers; waits for completion. */
int skw_knn_host(skw_kdtree *tree, const double *q, const double *qn, int64_t nq, int32_t k, double max_dist,
                 double cos_threshold, int32_t *out_idx, double *out_d2, int32_t *out_count);

/* Nearest accepted photon per query (-1 if none within max_dist), device
 * buffers.  Stands in for KDTree::GetNearestPoint (KDTree.h:485-503); the
 * filter applies as in skw_knn. */
int skw_nearest(skw_kdtree *tree, const double *q, const double *qn, int64_t nq, double max_dist,
                double cos_threshold, int32_t *out_idx, void *stream);

/* ------------------------------------------------ direct-lighting render -- */

/* Material kinds (Raytracer/Materials): */
#define SKW_MATERIAL_MATTE 0   /* MatteMaterial: Lambertian (sigma == 0) or Oren-Nayar */
#define SKW_MATERIAL_PLASTIC 1 /* PlasticMaterial: Lambertian(kd) + Blinn microfacet(ks, 1/roughness), dielectric 1.5 */
#define SKW_MATERIAL_METAL 2   /* MetalMaterial: Blinn microfacet with a conductor Fresnel (eta, k) */
#define SKW_MATERIAL_MEASURED 3 /* MERLMeasuredMaterial: a tabulated BRDF (skw_merl) */
/* TransparentMaterial (Raytracer/Materials/TransparentMaterial.cpp:29-55):
 * SpecularReflection(kd, FresnelDielectric(refractive_index, 1)) +
 * SpecularTransmission(ks, refractive_index, 1); kd / ks black = component absent. */
#define SKW_MATERIAL_TRANSPARENT 4
/* SubstrateMaterial (Raytracer/Materials/SubstrateMaterial.cpp:42-72):
 * with v_roughness <= 0 the one-roughness form, FresnelBlend<BlinnDistribution>
 * (kd, ks) with exponent 1 / clamp(roughness, 0.001, 1); with v_roughness > 0
 * the two-roughness form, FresnelBlend<AnisotropicDistribution> (Ashikhmin
 * and Shirley) with exponents 1 / clamp(roughness) along the shading tangent
 * and 1 / clamp(v_roughness) across it; kd, ks clamped to [0, 1]. */
#define SKW_MATERIAL_SUBSTRATE 5
/* UberMaterial (Raytracer/Materials/UberMaterial.cpp:39-85): with op =
 * clamp(opacity, 0, 1): SpecularTransmission(1 - op, refractive_index) when
 * some channel of op is outside [0.99, 1.01], Lambertian(clamp(op kd)),
 * Microfacet(clamp(op ks), FresnelDielectric(refractive_index, 1),
 * Blinn(1 / roughness)), SpecularReflection(clamp(kr), the same Fresnel);
 * black weights leave their component out.  opacity (1, 1, 1) is opaque. */
#define SKW_MATERIAL_UBER 6
/* MixMaterial (Raytracer/Materials/MixMaterial.cpp:29-57): the components of
 * materials mix[0] and mix[1] (indices into the same array; mix[1] = -1:
 * none) scaled by clamp(mix_scale, 0, 1) and 1 - that.  Neither may itself
 * be a mix, and at most one of them may have specular components
 * (SKW_ERR_UNSUPPORTED otherwise). */
#define SKW_MATERIAL_MIX 7

typedef struct skw_merl skw_merl;

typedef struct skw_material {
  int32_t kind;
  float kd[3];        /* matte reflectance, plastic diffuse reflectance */
  float ks[3];        /* plastic glossy reflectance */
  float roughness;    /* plastic / metal, clamped to [0.001, 1] like the reference */
  float sigma;        /* matte Oren-Nayar sigma (radians); 0 = Lambertian */
  float eta[3], k[3]; /* metal refractive index and absorption */
  const skw_merl *measured; /* SKW_MATERIAL_MEASURED: the tabulated BRDF (must outlive the scene) */
  float refractive_index;   /* SKW_MATERIAL_TRANSPARENT, _UBER: index inside (outside 1), > 0 */
  float kr[3];              /* SKW_MATERIAL_UBER: specular reflectance */
  float opacity[3];         /* SKW_MATERIAL_UBER: opacity (1: opaque) */
  int32_t mix[2];           /* SKW_MATERIAL_MIX: the two materials */
  float mix_scale[3];       /* SKW_MATERIAL_MIX: the first material's scale */
  float v_roughness;        /* SKW_MATERIAL_SUBSTRATE: > 0 selects the two-roughness form */
} skw_material;

/* A measured BRDF in the MERL binary layout (MERLMeasuredData(std::istream&),
 * Raytracer/BxDFs/MERLMeasured.cpp:169-217): 3 int32 dimensions (90, 90,
 * 180), then 3 channels of 1,458,000 doubles, scaled by 1/1500, 1.15/1500 and
 * 1.66/1500, converted RGB -> XYZ -> spectrum coefficients and stored in half
 * precision as the reference stores them; the sampling segmentations
 * (_InitializeSegmentations, :219-251) are built on the host. */
int skw_merl_create(skw_ctx *ctx, const void *bytes, int64_t n_bytes, skw_merl **out);
/* (ctx = NULL: host tables only -- the host entry points work, a scene
 * cannot use it.) */
void skw_merl_destroy(skw_merl *merl);
/* The converted half table (3 uint16 per entry) and the segmentations (90 x
 * 1,173 floats: 24 x 45 column CDFs, 24 row CDFs, 45 + 24 grid lines). */
int skw_merl_export(const skw_merl *merl, uint16_t *table, float *segmentation);
/* MERLMeasured::Evaluate / PDF / Sample (local frame, double, host) for n
 * directions: the reference's arithmetic, for checking. */
int skw_merl_eval_host(const skw_merl *merl, const double *wi, const double *wo, int64_t n, double *f, double *pdf);
int skw_merl_sample_host(const skw_merl *merl, const double *wi, const double *u, int64_t n, double *wo, double *f,
                         double *pdf);

/* A primitive of the render scene: mesh + transform as for the accelerator,
 * plus its material, optional area-light emission and shading normals. */
typedef struct skw_render_primitive {
  int32_t mesh;
  const double *mesh_to_world;   /* row-major 4x4 or NULL (area lights must use NULL) */
  int32_t material;              /* index into the materials array */
  const float *vertex_normals;   /* per-vertex shading normals (mesh space) or NULL:
                                    then the geometric normal shades (use_shading_normals = false) */
  const float *triangle_albedo;  /* optional per-triangle RGB replacing the material's kd */
  float emission[3];             /* DiffuseAreaLightSource radiance; all 0 = not a light */
  /* The shading tangent (the BSDF frame's first axis, which anisotropic
   * BxDFs read; TriangleMesh::ComputeDifferentialGeometry,
   * TriangleMesh.cpp:490-528): interpolated per-vertex tangents (mesh
   * space) if given, else the direction of increasing u of per-triangle uvs
   * (6 floats: u0 v0 u1 v1 u2 v2) if given, else -- and where the uvs are
   * degenerate -- CoordinateSystem of the shading normal; made
   * perpendicular to the shading normal. */
  const float *vertex_tangents;
  const float *triangle_uvs;
} skw_render_primitive;

typedef struct skw_point_light {
  float position[3];
  float intensity[3];
} skw_point_light;

/* Builds a render scene: the accelerator (as skw_accel_create) plus the
 * shading data.  Stands in for Scene(primitives, volume, lights)
 * (Raytracer/Core/Scene.h:107-113) with DiffuseAreaLightSource and
 * PointLight lights and no participating medium. */
int skw_scene_create(skw_ctx *ctx, const skw_mesh *meshes, int32_t n_meshes, const skw_render_primitive *prims,
                     int32_t n_prims, const skw_material *materials, int32_t n_materials,
                     const skw_point_light *point_lights, int32_t n_point_lights, skw_scene **out);
void skw_scene_destroy(skw_scene *scene);
/* The scene's accelerator (owned by the scene), for ray queries. */
skw_accel *skw_scene_accel(skw_scene *scene);

/* Pinhole PerspectiveCamera (Raytracer/Cameras/PerspectiveCamera.cpp:36-65):
 * camera-to-world row-major 4x4, horizontal view angle in radians, film size. */
typedef struct skw_camera {
  double camera_to_world[16];
  double x_view_angle;
  int32_t width, height;
} skw_camera;

#define SKW_SAMPLER_STRATIFIED 0 /* StratifiedSampler(spp_x, spp_y) (Samplers/StratifiedSampler.cpp:20-103) */
/* LDSampler(spp_x * spp_y rounded up to a power of two) (Samplers/LDSampler.cpp:20-190):
 * scrambled (0,2)-sequence image points and light / BSDF sample sequences,
 * the light-sample count rounded up to a power of two as the reference's
 * Sampler::AddSamplesSequence* do; the GUI's default sampler. */
#define SKW_SAMPLER_LD 1

typedef struct skw_render_params {
  int32_t spp_x, spp_y;        /* pixel samples: spp_x x spp_y strata, or spp_x * spp_y LD samples */
  int32_t light_samples;       /* DirectLightingLTEIntegratorParams::m_direct_light_samples_num */
  uint64_t seed;               /* counter-based random stream seed */
  int32_t sampler;             /* SKW_SAMPLER_STRATIFIED (0) or SKW_SAMPLER_LD */
} skw_render_params;

/* Renders the direct-lighting estimate of every pixel into film_rgb
 * (height x width x 3 floats, device buffer, row y = image y), the
 * SamplerBasedRenderer + DirectLightingLTEIntegrator + ImageFilm/BoxFilter
 * result (Renderers/SamplerBasedRenderer.cpp:200-239, 419-491,
 * LTEIntegrators/DirectLightingLTEIntegrator.cpp:33-60,
 * Core/DirectLightingIntegrator.cpp:54-366).  Sample radiances that are
 * NaN, negative or infinite count as black, as in the reference. */
int skw_render_direct(skw_scene *scene, const skw_camera *camera, const skw_render_params *params, float *film_rgb,
                      void *stream);

/* Homogeneous participating medium (HomogeneousVolumeRegion with an
 * HGPhaseFunction, VolumeRegions/HomogeneousVolumeRegion.cpp:20-73,
 * PhaseFunctions/HGPhaseFunction.h:53-57) filling an axis-aligned box, and
 * the ray-march step of DirectLightingLTEIntegratorParams::m_media_step_size.
 * With a medium, skw_render_direct, the batch and the adjoint march every
 * camera ray through it (DirectLightingLTEIntegrator.cpp:62-175: emission
 * and one light sample per step) and attenuate light samples through it. */
typedef struct skw_medium {
  float lo[3], hi[3];
  float sigma_a[3], sigma_s[3];
  float emission[3];
  float g;      /* Henyey-Greenstein asymmetry, (-1, 1) */
  float step;   /* march step (> 0) */
} skw_medium;
/* Sets (medium != NULL) or removes (NULL) the scene's medium. */
int skw_scene_set_medium(skw_scene *scene, const skw_medium *medium);

/* The differential geometry of closest hits, as TriangleAccelerator::Intersect
 * completes its Intersection with TriangleMesh::ComputeDifferentialGeometry
 * (Raytracer/Core/TriangleAccelerator.cpp:303-347, TriangleMesh.cpp:414-484):
 * the point o + d t, the geometric normal, the shading normal (interpolated
 * vertex normals, or the geometric normal) and the barycentrics b1, b2 and t
 * of the double Moller-Trumbore test, in double with the reference's
 * operation order, on the scene's world-space triangle.  NaN for a miss.
 * hits: as skw_intersect returns them for the scene's accelerator (prim, tri
 * index the scene's primitives).  Device buffers. */
typedef struct skw_hit_geometry {
  double point[3];
  double geometric_normal[3];
  double shading_normal[3];
  double b1, b2, t;
} skw_hit_geometry;
int skw_scene_hit_geometry(skw_scene *scene, const skw_ray *rays, const skw_hit *hits, int64_t n,
                           skw_hit_geometry *out, void *stream);

/* A RayDifferential (Math/Ray.h:68-111): the base ray in double plus,
 * when has_differentials is nonzero, the rays of the next pixel in x and y.
 * 168 bytes. */
typedef struct skw_ray_differential {
  skw_ray_d ray;
  double origin_dx[3], direction_dx[3];
  double origin_dy[3], direction_dy[3];
  int32_t has_differentials;
  int32_t reserved;
} skw_ray_differential;

/* The Intersection that TriangleAccelerator::Intersect fills
 * (Raytracer/Core/Intersection.h:26-54, DifferentialGeometry.h:25-90):
 * the DifferentialGeometry's point, normals, uv, the next-pixel points and
 * normals, uv derivatives and tangent, the m_cross / m_dot that
 * CoreUtils::GetNextMinT reads, the hit's t, primitive and mesh triangle.
 * 288 bytes. */
typedef struct skw_intersection {
  double point[3];
  double geometric_normal[3];
  double shading_normal[3];
  double uv[2];
  double point_dx[3], point_dy[3];
  double normal_dx[3], normal_dy[3];
  double duv_dx[2], duv_dy[2];
  double tangent[3];
  double cross[3];  /* m_cross */
  double dot;       /* m_dot */
  double t;
  int32_t prim, tri;
} skw_intersection;

/* Completes closest hits into Intersections: TriangleMesh::
 * ComputeDifferentialGeometry (Raytracer/Core/TriangleMesh.cpp:414-561) and
 * the rest of TriangleAccelerator::Intersect (TriangleAccelerator.cpp:
 * 303-347) on the GPU, in double with the reference's operation order.
 * rays / hits: as given to and returned by skw_intersect_d on the scene's
 * accelerator (skw_scene_accel).  Bit-identical to the reference for
 * primitives without a mesh-to-world matrix; a transformed primitive is
 * evaluated on its world-space triangle (the same quantities, rounded
 * differently).  The meshes carry no uv coordinates (the reference's
 * default of zero) and no tangents.  NaN fields and prim = tri = -1 for a
 * miss.  Device buffers. */
int skw_scene_intersection(skw_scene *scene, const skw_ray_differential *rays, const skw_hit_d *hits, int64_t n,
                           skw_intersection *out, void *stream);
/* CoreUtils::GetNextMinT (Raytracer/Core/CoreUtils.h:139-149) of an
 * Intersection for a normalised world direction of a primitive without a
 * mesh-to-world matrix: max(0, dot / (direction . cross) + 1e-14).  Host. */
double skw_next_min_t(const skw_intersection *isect, const double *direction);
/* The outgoing rays the renders make at closest hits (float rays and
 * skw_hit from skw_intersect on the scene's accelerator): origin = the float
 * hit point o + d t, direction = directions[3 i ..] (normalised), tmin =
 * GetNextMinT evaluated in double for that origin and rounded up to float,
 * tmax = +inf; NaN rays for misses.  Device buffers. */
int skw_scene_next_rays(skw_scene *scene, const skw_ray *rays, const skw_hit *hits, const float *directions,
                        int64_t n, skw_ray *out, void *stream);

/* DirectLightingLTEIntegratorParams::m_max_specular_depth
 * (LTEIntegrators/DirectLightingLTEIntegrator.cpp:48-54): camera rays have
 * depth 0, and a hit on a SKW_MATERIAL_TRANSPARENT surface reached by a ray
 * of depth d <= max_depth sends a reflected and a transmitted ray of depth
 * d + 1 (LTEIntegrator::_SpecularReflect / _SpecularTransmit,
 * Core/LTEIntegrator.cpp:66-126).  Default 10 (the GUI's default); range
 * [0, 11]: every branch of every sample's tree is given room, so a render
 * pass holds at most 2^25 >> (max_depth + 1) camera samples.  With a
 * medium the specular rays are marched through it too, in the single-camera
 * render, the batch and the adjoint; the adjoint replays the same trees (a transparent surface's reflectance is
 * its material's, never a per-triangle albedo); photon shooting follows
 * specular bounces (caustic map) and the photon-map render adds caustic
 * radiance and the final gather at the diffuse hits of every level
 * (PhotonLTEIntegrator.cpp:320-385). */
int skw_scene_set_max_specular_depth(skw_scene *scene, int32_t max_depth);

/* ---- Photon maps (PhotonLTEIntegrator, LTEIntegrators/PhotonLTEIntegrator/).
 *
 * A photon (PhotonLTEIntegrator::Photon, PhotonInternalTypes.h:35-59):
 * position, weight, and the 16-bit CompressedDirection ids of the incident
 * direction and of the surface's geometric normal.  28 bytes. */
typedef struct skw_photon {
  float position[3];
  float weight[3];
  uint16_t incident;
  uint16_t normal;
} skw_photon;

typedef struct skw_photon_map skw_photon_map;

typedef struct skw_photon_params {
  int64_t paths;          /* photon paths to shoot (ShootPhotons(i_photons)) */
  int32_t max_bounces;    /* intersections per path, 1..1024 (the reference has no cap) */
  float rr_probability;   /* 0: Russian roulette with the reference's luminance ratio
                             (PhotonShootingPipeline.cpp:243-250); > 0: that fixed
                             continue probability */
  uint64_t seed;          /* random numbers after the first bounce */
} skw_photon_params;

typedef struct skw_photon_map_info {
  int64_t n_caustic, n_direct, n_indirect, n_irradiance;
  int64_t paths_caustic, paths_direct, paths_indirect;
  double max_irradiance_lookup_dist;  /* m_max_irradiance_lookup_dist (inf if unbounded) */
  double scene_area;                  /* sum of the primitives' mesh areas */
  double shoot_ms, build_ms;          /* host wall time: GPU shooting; trees + irradiance map */
  int32_t trees_on_gpu;               /* bit i: map i's tree (caustic, direct, indirect) built on the GPU */
} skw_photon_map_info;

/* Photon maps from given photon arrays (caustic, direct, indirect; any may
 * be empty except that an indirect map needs a direct one) and the paths each
 * map's photons came from: builds the three kd-trees (the reference's median
 * builder, KDTree.h:428-473: on the GPU where no node's median ties on its
 * split axis, else on the host, the same tree either way) and the irradiance photon map
 * (_ConstructIrradiancePhotonMap, PhotonLTEIntegrator.cpp:171-245: every 10th
 * indirect photon in tree order, k = 100 filtered lookups in each map on the
 * GPU, its kd-tree, and the 0.1 % percentile lookup radius).  scene_area is
 * the scene's total mesh area (skw_scene_total_area). */
int skw_photon_map_create(skw_ctx *ctx, const skw_photon *const *photons, const int64_t *n, const int64_t *paths,
                          double scene_area, skw_photon_map **out);
/* Shoots params->paths photon paths through the scene on the GPU
 * (PhotonLTEIntegrator::ShootPhotons, PhotonLTEIntegrator.cpp:247-288 with
 * PhotonsShootingFilter, PhotonShootingPipeline.cpp:110-267) and builds the
 * maps as skw_photon_map_create.  Photons are in path order.  A map over the
 * reference's 40M-photon limit is an error (SKW_ERR_BUDGET). */
int skw_photon_shoot(skw_scene *scene, const skw_photon_params *params, skw_photon_map **out);
void skw_photon_map_destroy(skw_photon_map *map);
int skw_photon_map_get_info(const skw_photon_map *map, skw_photon_map_info *out);
/* Copies map `which` (0 caustic, 1 direct, 2 indirect) in its input order. */
int skw_photon_map_export(const skw_photon_map *map, int32_t which, skw_photon *out);
/* Irradiance photons in kd-tree order: position, external and internal
 * irradiance (3 floats each), normal id. */
int skw_photon_map_export_irradiance(const skw_photon_map *map, float *pos, float *ext, float *intr, uint16_t *nrm);
/* Photon-mapping render parameters (PhotonLTEIntegratorParams,
 * LTEIntegrators/PhotonLTEIntegrator.h:33-70). */
typedef struct skw_photon_render_params {
  int32_t gather_samples;   /* final-gather samples per strategy, rounded up to a square as the sampler does */
  int32_t caustic_lookup;   /* PhotonLTEIntegratorParams::m_caustic_lookup_photons_num (0..4096) */
  double max_caustic_dist;  /* PhotonLTEIntegratorParams::m_max_caustic_lookup_dist (> 0 when caustics are used) */
} skw_photon_render_params;

/* Renders (camera, params) with PhotonLTEIntegrator::_SurfaceRadiance
 * (PhotonLTEIntegrator.cpp:320-385): emission + direct lighting (as
 * skw_render_direct) + the caustic-map radiance (_LookupCausticRadiance,
 * :579-627: the caustic_lookup nearest filtered caustic photons within
 * max_caustic_dist, Simpson's kernel) + final gathering (_FinalGather,
 * :387-577: BSDF- and photon-guided gather rays, the nearest irradiance
 * photon and BSDF::TotalScattering at each gather hit).  No BSDF here is
 * specular, so maps shot by skw_photon_shoot have no caustic photons; maps
 * made from photon arrays (skw_photon_map_create) may. */
int skw_render_photon(skw_scene *scene, const skw_photon_map *map, const skw_camera *camera,
                      const skw_render_params *params, const skw_photon_render_params *photon_params, float *film_rgb,
                      void *stream);
/* The scene's total mesh area (TriangleMesh::GetArea summed over the
 * primitives, PhotonLTEIntegrator.cpp:52-55). */
double skw_scene_total_area(const skw_scene *scene);

/* ---- Direct-lighting adjoint (no counterpart in the reference, which has no
 * derivatives).  Parameters: the per-triangle albedo (the kd of matte and
 * plastic materials; metal has none) and one scale that multiplies every
 * area light's radiance.  Geometry and visibility are held fixed: the
 * adjoint replays the forward render's rays from the same seed (nothing is
 * stored between the two) and accumulates the derivatives of its
 * contributions.  The renderer's rule that drops NaN / negative / infinite
 * sample radiances is not differentiated (it drops nothing on finite
 * inputs). */
/* Triangles in mesh order over all primitives: the albedo arrays below have
 * 3 floats per triangle, triangle g = (sum of the earlier primitives'
 * triangles) + mesh triangle index. */
int64_t skw_scene_n_triangles(const skw_scene *scene);
/* Replaces the per-triangle albedo (3 floats per triangle, any memory the
 * device can read, stream-ordered; NaN in the first channel = the
 * material's kd).  Values are clamped to [0, 1] when shading. */
int skw_scene_set_triangle_albedo(skw_scene *scene, const float *albedo, void *stream);
/* Multiplies every area light's radiance (default 1); takes effect for
 * renders queued afterwards. */
int skw_scene_set_emission_scale(skw_scene *scene, float scale);
/* Given d_film = dL/dI (device, same layout as skw_render_direct's film),
 * ADDS dL/d(albedo) to g_albedo (device, 3 floats per triangle) and
 * dL/d(emission scale) to *g_emission (device double), for the render of
 * (camera, params) -- the same seed gives the same rays as the forward. */
int skw_render_direct_adjoint(skw_scene *scene, const skw_camera *camera, const skw_render_params *params,
                              const float *d_film, float *g_albedo, double *g_emission, void *stream);

/* ---- Batched multi-view render (no counterpart in the reference, whose
 * SamplerBasedRenderer::Render renders one camera per call; the batch is the
 * same estimator as skw_render_direct for every view). ---------------------
 *
 * A batch renders n_views cameras of one scene, each with its own film size,
 * as one wavefront: the views' pixels are concatenated and processed in
 * passes of up to samples_per_pass samples, alternating between two
 * workspaces so that consecutive passes overlap on the GPU.  The whole
 * sequence of passes is captured once into a CUDA graph and each run is a
 * single graph launch.  View v renders exactly what skw_render_direct renders
 * for that camera with seed = view_seeds[v] (params->seed + v when
 * view_seeds is NULL): images are bit-identical to per-view calls. */
typedef struct skw_render_batch skw_render_batch;

typedef struct skw_batch_config {
  int64_t samples_per_pass;    /* wavefront queue capacity (samples in flight per workspace) */
  int32_t stack_cap;           /* traversal stack entries: 48, 96, 192 or 416, at least the tree's need */
  int32_t trace_ctas_per_sm;   /* persistent traversal CTAs per SM, 0 = as many as fit */
  int32_t shade_block;         /* threads per CTA of the shading kernel: 64 or 128 */
  int32_t overlap;             /* 1 = two workspaces on two graph branches, 0 = one */
} skw_batch_config;

/* cfg may be NULL (defaults).  The batch owns its device workspace. */
int skw_render_batch_create(skw_scene *scene, const skw_camera *cameras, int32_t n_views,
                            const skw_render_params *params, const uint64_t *view_seeds,
                            const skw_batch_config *cfg, skw_render_batch **out);
void skw_render_batch_destroy(skw_render_batch *batch);
/* Floats needed for all views' films, and view v's offset (in floats) into
 * the packed film buffer: view v occupies height_v x width_v x 3 floats. */
int64_t skw_render_batch_film_floats(const skw_render_batch *batch);
int64_t skw_render_batch_film_offset(const skw_render_batch *batch, int32_t view);
int skw_render_batch_get_config(const skw_render_batch *batch, skw_batch_config *out);
/* Renders every view into films (device, packed as above), stream-ordered
 * after the work already queued on stream.  The first run with a given films
 * pointer captures the graph; later runs replay it. */
int skw_render_batch_run(skw_render_batch *batch, float *films, void *stream);
/* Autotuner: times candidate configurations of this batch on the GPU
 * (coordinate descent over samples_per_pass, trace_ctas_per_sm, stack_cap,
 * shade_block and overlap; each candidate is a captured graph, one warm-up
 * and two timed launches, CUDA events), installs the fastest and returns it
 * with its time per run in milliseconds.  scratch_films: device buffer of
 * skw_render_batch_film_floats floats that the candidates render into. */
int skw_render_batch_autotune(skw_render_batch *batch, float *scratch_films, void *stream, skw_batch_config *best,
                              float *best_ms, int32_t *n_candidates);

#ifdef __cplusplus
}
#endif

#endif /* SKW_H */
