// C ABI (include/skw.h): contexts, accelerator handles and ray queries.
// Host-side logic only; the kernels live in the .cu translation units.
#include "../../include/skw.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "accel_build.h"
#include "kernels.h"
#include "skw_internal.h"

using skw::DevNode;
using skw::DevTri;

namespace skw {

int fail(skw_ctx *ctx, int code, const std::string &msg) {
  if (ctx) ctx->err = msg;
  return code;
}

int cuda_fail(skw_ctx *ctx, cudaError_t e, const char *what) {
  return fail(ctx, e == cudaErrorMemoryAllocation ? SKW_ERR_OOM : SKW_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

cudaError_t ctx_pool(skw_ctx *ctx, cudaMemPool_t *pool) {
  if (!ctx->pool) {
    cudaMemPoolProps props{};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = ctx->device;
    cudaError_t e = cudaMemPoolCreate(&ctx->pool, &props);
    if (e != cudaSuccess) return e;
    uint64_t keep = UINT64_MAX;
    e = cudaMemPoolSetAttribute(ctx->pool, cudaMemPoolAttrReleaseThreshold, &keep);
    if (e != cudaSuccess) return e;
  }
  *pool = ctx->pool;
  return cudaSuccess;
}

}  // namespace skw

using skw::cuda_fail;
using skw::fail;

extern "C" {

int skw_version(void) { return 100; }

int skw_ctx_create(int device, skw_ctx **out) {
  if (!out) return SKW_ERR_ARG;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return SKW_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= count) return SKW_ERR_ARG;
  auto *ctx = new (std::nothrow) skw_ctx();
  if (!ctx) return SKW_ERR_OOM;
  ctx->device = device;
  cudaDeviceGetAttribute(&ctx->sms, cudaDevAttrMultiProcessorCount, device);
  *out = ctx;
  return SKW_OK;
}

void skw_ctx_destroy(skw_ctx *ctx) {
  if (!ctx) return;
  for (int i = 0; i < 2; ++i) {
    if (ctx->host_st[i]) cudaStreamDestroy(ctx->host_st[i]);
    if (ctx->host_ev[i]) cudaEventDestroy(ctx->host_ev[i]);
    if (ctx->aux_st[i]) cudaStreamDestroy(ctx->aux_st[i]);
  }
  if (ctx->pool) cudaMemPoolDestroy(ctx->pool);
  delete ctx;
}

const char *skw_last_error(const skw_ctx *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int64_t skw_launch_count(const skw_ctx *ctx) { return ctx ? ctx->launches.load() : 0; }

static bool coherent_host_link(int dev);
int skw_ctx_host_buffers_in_place(const skw_ctx *ctx) { return ctx && coherent_host_link(ctx->device) ? 1 : 0; }

struct skw_flat_tree {
  skw::FlatTree ft;
  double build_ms = 0.0;
  bool on_device = false;
};

int skw_flat_tree_build(const skw_mesh *meshes, int32_t n_meshes, const skw_primitive *prims, int32_t n_prims,
                        int threads, skw_flat_tree **out, char *err, size_t errlen) {
  auto set_err = [&](const std::string &m) {
    if (err && errlen > 0) {
      std::strncpy(err, m.c_str(), errlen - 1);
      err[errlen - 1] = 0;
    }
  };
  if (!out || (n_meshes > 0 && !meshes) || (n_prims > 0 && !prims)) {
    set_err("null argument");
    return SKW_ERR_ARG;
  }
  *out = nullptr;
  std::vector<skw::MeshIn> m((size_t)std::max(n_meshes, 0));
  for (int32_t i = 0; i < n_meshes; ++i)
    m[(size_t)i] = skw::MeshIn{meshes[i].vertices, meshes[i].n_vertices, meshes[i].triangles, meshes[i].n_triangles};
  std::vector<skw::PrimIn> p((size_t)std::max(n_prims, 0));
  for (int32_t i = 0; i < n_prims; ++i) p[(size_t)i] = skw::PrimIn{prims[i].mesh, prims[i].mesh_to_world};
  auto *t = new (std::nothrow) skw_flat_tree();
  if (!t) return SKW_ERR_OOM;
  auto t0 = std::chrono::steady_clock::now();
  std::string e = skw::build_accel(m.data(), n_meshes, p.data(), n_prims, threads, t->ft);
  t->build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (!e.empty()) {
    delete t;
    set_err(e);
    return SKW_ERR_ARG;
  }
  *out = t;
  return SKW_OK;
}

int skw_flat_tree_build_device(skw_ctx *ctx, const skw_mesh *meshes, int32_t n_meshes, const skw_primitive *prims,
                               int32_t n_prims, int64_t min_device_triangles, skw_flat_tree **out, int32_t *on_device) {
  if (!ctx || !out || (n_meshes > 0 && !meshes) || (n_prims > 0 && !prims))
    return fail(ctx, SKW_ERR_ARG, "null argument");
  *out = nullptr;
  if (on_device) *on_device = 0;
  cudaError_t ce = cudaSetDevice(ctx->device);
  if (ce != cudaSuccess) return cuda_fail(ctx, ce, "cudaSetDevice");
  std::vector<skw::MeshIn> m((size_t)std::max(n_meshes, 0));
  for (int32_t i = 0; i < n_meshes; ++i)
    m[(size_t)i] = skw::MeshIn{meshes[i].vertices, meshes[i].n_vertices, meshes[i].triangles, meshes[i].n_triangles};
  std::vector<skw::PrimIn> p((size_t)std::max(n_prims, 0));
  for (int32_t i = 0; i < n_prims; ++i) p[(size_t)i] = skw::PrimIn{prims[i].mesh, prims[i].mesh_to_world};
  auto *t = new (std::nothrow) skw_flat_tree();
  if (!t) return fail(ctx, SKW_ERR_OOM, "out of host memory");
  cudaStream_t st = nullptr;
  if ((ce = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) != cudaSuccess) {
    delete t;
    return cuda_fail(ctx, ce, "cudaStreamCreate");
  }
  auto t0 = std::chrono::steady_clock::now();
  bool on_gpu = false;
  std::string e = skw::build_accel_device(m.data(), n_meshes, p.data(), n_prims, 0, st, min_device_triangles,
                                          t->ft, &on_gpu);
  t->build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  cudaStreamDestroy(st);
  if (!e.empty()) {
    delete t;
    return fail(ctx, e.rfind("GPU tree build", 0) == 0 ? SKW_ERR_CUDA : SKW_ERR_ARG, e);
  }
  t->on_device = on_gpu;
  if (on_device) *on_device = on_gpu ? 1 : 0;
  *out = t;
  return SKW_OK;
}

void skw_flat_tree_destroy(skw_flat_tree *t) { delete t; }

int skw_flat_tree_sizes(const skw_flat_tree *t, int64_t *n_nodes, int64_t *n_triangles, int32_t *max_depth) {
  if (!t) return SKW_ERR_ARG;
  if (n_nodes) *n_nodes = (int64_t)t->ft.nodes.size();
  if (n_triangles) *n_triangles = (int64_t)t->ft.tris.size();
  if (max_depth) *max_depth = t->ft.max_depth;
  return SKW_OK;
}

int skw_flat_tree_export(const skw_flat_tree *t, uint32_t *nodes, float *tris, int32_t *tri_prim, int32_t *tri_index) {
  if (!t) return SKW_ERR_ARG;
  if (nodes) std::memcpy(nodes, t->ft.nodes.data(), t->ft.nodes.size() * sizeof(DevNode));
  for (size_t i = 0; i < t->ft.tris.size(); ++i) {
    const DevTri &d = t->ft.tris[i];
    if (tris) {
      std::memcpy(tris + 9 * i, d.v0, 12);
      std::memcpy(tris + 9 * i + 3, d.v1, 12);
      std::memcpy(tris + 9 * i + 6, d.v2, 12);
    }
    if (tri_prim) tri_prim[i] = d.prim;
    if (tri_index) tri_index[i] = d.tri;
  }
  return SKW_OK;
}

int skw_flat_tree_instances(const skw_flat_tree *t, int64_t *n_instances, int32_t *prim, uint32_t *subtree_root,
                            double *world_to_mesh, int64_t *n_subtrees, uint32_t *subtree_roots) {
  if (!t) return SKW_ERR_ARG;
  if (n_instances) *n_instances = (int64_t)t->ft.inst.size();
  if (n_subtrees) *n_subtrees = (int64_t)t->ft.subtree_roots.size();
  for (size_t i = 0; i < t->ft.inst.size(); ++i) {
    if (prim) prim[i] = t->ft.inst[i].prim;
    if (subtree_root) subtree_root[i] = t->ft.inst[i].root;
    if (world_to_mesh) std::memcpy(world_to_mesh + 16 * i, t->ft.inst[i].world_to_mesh, 16 * sizeof(double));
  }
  if (subtree_roots)
    for (size_t i = 0; i < t->ft.subtree_roots.size(); ++i) subtree_roots[i] = t->ft.subtree_roots[i];
  return SKW_OK;
}

int skw_flat_tree_leaf_ranges(const skw_flat_tree *t, uint32_t leaf_word_a, uint32_t *out4) {
  if (!t || !out4 || leaf_word_a >= t->ft.leaf_ext.size()) return SKW_ERR_ARG;
  const skw::LeafExt &e = t->ft.leaf_ext[leaf_word_a];
  out4[0] = e.tri_first;
  out4[1] = e.tri_count;
  out4[2] = e.inst_first;
  out4[3] = e.inst_count;
  return SKW_OK;
}

// take: the tree's host arrays move into the accelerator (the caller
// destroys the tree next) instead of being copied.
static int accel_from_flat(skw_ctx *ctx, skw_flat_tree *tree, bool take, skw_accel **out);

int skw_accel_create_from_flat(skw_ctx *ctx, const skw_flat_tree *tree, skw_accel **out) {
  return accel_from_flat(ctx, const_cast<skw_flat_tree *>(tree), false, out);
}

static int accel_from_flat(skw_ctx *ctx, skw_flat_tree *tree, bool take, skw_accel **out) {
  if (!ctx || !tree || !out) return fail(ctx, SKW_ERR_ARG, "null argument");
  *out = nullptr;
  const skw::FlatTree &ft = tree->ft;
  auto *a = new (std::nothrow) skw_accel();
  if (!a) return fail(ctx, SKW_ERR_OOM, "host allocation failed");
  a->ctx = ctx;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) {
    delete a;
    return cuda_fail(ctx, e, "cudaSetDevice");
  }
  const size_t nb = ft.nodes.size() * sizeof(DevNode), tb = std::max<size_t>(ft.tris.size(), 1) * sizeof(DevTri);
  if ((e = cudaMalloc(&a->d_nodes, nb)) != cudaSuccess || (e = cudaMalloc(&a->d_tris, tb)) != cudaSuccess ||
      (e = cudaMalloc(&a->d_status, sizeof(unsigned))) != cudaSuccess ||
      (e = cudaMalloc(&a->d_traced, sizeof(unsigned long long))) != cudaSuccess) {
    skw_accel_destroy(a);
    return cuda_fail(ctx, e, "cudaMalloc (accelerator)");
  }
  const size_t ib = ft.inst.size() * sizeof(skw::DevInst), eb = ft.leaf_ext.size() * sizeof(skw::LeafExt);
  if (!ft.inst.empty() && ((e = cudaMalloc(&a->d_inst, ib)) != cudaSuccess ||
                           (e = cudaMalloc(&a->d_leaf_ext, std::max<size_t>(eb, 16))) != cudaSuccess ||
                           (e = cudaMemcpy(a->d_inst, ft.inst.data(), ib, cudaMemcpyHostToDevice)) != cudaSuccess ||
                           (eb > 0 && (e = cudaMemcpy(a->d_leaf_ext, ft.leaf_ext.data(), eb, cudaMemcpyHostToDevice)) !=
                                          cudaSuccess))) {
    skw_accel_destroy(a);
    return cuda_fail(ctx, e, "instance tables");
  }
  if ((e = cudaMemcpy(a->d_nodes, ft.nodes.data(), nb, cudaMemcpyHostToDevice)) != cudaSuccess ||
      (!ft.tris.empty() &&
       (e = cudaMemcpy(a->d_tris, ft.tris.data(), ft.tris.size() * sizeof(DevTri), cudaMemcpyHostToDevice)) !=
           cudaSuccess) ||
      (e = cudaMemset(a->d_status, 0, sizeof(unsigned))) != cudaSuccess ||
      (e = cudaMemset(a->d_traced, 0, sizeof(unsigned long long))) != cudaSuccess) {
    skw_accel_destroy(a);
    return cuda_fail(ctx, e, "upload (accelerator)");
  }
  a->stack_cap = skw::traversal_stack_capacity(ft.max_depth);
  for (int k = 0; k < 6; ++k)
    if (std::isfinite(ft.bounds[k])) a->scene_abs = std::max(a->scene_abs, std::fabs(ft.bounds[k]));
  skw_accel_info &info = a->info;
  info.n_triangles = (int64_t)ft.tris.size();
  info.n_nodes = (int64_t)ft.nodes.size();
  info.n_leaves = ft.n_leaves;
  info.max_depth = ft.max_depth;
  info.stack_need = 2 * ft.max_depth + 1;
  std::memcpy(info.bounds, ft.bounds, sizeof(info.bounds));
  info.build_ms = tree->build_ms;
  info.built_on_device = tree->on_device ? 1 : 0;
  info.device_bytes = (int64_t)(nb + tb + ib + eb);
  if (take) {
    skw::FlatTree &mft = tree->ft;
    a->h_nodes = std::move(mft.nodes);
    a->h_tris = std::move(mft.tris);
    a->h_inst = std::move(mft.inst);
    a->h_leaf_ext = std::move(mft.leaf_ext);
    a->h_subtree_roots = std::move(mft.subtree_roots);
  } else {
    a->h_nodes = ft.nodes;
    a->h_tris = ft.tris;
    a->h_inst = ft.inst;
    a->h_leaf_ext = ft.leaf_ext;
    a->h_subtree_roots = ft.subtree_roots;
  }
  // instances need the stack of the top tree and of the deepest subtree at once
  if (a->d_inst) skw::register_instances(a->d_nodes, a->d_inst, a->d_leaf_ext);
  skw::register_ray_counter(a->d_nodes, a->d_traced);
  *out = a;
  return SKW_OK;
}

// Accelerators of at least this many triangles (and no instancing) build
// their tree on the GPU; below it the host build is as fast.
constexpr int64_t kDeviceBuildMin = 16384;

int skw_accel_create(skw_ctx *ctx, const skw_mesh *meshes, int32_t n_meshes, const skw_primitive *prims,
                     int32_t n_prims, skw_accel **out) {
  if (!ctx || !out) return fail(ctx, SKW_ERR_ARG, "null argument");
  skw_flat_tree *t = nullptr;
  int rc = skw_flat_tree_build_device(ctx, meshes, n_meshes, prims, n_prims, kDeviceBuildMin, &t, nullptr);
  if (rc != SKW_OK) return rc;
  rc = accel_from_flat(ctx, t, true, out);
  skw_flat_tree_destroy(t);
  return rc;
}

void skw_accel_destroy(skw_accel *a) {
  if (!a) return;
  if (a->d_nodes) skw::unregister_instances(a->d_nodes);
  cudaFree(a->d_traced);
  cudaFree(a->d_inst);
  cudaFree(a->d_leaf_ext);
  cudaFree(a->d_nodes);
  cudaFree(a->d_tris);
  cudaFree(a->d_status);
  delete a;
}

int skw_accel_rays_traced(const skw_accel *a, uint64_t *out) {
  if (!a || !out) return fail(a ? a->ctx : nullptr, SKW_ERR_ARG, "null argument");
  cudaError_t e = cudaSetDevice(a->ctx->device);
  unsigned long long v = 0;
  if (e == cudaSuccess) e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaMemcpy(&v, a->d_traced, sizeof(v), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(a->ctx, e, "rays traced");
  *out = (uint64_t)v;
  return SKW_OK;
}

int skw_accel_get_info(const skw_accel *a, skw_accel_info *info) {
  if (!a || !info) return SKW_ERR_ARG;
  *info = a->info;
  return SKW_OK;
}

int skw_accel_export(const skw_accel *a, uint32_t *nodes, int32_t *tri_prim, int32_t *tri_index) {
  if (!a) return SKW_ERR_ARG;
  if (nodes) std::memcpy(nodes, a->h_nodes.data(), a->h_nodes.size() * sizeof(DevNode));
  for (size_t i = 0; i < a->h_tris.size(); ++i) {
    if (tri_prim) tri_prim[i] = a->h_tris[i].prim;
    if (tri_index) tri_index[i] = a->h_tris[i].tri;
  }
  return SKW_OK;
}

static int run_query(skw_accel *a, bool closest, bool dray, const void *rays, int64_t n, void *out, void *stream) {
  if (!a) return SKW_ERR_ARG;
  if (n < 0 || (n > 0 && (!rays || !out))) return fail(a->ctx, SKW_ERR_ARG, "bad ray buffer");
  if (n > (int64_t)INT32_MAX) return fail(a->ctx, SKW_ERR_ARG, "too many rays for one call (max 2^31-1)");
  if (n == 0) return SKW_OK;
  skw_ctx *ctx = a->ctx;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaSetDevice");
  // the launch's ray-group counter, stream-ordered from the context's pool
  // (its own for every call, so calls on different streams never share one)
  cudaStream_t st = (cudaStream_t)stream;
  cudaMemPool_t pool;
  int *work = nullptr;
  if ((e = skw::ctx_pool(ctx, &pool)) != cudaSuccess ||
      (e = cudaMallocFromPoolAsync((void **)&work, 256, pool, st)) != cudaSuccess)
    return cuda_fail(ctx, e, "work counter");
  e = dray ? skw::launch_traversal_d(closest, a->stack_cap, a->d_nodes, a->d_tris, rays, n, a->scene_abs, out,
                                     a->d_status, st, work)
           : skw::launch_traversal(closest, a->stack_cap, a->d_nodes, a->d_tris, rays, n, nullptr, a->scene_abs,
                                   nullptr, out, a->d_status, st, 0, work);
  cudaFreeAsync(work, st);
  if (e != cudaSuccess) return cuda_fail(ctx, e, closest ? "closest-hit launch" : "any-hit launch");
  ctx->launches.fetch_add(1);
  return SKW_OK;
}

int skw_intersect(skw_accel *a, const skw_ray *rays, int64_t n, skw_hit *hits, void *stream) {
  return run_query(a, true, false, rays, n, hits, stream);
}

int skw_intersect_test(skw_accel *a, const skw_ray *rays, int64_t n, uint8_t *occluded, void *stream) {
  return run_query(a, false, false, rays, n, occluded, stream);
}

int skw_intersect_d(skw_accel *a, const skw_ray_d *rays, int64_t n, skw_hit_d *hits, void *stream) {
  return run_query(a, true, true, rays, n, hits, stream);
}

int skw_intersect_test_d(skw_accel *a, const skw_ray_d *rays, int64_t n, uint8_t *occluded, void *stream) {
  return run_query(a, false, true, rays, n, occluded, stream);
}

// Host-buffer queries.  Above kHostChunk rays the rays go in and the results
// come out in chunks of kHostChunk alternating over two streams, so that the
// copies of one chunk (H2D and D2H use separate copy engines) overlap the
// traversal of the other; each chunk's persistent traversal takes half the
// resident CTAs per SM, so the two chunks trace side by side and one's tail
// overlaps the other's body (a full-size grid per chunk would serialise the
// chunks and add a tail per chunk).  Measured on 4M rays: 846 Mrays/s end to
// end against 787 for one copy-in, query, copy-out sequence.
static constexpr int64_t kHostChunk = (int64_t)1 << 21;

// Whether the device reaches host memory over a coherent link (NVLink-C2C on
// a Grace system: native atomics across the link), once per device.
static bool coherent_host_link(int dev) {
  static std::mutex mu;
  static int known[64] = {0};  // 0 unknown, 1 no, 2 yes
  if (dev < 0 || dev >= 64) return false;
  std::lock_guard<std::mutex> lock(mu);
  if (!known[dev]) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrHostNativeAtomicSupported, dev) != cudaSuccess) {
      cudaGetLastError();
      v = 0;
    }
    known[dev] = v ? 2 : 1;
  }
  return known[dev] == 2;
}

// The device address of a page-locked host buffer (cudaHostAlloc /
// cudaHostRegister), or null when the buffer is not one.
static void *mapped_host(const void *p) {
  cudaPointerAttributes at{};
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return at.type == cudaMemoryTypeHost ? at.devicePointer : nullptr;
}

// Status check after a host-buffer query.
static int query_status(skw_accel *a) {
  unsigned sv = 0;
  cudaError_t e = cudaMemcpy(&sv, a->d_status, sizeof(sv), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(a->ctx, e, "status read");
  if (sv & 1u) {
    cudaMemset(a->d_status, 0, sizeof(unsigned));
    return fail(a->ctx, SKW_ERR_STACK_OVERFLOW, "traversal stack overflow");
  }
  return SKW_OK;
}

static int run_query_host(skw_accel *a, bool closest, bool dray, const void *rays, int64_t n, void *out) {
  if (!a) return SKW_ERR_ARG;
  if (n < 0 || (n > 0 && (!rays || !out))) return fail(a->ctx, SKW_ERR_ARG, "bad ray buffer");
  if (n == 0) return SKW_OK;
  cudaError_t e = cudaSetDevice(a->ctx->device);
  if (e != cudaSuccess) return cuda_fail(a->ctx, e, "cudaSetDevice");
  // Page-locked host buffers on a coherent CPU-GPU link: the traversal reads
  // the rays from host memory and writes the results there itself, so the
  // transfers run inside the kernel, overlapped with its work, with no
  // staging buffers and no separate copies.
  void *hr = nullptr, *ho = nullptr;
  if (coherent_host_link(a->ctx->device) && (hr = mapped_host(rays)) != nullptr && (ho = mapped_host(out)) != nullptr) {
    skw_ctx *c = a->ctx;
    if (!c->host_st[0] && (e = cudaStreamCreateWithFlags(&c->host_st[0], cudaStreamNonBlocking)) != cudaSuccess)
      return cuda_fail(c, e, "stream");
    cudaStream_t s = c->host_st[0];
    cudaMemPool_t pool;
    if ((e = skw::ctx_pool(c, &pool)) != cudaSuccess) return cuda_fail(c, e, "workspace pool");
    int *d_work = nullptr;
    if ((e = cudaMallocFromPoolAsync((void **)&d_work, 256, pool, s)) != cudaSuccess)
      return cuda_fail(c, e, "cudaMallocAsync");
    const size_t ru = dray ? sizeof(skw_ray_d) : sizeof(skw_ray);
    const size_t ou = closest ? (dray ? sizeof(skw_hit_d) : sizeof(skw_hit)) : 1;
    const int64_t per = (int64_t)1 << 30;  // rays per launch (the kernels index rays with 32-bit ints)
    for (int64_t r0 = 0; r0 < n && e == cudaSuccess; r0 += per) {
      const int64_t m = std::min(per, n - r0);
      const char *rr = (const char *)hr + (size_t)r0 * ru;
      char *oo = (char *)ho + (size_t)r0 * ou;
      e = dray ? skw::launch_traversal_d(closest, a->stack_cap, a->d_nodes, a->d_tris, rr, m, a->scene_abs, oo,
                                         a->d_status, s, d_work)
               : skw::launch_traversal(closest, a->stack_cap, a->d_nodes, a->d_tris, rr, m, nullptr, a->scene_abs,
                                       nullptr, oo, a->d_status, s, 0, d_work);
    }
    cudaFreeAsync(d_work, s);
    cudaError_t es = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(c, e, "launch");
    if (es != cudaSuccess) return cuda_fail(c, es, "query execution");
    c->launches.fetch_add(1);
    return query_status(a);
  }
  const size_t out_unit = closest ? (dray ? sizeof(skw_hit_d) : sizeof(skw_hit)) : 1;
  const size_t ray_unit = dray ? sizeof(skw_ray_d) : sizeof(skw_ray);
  const int64_t n_chunks = (n + kHostChunk - 1) / kHostChunk;
  const int n_streams = (int)std::min<int64_t>(n_chunks, 2);
  const int ctas = n_chunks > 1 ? std::max(1, skw::traversal_max_ctas_per_sm(a->stack_cap) / 2) : 0;
  cudaMemPool_t pool;
  if ((e = skw::ctx_pool(a->ctx, &pool)) != cudaSuccess) return cuda_fail(a->ctx, e, "workspace pool");
  cudaStream_t st[2] = {nullptr, nullptr};
  cudaEvent_t ev[2] = {nullptr, nullptr};
  int rc = SKW_OK;
  for (int i = 0; i < n_streams && rc == SKW_OK; ++i) {
    skw_ctx *c = a->ctx;
    if ((!c->host_st[i] && (e = cudaStreamCreateWithFlags(&c->host_st[i], cudaStreamNonBlocking)) != cudaSuccess) ||
        (!c->host_ev[i] && (e = cudaEventCreateWithFlags(&c->host_ev[i], cudaEventDisableTiming)) != cudaSuccess))
      rc = cuda_fail(c, e, "stream");
    st[i] = c->host_st[i];
    ev[i] = c->host_ev[i];
  }
  // One chunk of rays and results per stream: chunks c, c + 2, ... reuse
  // their stream's buffers in stream order, so device memory stays at two
  // chunks however many rays the call has.
  const int64_t chunk_rays = std::min(n, kHostChunk);
  void *d_rays = nullptr, *d_out = nullptr;
  int *d_work = nullptr;  // one ray-group counter per stream (256 bytes apart)
  if (rc == SKW_OK &&
      ((e = cudaMallocFromPoolAsync(&d_rays, (size_t)(n_streams * chunk_rays) * ray_unit, pool, st[0])) !=
           cudaSuccess ||
       (e = cudaMallocFromPoolAsync(&d_out, (size_t)(n_streams * chunk_rays) * out_unit, pool, st[0])) != cudaSuccess ||
       (e = cudaMallocFromPoolAsync((void **)&d_work, 512, pool, st[0])) != cudaSuccess))
    rc = cuda_fail(a->ctx, e, "cudaMallocAsync");
  // the other streams start after the allocations
  if (rc == SKW_OK && (e = cudaEventRecord(ev[0], st[0])) != cudaSuccess) rc = cuda_fail(a->ctx, e, "event");
  for (int i = 1; i < n_streams && rc == SKW_OK; ++i)
    if ((e = cudaStreamWaitEvent(st[i], ev[0], 0)) != cudaSuccess) rc = cuda_fail(a->ctx, e, "event");
  for (int64_t c = 0; c < n_chunks && rc == SKW_OK; ++c) {
    const int si = (int)(c % n_streams);
    cudaStream_t s = st[si];
    const int64_t r0 = c * kHostChunk, m = std::min(kHostChunk, n - r0);
    char *dr = (char *)d_rays + (size_t)(si * chunk_rays) * ray_unit;
    char *dout = (char *)d_out + (size_t)(si * chunk_rays) * out_unit;
    if ((e = cudaMemcpyAsync(dr, (const char *)rays + (size_t)r0 * ray_unit, (size_t)m * ray_unit,
                             cudaMemcpyHostToDevice, s)) != cudaSuccess) {
      rc = cuda_fail(a->ctx, e, "copy rays in");
    } else if ((e = dray ? skw::launch_traversal_d(closest, a->stack_cap, a->d_nodes, a->d_tris, dr, m, a->scene_abs,
                                                   dout, a->d_status, s, d_work + 64 * si)
                         : skw::launch_traversal(closest, a->stack_cap, a->d_nodes, a->d_tris, dr, m, nullptr,
                                                 a->scene_abs, nullptr, dout, a->d_status, s, ctas,
                                                 d_work + 64 * si)) != cudaSuccess) {
      rc = cuda_fail(a->ctx, e, "launch");
    } else {
      a->ctx->launches.fetch_add(1);
      if ((e = cudaMemcpyAsync((char *)out + (size_t)r0 * out_unit, dout, (size_t)m * out_unit,
                               cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        rc = cuda_fail(a->ctx, e, "copy results out");
    }
  }
  // free on the first stream once every stream is done with the buffers
  for (int i = 1; i < n_streams; ++i) {
    if (cudaEventRecord(ev[i], st[i]) == cudaSuccess) cudaStreamWaitEvent(st[0], ev[i], 0);
  }
  if (d_rays) cudaFreeAsync(d_rays, st[0]);
  if (d_out) cudaFreeAsync(d_out, st[0]);
  if (d_work) cudaFreeAsync(d_work, st[0]);
  for (int i = 0; i < n_streams; ++i) {
    if (st[i]) {
      e = cudaStreamSynchronize(st[i]);
      if (rc == SKW_OK && e != cudaSuccess) rc = cuda_fail(a->ctx, e, "query execution");
    }
  }
  if (rc == SKW_OK) return query_status(a);
  return rc;
}

int skw_intersect_host(skw_accel *a, const skw_ray *rays, int64_t n, skw_hit *hits) {
  return run_query_host(a, true, false, rays, n, hits);
}

int skw_intersect_test_host(skw_accel *a, const skw_ray *rays, int64_t n, uint8_t *occluded) {
  return run_query_host(a, false, false, rays, n, occluded);
}

int skw_intersect_d_host(skw_accel *a, const skw_ray_d *rays, int64_t n, skw_hit_d *hits) {
  return run_query_host(a, true, true, rays, n, hits);
}

int skw_intersect_test_d_host(skw_accel *a, const skw_ray_d *rays, int64_t n, uint8_t *occluded) {
  return run_query_host(a, false, true, rays, n, occluded);
}

}  // extern "C"
