// C ABI (include/skw.h): photon kd-tree handles and lookups.
#include "../../include/skw.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "kernels.h"
#include "photon_tree.h"
#include "skw_internal.h"

struct skw_kdtree {
  skw_ctx *ctx = nullptr;
  int64_t n = 0;
  void *d_nodes = nullptr;       // KdNode[n]
  uint16_t *d_nids = nullptr;    // normal id per tree position
  double *d_dirs = nullptr;      // 3 << 16 doubles
  unsigned *d_status = nullptr;
  std::vector<int32_t> perm;
  float lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};  // the points' bounds (the queries' spatial bins)
};

using skw::cuda_fail;
using skw::fail;

namespace {
constexpr int kMaxK = 4096;
constexpr int64_t kBinMin = 65536;  // batches from this size are looked up in spatial-bin order

int check_query_args(skw_kdtree *t, const double *q, const double *qn, int64_t nq, int32_t k, double max_dist,
                     double cos_threshold, bool need_k) {
  if (!t) return SKW_ERR_ARG;
  if (nq < 0 || nq > (int64_t)INT32_MAX) return fail(t->ctx, SKW_ERR_ARG, "query count out of range");
  if (nq > 0 && !q) return fail(t->ctx, SKW_ERR_ARG, "null query buffer");
  if (cos_threshold >= 0.0 && nq > 0 && !qn) return fail(t->ctx, SKW_ERR_ARG, "filtered lookup needs normals");
  if (cos_threshold > 1.0) return fail(t->ctx, SKW_ERR_ARG, "cos_threshold must be <= 1");
  if (!(max_dist >= 0.0)) return fail(t->ctx, SKW_ERR_ARG, "max_dist must be >= 0");
  if (need_k && (k < 0 || k > kMaxK)) return fail(t->ctx, SKW_ERR_ARG, "k out of range (0..4096)");
  return SKW_OK;
}
}  // namespace

extern "C" {

uint16_t skw_compress_direction(double x, double y, double z) { return skw::compress_direction(x, y, z); }

int skw_direction_table(double *out) {
  if (!out) return SKW_ERR_ARG;
  const std::vector<double> &t = skw::direction_table();
  std::memcpy(out, t.data(), t.size() * sizeof(double));
  return SKW_OK;
}

namespace {
// perm and the (split, word) node pairs of a built tree.
void export_tree(const std::vector<skw::KdNode> &nodes, const std::vector<int32_t> &p, int64_t n, int32_t *perm,
                 uint32_t *node_words) {
  for (int64_t i = 0; i < n; ++i) {
    if (perm) perm[i] = p[(size_t)i];
    if (node_words) {
      const skw::KdNode &nd = nodes[(size_t)i];
      const uint32_t axis = nd.word & 3u;
      float split = 0.0f;  // the reference leaves a leaf's split at 0
      if (axis != 3u) split = axis == 0 ? nd.x : (axis == 1 ? nd.y : nd.z);
      std::memcpy(&node_words[2 * i], &split, 4);
      node_words[2 * i + 1] = nd.word;
    }
  }
}
}  // namespace

int skw_kdtree_build_host(const float *positions, int64_t n, int threads, int32_t *perm, uint32_t *node_words) {
  if (n < 0 || (n > 0 && !positions) || n >= ((int64_t)1 << 29)) return SKW_ERR_ARG;
  std::vector<skw::KdNode> nodes;
  std::vector<int32_t> p;
  skw::build_photon_tree(positions, n, threads, nodes, p);
  export_tree(nodes, p, n, perm, node_words);
  return SKW_OK;
}

int skw_kdtree_repair_host(const float *positions, int64_t n, const int32_t *ties, int64_t n_ties, int32_t *perm,
                           uint32_t *node_words) {
  if (n < 0 || (n > 0 && (!positions || !perm || !node_words)) || n >= ((int64_t)1 << 29) || n_ties < 0 ||
      (n_ties > 0 && !ties))
    return SKW_ERR_ARG;
  std::vector<skw::KdNode> nodes((size_t)n);
  std::vector<int32_t> p(perm, perm + n);
  for (int64_t i = 0; i < n; ++i) {
    const int32_t s = p[(size_t)i];
    if (s < 0 || s >= n) return SKW_ERR_ARG;
    nodes[(size_t)i] = skw::KdNode{positions[3 * s], positions[3 * s + 1], positions[3 * s + 2], node_words[2 * i + 1]};
  }
  for (int64_t i = 0; i < n_ties; ++i)
    if (ties[i] < 0 || ties[i] >= n) return SKW_ERR_ARG;
  skw::repair_photon_tree(positions, n, std::vector<int32_t>(ties, ties + n_ties), nodes, p);
  export_tree(nodes, p, n, perm, node_words);
  return SKW_OK;
}

int skw_kdtree_build_device(skw_ctx *ctx, const float *positions, int64_t n, int32_t *perm, uint32_t *node_words,
                            int32_t *median_tie) {
  if (!ctx || !median_tie) return fail(ctx, SKW_ERR_ARG, "null argument");
  if (n < 0 || (n > 0 && !positions) || n >= ((int64_t)1 << 29)) return fail(ctx, SKW_ERR_ARG, "bad photon buffer");
  *median_tie = 0;
  if (n == 0) return SKW_OK;
  cudaError_t e = cudaSetDevice(ctx->device);
  float *d_pos = nullptr;
  int32_t *d_perm = nullptr;
  int *d_tie = nullptr;
  skw::KdNode *d_nodes = nullptr;
  void *scratch = nullptr;
  std::vector<int> tie(1 + skw::kTieCap, 0);
  std::vector<skw::KdNode> nodes((size_t)n);
  std::vector<int32_t> p((size_t)n);
  if (e == cudaSuccess) e = cudaMalloc((void **)&d_pos, (size_t)n * 12);
  if (e == cudaSuccess) e = cudaMalloc((void **)&d_perm, (size_t)n * 4);
  if (e == cudaSuccess) e = cudaMalloc((void **)&d_tie, tie.size() * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc((void **)&d_nodes, (size_t)n * sizeof(skw::KdNode));
  if (e == cudaSuccess) e = cudaMalloc(&scratch, skw::photon_tree_gpu_scratch(n));
  if (e == cudaSuccess) e = cudaMemcpy(d_pos, positions, (size_t)n * 12, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = skw::build_photon_tree_gpu(d_pos, n, d_nodes, d_perm, d_tie, scratch, nullptr);
  if (e == cudaSuccess) e = cudaMemcpy(tie.data(), d_tie, tie.size() * sizeof(int), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(nodes.data(), d_nodes, (size_t)n * sizeof(skw::KdNode), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(p.data(), d_perm, (size_t)n * 4, cudaMemcpyDeviceToHost);
  for (void *q : {(void *)d_pos, (void *)d_perm, (void *)d_tie, (void *)d_nodes, scratch}) cudaFree(q);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "photon tree build");
  if (tie[0] > skw::kTieCap)  // too many tied medians to repair: the host build
    skw::build_photon_tree(positions, n, 0, nodes, p);
  else if (tie[0] > 0)
    skw::repair_photon_tree(positions, n, std::vector<int32_t>(tie.begin() + 1, tie.begin() + 1 + tie[0]), nodes, p);
  export_tree(nodes, p, n, perm, node_words);
  *median_tie = tie[0];
  return SKW_OK;
}

int skw_kdtree_create(skw_ctx *ctx, const float *positions, const uint16_t *normal_ids, int64_t n,
                      skw_kdtree **out) {
  if (!ctx || !out) return fail(ctx, SKW_ERR_ARG, "null argument");
  *out = nullptr;
  if (n < 0 || (n > 0 && !positions)) return fail(ctx, SKW_ERR_ARG, "bad photon buffer");
  if (n >= ((int64_t)1 << 29)) return fail(ctx, SKW_ERR_ARG, "too many photons (the node format holds < 2^29)");
  auto *t = new (std::nothrow) skw_kdtree();
  if (!t) return fail(ctx, SKW_ERR_OOM, "host allocation failed");
  t->ctx = ctx;
  t->n = n;
  for (int a = 0; a < 3; ++a) {
    t->lo[a] = INFINITY;
    t->hi[a] = -INFINITY;
  }
  for (int64_t i = 0; i < n; ++i)
    for (int a = 0; a < 3; ++a) {
      t->lo[a] = std::min(t->lo[a], positions[3 * i + a]);
      t->hi[a] = std::max(t->hi[a], positions[3 * i + a]);
    }
  cudaError_t e = cudaSetDevice(ctx->device);
  // the tree on the GPU where that gives the reference's (no median ties),
  // else on the host
  skw::KdNode *dn = nullptr;
  int32_t *d_perm = nullptr;
  bool on_gpu = false;
  if (e == cudaSuccess) e = skw::build_photon_tree_device(positions, n, nullptr, &dn, t->perm, &d_perm, &on_gpu);
  cudaFree(d_perm);
  t->d_nodes = dn;
  std::vector<uint16_t> nids((size_t)std::max<int64_t>(n, 1), 0);
  if (normal_ids && e == cudaSuccess)
    for (int64_t i = 0; i < n; ++i) nids[(size_t)i] = normal_ids[t->perm[(size_t)i]];
  const std::vector<double> &dirs = skw::direction_table_device();
  if (e == cudaSuccess) e = cudaMalloc(&t->d_nids, nids.size() * sizeof(uint16_t));
  if (e == cudaSuccess) e = cudaMalloc(&t->d_dirs, dirs.size() * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc(&t->d_status, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemcpy(t->d_nids, nids.data(), nids.size() * sizeof(uint16_t), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(t->d_dirs, dirs.data(), dirs.size() * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemset(t->d_status, 0, sizeof(unsigned));
  if (e != cudaSuccess) {
    skw_kdtree_destroy(t);
    return cuda_fail(ctx, e, "photon tree upload");
  }
  *out = t;
  return SKW_OK;
}

void skw_kdtree_destroy(skw_kdtree *t) {
  if (!t) return;
  cudaFree(t->d_nodes);
  cudaFree(t->d_nids);
  cudaFree(t->d_dirs);
  cudaFree(t->d_status);
  delete t;
}

int skw_kdtree_size(const skw_kdtree *t, int64_t *n) {
  if (!t || !n) return SKW_ERR_ARG;
  *n = t->n;
  return SKW_OK;
}

int skw_kdtree_permutation(const skw_kdtree *t, int32_t *perm) {
  if (!t || (!perm && t->n > 0)) return SKW_ERR_ARG;
  if (t->n > 0) std::memcpy(perm, t->perm.data(), (size_t)t->n * sizeof(int32_t));
  return SKW_OK;
}

int skw_knn(skw_kdtree *t, const double *q, const double *qn, int64_t nq, int32_t k, double max_dist,
            double cos_threshold, int32_t *out_idx, double *out_d2, int32_t *out_count, void *stream) {
  int rc = check_query_args(t, q, qn, nq, k, max_dist, cos_threshold, true);
  if (rc != SKW_OK) return rc;
  if (nq > 0 && (!out_count || (k > 0 && (!out_idx || !out_d2))))
    return fail(t->ctx, SKW_ERR_ARG, "null output buffer");
  if (nq == 0) return SKW_OK;
  cudaError_t e = cudaSetDevice(t->ctx->device);
  if (e != cudaSuccess) return cuda_fail(t->ctx, e, "cudaSetDevice");
  cudaStream_t s = (cudaStream_t)stream;
  void *scratch = nullptr;
  const size_t sb = skw::knn_scratch_bytes(nq, k);
  cudaMemPool_t pool;
  if ((e = skw::ctx_pool(t->ctx, &pool)) != cudaSuccess) return cuda_fail(t->ctx, e, "workspace pool");
  if (sb > 0 && (e = cudaMallocFromPoolAsync(&scratch, sb, pool, s)) != cudaSuccess)
    return cuda_fail(t->ctx, e, "k-NN heap workspace");
  // Large batches are looked up in spatial-bin order of the queries (64^3
  // cells over the points' bounds, sorted stably so that each cell's
  // queries keep their order): a warp's walks then start near each other.
  int32_t *order = nullptr;
  void *bin_ws = nullptr;
  if (nq >= kBinMin && t->n > 0) {
    const size_t ob = ((size_t)nq * 4 + 255) & ~(size_t)255;
    if ((e = cudaMallocFromPoolAsync(&bin_ws, ob + skw::sort_order_bytes(nq), pool, s)) == cudaSuccess) {
      char *w = (char *)bin_ws;
      order = (int32_t *)w;
      e = skw::launch_sort_order(q, nq, t->lo, t->hi, w + ob, order, s);
    }
    if (e != cudaSuccess) {
      if (bin_ws) cudaFreeAsync(bin_ws, s);
      if (scratch) cudaFreeAsync(scratch, s);
      return cuda_fail(t->ctx, e, "k-NN query bins");
    }
  }
  e = skw::launch_knn(t->d_nodes, t->d_nids, t->d_dirs, (int)t->n, q, qn, nq, k, max_dist, cos_threshold, out_idx,
                      out_d2, out_count, nullptr, scratch, t->d_status, s, nullptr, order);
  if (bin_ws) cudaFreeAsync(bin_ws, s);
  if (scratch) cudaFreeAsync(scratch, s);
  if (e != cudaSuccess) return cuda_fail(t->ctx, e, "k-NN launch");
  t->ctx->launches.fetch_add(1);
  return SKW_OK;
}

int skw_knn_noalloc(skw_kdtree *t, const double *q, const double *qn, int64_t nq, int32_t k, double max_dist,
                    double cos_threshold, int32_t *out_idx, double *out_d2, int32_t *out_count, void *stream) {
  int rc = check_query_args(t, q, qn, nq, k, max_dist, cos_threshold, true);
  if (rc != SKW_OK) return rc;
  if (nq > 0 && (!out_count || (k > 0 && (!out_idx || !out_d2))))
    return fail(t->ctx, SKW_ERR_ARG, "null output buffer");
  const int64_t cap = skw::knn_noalloc_capacity();
  if (nq * (int64_t)k > cap)
    return fail(t->ctx, SKW_ERR_ARG,
                "skw_knn_noalloc: nq * k = " + std::to_string(nq * (int64_t)k) +
                    " heap entries exceeds the static scratch capacity of " + std::to_string(cap) +
                    "; split the queries into smaller batches");
  if (nq == 0) return SKW_OK;
  cudaError_t e = cudaSetDevice(t->ctx->device);
  if (e != cudaSuccess) return cuda_fail(t->ctx, e, "cudaSetDevice");
  e = skw::launch_knn_noalloc(t->d_nodes, t->d_nids, t->d_dirs, (int)t->n, q, qn, nq, k, max_dist, cos_threshold,
                              out_idx, out_d2, out_count, t->d_status, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(t->ctx, e, "k-NN (no allocation) launch");
  t->ctx->launches.fetch_add(1);
  return SKW_OK;
}

int skw_knn_host(skw_kdtree *t, const double *q, const double *qn, int64_t nq, int32_t k, double max_dist,
                 double cos_threshold, int32_t *out_idx, double *out_d2, int32_t *out_count) {
  int rc = check_query_args(t, q, qn, nq, k, max_dist, cos_threshold, true);
  if (rc != SKW_OK) return rc;
  if (nq > 0 && (!out_count || (k > 0 && (!out_idx || !out_d2))))
    return fail(t->ctx, SKW_ERR_ARG, "null output buffer");
  if (nq == 0) return SKW_OK;
  cudaError_t e = cudaSetDevice(t->ctx->device);
  if (e != cudaSuccess) return cuda_fail(t->ctx, e, "cudaSetDevice");
  cudaMemPool_t pool;
  if ((e = skw::ctx_pool(t->ctx, &pool)) != cudaSuccess) return cuda_fail(t->ctx, e, "workspace pool");
  cudaStream_t s = nullptr;
  if ((e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking)) != cudaSuccess) return cuda_fail(t->ctx, e, "stream");
  const bool filt = cos_threshold >= 0.0;
  const size_t qb = (size_t)nq * 3 * sizeof(double), ib = (size_t)nq * (size_t)k * 4, db = (size_t)nq * (size_t)k * 8,
               cb = (size_t)nq * 4;
  char *buf = nullptr;
  const size_t total = qb * (filt ? 2 : 1) + ib + db + cb + 64;
  rc = SKW_OK;
  if ((e = cudaMallocFromPoolAsync((void **)&buf, total, pool, s)) != cudaSuccess) {
    rc = cuda_fail(t->ctx, e, "k-NN buffers");
  } else {
    double *dq = (double *)buf;
    double *dqn = filt ? (double *)(buf + qb) : nullptr;
    char *p = buf + qb * (filt ? 2 : 1);
    double *dd2 = (double *)p;
    int32_t *didx = (int32_t *)(p + db);
    int32_t *dcnt = (int32_t *)(p + db + ib);
    if ((e = cudaMemcpyAsync(dq, q, qb, cudaMemcpyHostToDevice, s)) != cudaSuccess ||
        (filt && (e = cudaMemcpyAsync(dqn, qn, qb, cudaMemcpyHostToDevice, s)) != cudaSuccess)) {
      rc = cuda_fail(t->ctx, e, "copy queries in");
    } else if ((rc = skw_knn(t, dq, dqn, nq, k, max_dist, cos_threshold, didx, dd2, dcnt, s)) == SKW_OK) {
      if ((k > 0 && ((e = cudaMemcpyAsync(out_idx, didx, ib, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
                     (e = cudaMemcpyAsync(out_d2, dd2, db, cudaMemcpyDeviceToHost, s)) != cudaSuccess)) ||
          (e = cudaMemcpyAsync(out_count, dcnt, cb, cudaMemcpyDeviceToHost, s)) != cudaSuccess)
        rc = cuda_fail(t->ctx, e, "copy results out");
    }
    cudaFreeAsync(buf, s);
  }
  e = cudaStreamSynchronize(s);
  if (rc == SKW_OK && e != cudaSuccess) rc = cuda_fail(t->ctx, e, "k-NN execution");
  cudaStreamDestroy(s);
  if (rc == SKW_OK) {
    unsigned st = 0;
    if ((e = cudaMemcpy(&st, t->d_status, sizeof(st), cudaMemcpyDeviceToHost)) != cudaSuccess)
      return cuda_fail(t->ctx, e, "status read");
    if (st & 2u) {
      cudaMemset(t->d_status, 0, sizeof(unsigned));
      return fail(t->ctx, SKW_ERR_STACK_OVERFLOW, "k-NN stack overflow");
    }
  }
  return rc;
}

int skw_nearest(skw_kdtree *t, const double *q, const double *qn, int64_t nq, double max_dist, double cos_threshold,
                int32_t *out_idx, void *stream) {
  int rc = check_query_args(t, q, qn, nq, 1, max_dist, cos_threshold, false);
  if (rc != SKW_OK) return rc;
  if (nq > 0 && !out_idx) return fail(t->ctx, SKW_ERR_ARG, "null output buffer");
  if (nq == 0) return SKW_OK;
  cudaError_t e = cudaSetDevice(t->ctx->device);
  if (e != cudaSuccess) return cuda_fail(t->ctx, e, "cudaSetDevice");
  e = skw::launch_nearest(t->d_nodes, t->d_nids, t->d_dirs, (int)t->n, q, qn, nq, max_dist, cos_threshold, out_idx,
                          t->d_status, (cudaStream_t)stream);
  if (e != cudaSuccess) return cuda_fail(t->ctx, e, "nearest launch");
  t->ctx->launches.fetch_add(1);
  return SKW_OK;
}

}  // extern "C"
