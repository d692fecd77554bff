// C ABI (include/skw.h): measured BRDFs.
#include "../../include/skw.h"

#include <cuda_runtime.h>

#include <new>

#include "merl.h"
#include "skw_internal.h"

using skw::cuda_fail;
using skw::fail;

struct skw_merl {
  skw_ctx *ctx = nullptr;
  skw::MerlHost host;
  skw::MerlDev dev{};
};

extern "C" {

int skw_merl_create(skw_ctx *ctx, const void *bytes, int64_t n_bytes, skw_merl **out) {
  if (!bytes || !out) return fail(ctx, SKW_ERR_ARG, "null argument");
  *out = nullptr;
  auto *m = new (std::nothrow) skw_merl();
  if (!m) return fail(ctx, SKW_ERR_OOM, "host allocation");
  m->ctx = ctx;
  if (!skw::merl_load(bytes, n_bytes, m->host)) {
    delete m;
    return fail(ctx, SKW_ERR_ARG, "not a 90 x 90 x 180 MERL BRDF image");
  }
  if (!ctx) {  // host only: for the host entry points, not for scenes
    *out = m;
    return SKW_OK;
  }
  cudaError_t e = cudaSetDevice(ctx->device);
  void *t = nullptr, *sg = nullptr;
  if (e == cudaSuccess) e = cudaMalloc(&t, m->host.table.size() * 2);
  if (e == cudaSuccess) e = cudaMalloc(&sg, m->host.seg.size() * 4);
  if (e == cudaSuccess) e = cudaMemcpy(t, m->host.table.data(), m->host.table.size() * 2, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(sg, m->host.seg.data(), m->host.seg.size() * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(t);
    cudaFree(sg);
    delete m;
    return cuda_fail(ctx, e, "measured BRDF upload");
  }
  m->dev.table = (const uint16_t *)t;
  m->dev.seg = (const float *)sg;
  *out = m;
  return SKW_OK;
}

void skw_merl_destroy(skw_merl *m) {
  if (!m) return;
  cudaFree((void *)m->dev.table);
  cudaFree((void *)m->dev.seg);
  delete m;
}

int skw_merl_export(const skw_merl *m, uint16_t *table, float *seg) {
  if (!m) return SKW_ERR_ARG;
  if (table) std::copy(m->host.table.begin(), m->host.table.end(), table);
  if (seg) std::copy(m->host.seg.begin(), m->host.seg.end(), seg);
  return SKW_OK;
}

int skw_merl_eval_host(const skw_merl *m, const double *wi, const double *wo, int64_t n, double *f, double *pdf) {
  if (!m || n < 0 || (n > 0 && (!wi || !wo || !f || !pdf))) return SKW_ERR_ARG;
  for (int64_t i = 0; i < n; ++i) skw::merl_eval(m->host, wi + 3 * i, wo + 3 * i, f + 3 * i, pdf + i);
  return SKW_OK;
}

int skw_merl_sample_host(const skw_merl *m, const double *wi, const double *u, int64_t n, double *wo, double *f,
                         double *pdf) {
  if (!m || n < 0 || (n > 0 && (!wi || !u || !wo || !f || !pdf))) return SKW_ERR_ARG;
  for (int64_t i = 0; i < n; ++i) skw::merl_sample(m->host, wi + 3 * i, u + 2 * i, wo + 3 * i, f + 3 * i, pdf + i);
  return SKW_OK;
}

// The device view of a handle, for the scene builder.
skw::MerlDev skw_merl_device_view(const skw_merl *m) { return m ? m->dev : skw::MerlDev{}; }

}  // extern "C"
