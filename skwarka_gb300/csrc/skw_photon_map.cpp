// C ABI (include/skw.h): photon maps -- GPU photon shooting, the three photon
// kd-trees (built on the host for tree identity with the reference) and the
// irradiance photon map (PhotonLTEIntegrator::_ConstructIrradiancePhotonMap,
// LTEIntegrators/PhotonLTEIntegrator/PhotonLTEIntegrator.cpp:171-245).
#include "../../include/skw.h"

#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <functional>
#include <limits>
#include <new>
#include <thread>
#include <vector>

#include "kernels.h"
#include "photon_tree.h"
#include "photon_map_internal.h"
#include "photon_types.h"
#include "skw_internal.h"

using skw::cuda_fail;
using skw::fail;
using skw::PhotonRec;
using Map = skw::PhotonMapData;

namespace {

constexpr double kMaxNormalDeviationCos = 0.87;  // PhotonLTEIntegrator.cpp:26
constexpr int kLookupIrradiance = 100;            // LOOKUP_PHOTONS_NUM_FOR_IRRADIANCE (PhotonLTEIntegrator.h:218)
constexpr int64_t kMaxPhotonsInMap = 40000000;    // MAX_PHOTONS_IN_MAP (PhotonLTEIntegrator.h:224)
constexpr double kInvPi = 0.31830988618379067154;

template <class T>
cudaError_t upload(const std::vector<T> &v, T **out) {
  *out = nullptr;
  const size_t b = std::max<size_t>(v.size(), 1) * sizeof(T);
  cudaError_t e = cudaMalloc((void **)out, b);
  if (e == cudaSuccess && !v.empty()) e = cudaMemcpy(*out, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
  return e;
}

void free_map(Map &m) {
  cudaFree(m.d_nodes);
  cudaFree(m.d_nids);
  cudaFree(m.d_dirid);
  cudaFree(m.d_weight);
  m.d_nodes = nullptr;
  m.d_nids = m.d_dirid = nullptr;
  m.d_weight = nullptr;
}

// KDTree<Photon>(photons) (Core/KDTree.h:428-473): on the GPU where that
// gives the reference's tree (no median ties; build_photon_tree_device),
// else on the host; the photons' attributes in tree order.
cudaError_t build_map(Map &m, cudaStream_t st) {
  m.n = (int64_t)m.input.size();
  const size_t n = (size_t)m.n;
  std::vector<float> pos(n * 3), w(n * 3);
  std::vector<uint16_t> nids(n), dirid(n);
  for (size_t i = 0; i < n; ++i) {
    const PhotonRec &r = m.input[i];
    for (int k = 0; k < 3; ++k) {
      pos[3 * i + k] = r.p[k];
      w[3 * i + k] = r.w[k];
    }
    nids[i] = r.nrm;
    dirid[i] = r.dir;
  }
  skw::KdNode *dn = nullptr;
  int32_t *d_perm = nullptr;
  bool on_gpu = false;
  cudaError_t e = skw::build_photon_tree_device(pos.data(), m.n, st, &dn, m.perm, &d_perm, &on_gpu);
  m.d_nodes = dn;
  m.built_on_gpu = on_gpu;
  if (e == cudaSuccess && on_gpu) {
    // the attributes uploaded in photon order and gathered into tree order
    uint16_t *nin = nullptr, *din = nullptr;
    float *win = nullptr;
    if ((e = upload(nids, &nin)) == cudaSuccess && (e = upload(dirid, &din)) == cudaSuccess &&
        (e = upload(w, &win)) == cudaSuccess && (e = cudaMalloc(&m.d_nids, n * 2)) == cudaSuccess &&
        (e = cudaMalloc(&m.d_dirid, n * 2)) == cudaSuccess && (e = cudaMalloc(&m.d_weight, n * 12)) == cudaSuccess &&
        (e = skw::gather_tree_order(d_perm, m.n, nin, din, win, m.d_nids, m.d_dirid, m.d_weight, st)) ==
            cudaSuccess)
      e = cudaStreamSynchronize(st);
    cudaFree(nin);
    cudaFree(din);
    cudaFree(win);
    cudaFree(d_perm);
    return e;
  }
  cudaFree(d_perm);
  if (e != cudaSuccess) return e;
  std::vector<uint16_t> nt(n), dt(n);
  std::vector<float> wt(n * 3);
  for (size_t t = 0; t < n; ++t) {
    const size_t i = (size_t)m.perm[t];
    nt[t] = nids[i];
    dt[t] = dirid[i];
    for (int k = 0; k < 3; ++k) wt[3 * t + k] = w[3 * i + k];
  }
  if (e == cudaSuccess) e = upload(nt, &m.d_nids);
  if (e == cudaSuccess) e = upload(dt, &m.d_dirid);
  if (e == cudaSuccess) e = upload(wt, &m.d_weight);
  return e;
}

const PhotonRec &tree_photon(const Map &m, int64_t t) { return m.input[(size_t)m.perm[(size_t)t]]; }

// One map's build_map on a host thread and stream of its own, joined (and
// its stream destroyed) on every path out of the caller.
struct SideBuild {
  std::thread worker;
  cudaStream_t s = nullptr;
  cudaError_t e = cudaSuccess;
  bool started = false;
  void start(Map &m, int device) {
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) {
      s = nullptr;  // the caller builds the map in line
      return;
    }
    started = true;
    worker = std::thread([this, &m, device]() {
      e = cudaSetDevice(device);
      if (e == cudaSuccess) e = build_map(m, s);
    });
  }
  cudaError_t finish() {
    if (worker.joinable()) worker.join();
    return e;
  }
  ~SideBuild() {
    if (worker.joinable()) worker.join();
    if (s) cudaStreamDestroy(s);
  }
};

// Device buffers of the irradiance construction, freed on every path.
struct IrrBuffers {
  double *q = nullptr, *qn = nullptr, *sq = nullptr, *sqn = nullptr;
  int32_t *idx[3] = {nullptr, nullptr, nullptr}, *cnt[3] = {nullptr, nullptr, nullptr};
  double *d2[3] = {nullptr, nullptr, nullptr};
  float *ext = nullptr, *intr = nullptr;
  int32_t *near = nullptr;
  cudaStream_t side[2] = {nullptr, nullptr};
  cudaEvent_t fork = nullptr, join[2] = {nullptr, nullptr};
  ~IrrBuffers() {
    for (void *p : {(void *)q, (void *)qn, (void *)sq, (void *)sqn, (void *)ext, (void *)intr, (void *)near}) cudaFree(p);
    for (int i = 0; i < 3; ++i) {
      cudaFree(idx[i]);
      cudaFree(cnt[i]);
      cudaFree(d2[i]);
    }
    for (int i = 0; i < 2; ++i) {
      if (side[i]) cudaStreamDestroy(side[i]);
      if (join[i]) cudaEventDestroy(join[i]);
    }
    if (fork) cudaEventDestroy(fork);
  }
};

// The maps' kd-trees and _ConstructIrradiancePhotonMap: every 10th indirect
// photon (in tree order) becomes an irradiance photon whose irradiance is
// estimated from the three maps; then the 0.1 % percentile of the distance
// from every 11th indirect photon to its nearest irradiance photon bounds
// the irradiance lookups.
//
// The work is one pipeline.  The indirect map's tree is built first (the
// irradiance photons are its photons); its lookups start on a side stream
// while the host builds the direct and caustic trees, whose lookups start
// on a second side stream as each is uploaded; the irradiance photons' own
// tree (built from their positions alone) and the lookup-distance queries
// run on the caller's stream meanwhile.  The three maps' estimates are then
// added on the caller's stream in map order (caustic, direct, indirect), so
// every float sum is the one the sequential construction makes.
int build_maps(skw_photon_map *pm, cudaStream_t st) {
  skw_ctx *ctx = pm->ctx;
  Map &im = pm->maps[2];
  // the direct map's tree (the largest; a host repair where its medians
  // tie) on a thread of its own while the indirect map's is built and its
  // irradiance photons set up
  SideBuild direct;
  if (!im.input.empty() && !pm->maps[1].input.empty()) direct.start(pm->maps[1], ctx->device);
  cudaError_t e = build_map(im, st);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "photon map upload");
  if (im.n == 0) {  // no indirect map: no irradiance photons
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = build_map(pm->maps[i], st);
    return e == cudaSuccess ? SKW_OK : cuda_fail(ctx, e, "photon map upload");
  }
  const std::vector<double> &dirs = skw::direction_table();
  for (int64_t i = 0; i < im.n; i += 10) {
    const PhotonRec &r = tree_photon(im, i);
    pm->irr_pos.insert(pm->irr_pos.end(), r.p, r.p + 3);
    pm->irr_nrm.push_back(r.nrm);
  }
  const int64_t nq = (int64_t)pm->irr_nrm.size();
  const int64_t nd = (int64_t)pm->maps[1].input.size(), nc = (int64_t)pm->maps[0].input.size();
  const double da = nd == 0 ? 0.0 : pm->scene_area / nd;
  const double ia = pm->scene_area / im.n;
  pm->lookup_dist[1] = std::sqrt(da * kLookupIrradiance * kInvPi);
  pm->lookup_dist[2] = std::sqrt(ia * kLookupIrradiance * kInvPi);
  pm->lookup_dist[0] = std::max(pm->lookup_dist[1], pm->lookup_dist[2]);
  std::vector<double> q((size_t)nq * 3), qn((size_t)nq * 3);
  for (int64_t i = 0; i < nq; ++i)
    for (int k = 0; k < 3; ++k) {
      q[(size_t)(3 * i + k)] = (double)pm->irr_pos[(size_t)(3 * i + k)];
      qn[(size_t)(3 * i + k)] = dirs[3 * (size_t)pm->irr_nrm[(size_t)i] + k];
    }
  // queries of the lookup-distance percentile: every 11th indirect photon
  const int64_t step = 11, ns = (im.n + step - 1) / step;
  std::vector<double> sq((size_t)ns * 3), sqn((size_t)ns * 3);
  for (int64_t i = 0; i < ns; ++i) {
    const PhotonRec &r = tree_photon(im, i * step);
    for (int k = 0; k < 3; ++k) {
      sq[(size_t)(3 * i + k)] = (double)r.p[k];
      sqn[(size_t)(3 * i + k)] = dirs[3 * (size_t)r.nrm + k];
    }
  }
  // Lookups in chunks of queries (k-NN output is 12 bytes per neighbour),
  // each map's into its own buffers.
  const int64_t chunk = std::min<int64_t>(nq, (int64_t)1 << 20);
  const bool has[3] = {nc > 0, nd > 0, true};
  IrrBuffers B;
  e = cudaMalloc(&B.q, (size_t)nq * 24);
  if (e == cudaSuccess) e = cudaMalloc(&B.qn, (size_t)nq * 24);
  for (int mi = 0; mi < 3 && e == cudaSuccess; ++mi) {
    if (!has[mi]) continue;
    if ((e = cudaMalloc(&B.idx[mi], (size_t)chunk * kLookupIrradiance * 4)) == cudaSuccess &&
        (e = cudaMalloc(&B.d2[mi], (size_t)chunk * kLookupIrradiance * 8)) == cudaSuccess)
      e = cudaMalloc(&B.cnt[mi], (size_t)chunk * 4);
  }
  if (e == cudaSuccess) e = cudaMalloc(&B.ext, (size_t)nq * 12);
  if (e == cudaSuccess) e = cudaMalloc(&B.intr, (size_t)nq * 12);
  if (e == cudaSuccess) e = cudaMalloc(&B.sq, (size_t)ns * 24);
  if (e == cudaSuccess) e = cudaMalloc(&B.sqn, (size_t)ns * 24);
  if (e == cudaSuccess) e = cudaMalloc(&B.near, (size_t)ns * 4);
  for (int i = 0; i < 2 && e == cudaSuccess; ++i)
    if ((e = cudaStreamCreateWithFlags(&B.side[i], cudaStreamNonBlocking)) == cudaSuccess)
      e = cudaEventCreateWithFlags(&B.join[i], cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&B.fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaMemcpy(B.q, q.data(), (size_t)nq * 24, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(B.qn, qn.data(), (size_t)nq * 24, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(B.sq, sq.data(), (size_t)ns * 24, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(B.sqn, sqn.data(), (size_t)ns * 24, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "irradiance photon buffers");
  std::vector<float> ext((size_t)nq * 3), intr((size_t)nq * 3);
  std::vector<int32_t> nearest((size_t)ns);
  std::vector<int32_t> irr_perm;
  // side stream of each map's lookups: the indirect map's alone, the
  // caustic and direct maps' together
  const int side_of[3] = {1, 1, 0};
  for (int64_t q0 = 0; q0 < nq && e == cudaSuccess; q0 += chunk) {
    const int64_t c = std::min(chunk, nq - q0);
    if ((e = cudaEventRecord(B.fork, st)) != cudaSuccess) break;
    for (int i = 0; i < 2 && e == cudaSuccess; ++i) e = cudaStreamWaitEvent(B.side[i], B.fork, 0);
    for (int mi : {2, 1, 0}) {  // the indirect map's tree exists; the others are built as they are needed
      if (e != cudaSuccess) break;
      Map &m = pm->maps[mi];
      if (q0 == 0 && mi != 2 && (e = mi == 1 && direct.started ? direct.finish() : build_map(m, st)) != cudaSuccess)
        break;
      if (!has[mi]) continue;
      e = skw::launch_knn(m.d_nodes, m.d_nids, pm->d_dirs, (int)m.n, B.q + 3 * q0, B.qn + 3 * q0, c,
                          kLookupIrradiance, pm->lookup_dist[mi], kMaxNormalDeviationCos, B.idx[mi], B.d2[mi],
                          B.cnt[mi], nullptr, nullptr, pm->d_status, B.side[side_of[mi]]);
    }
    if (e == cudaSuccess && q0 == 0) {
      // KDTree<IrradiancePhoton>(irradiance_photons) on the positions, and
      // the lookup-distance queries against it, on the caller's stream
      std::vector<skw::KdNode> nodes;
      skw::build_photon_tree(pm->irr_pos.data(), nq, 0, nodes, irr_perm);
      std::vector<uint16_t> nrm_t((size_t)nq);
      for (int64_t t = 0; t < nq; ++t) nrm_t[(size_t)t] = pm->irr_nrm[(size_t)irr_perm[(size_t)t]];
      skw::KdNode *dn = nullptr;
      e = upload(nodes, &dn);
      pm->d_irr_nodes = dn;
      if (e == cudaSuccess) e = upload(nrm_t, &pm->d_irr_nids);
      if (e == cudaSuccess)
        e = skw::launch_nearest(pm->d_irr_nodes, pm->d_irr_nids, pm->d_dirs, (int)nq, B.sq, B.sqn, ns,
                                std::numeric_limits<double>::infinity(), kMaxNormalDeviationCos, B.near,
                                pm->d_status, st);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(nearest.data(), B.near, (size_t)ns * 4, cudaMemcpyDeviceToHost, st);
    }
    for (int i = 0; i < 2 && e == cudaSuccess; ++i)
      if ((e = cudaEventRecord(B.join[i], B.side[i])) == cudaSuccess) e = cudaStreamWaitEvent(st, B.join[i], 0);
    bool first = true;
    for (int mi = 0; mi < 3 && e == cudaSuccess; ++mi) {
      if (!has[mi]) continue;  // a null map adds nothing
      const Map &m = pm->maps[mi];
      e = skw::launch_irradiance_sum(m.d_nodes, m.d_weight, m.d_dirid, pm->d_dirs, B.q + 3 * q0, B.qn + 3 * q0,
                                     B.idx[mi], B.cnt[mi], c, kLookupIrradiance, (double)m.paths,
                                     pm->lookup_dist[mi], first, B.ext + 3 * q0, B.intr + 3 * q0, st);
      first = false;
    }
  }
  if (e == cudaSuccess) e = cudaMemcpyAsync(ext.data(), B.ext, (size_t)nq * 12, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(intr.data(), B.intr, (size_t)nq * 12, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "irradiance photon estimates");
  // the irradiance photons in their tree's order
  std::vector<float> pos_t((size_t)nq * 3), ext_t((size_t)nq * 3), int_t((size_t)nq * 3);
  std::vector<uint16_t> nrm_t((size_t)nq);
  for (int64_t t = 0; t < nq; ++t) {
    const int32_t s = irr_perm[(size_t)t];
    for (int k = 0; k < 3; ++k) {
      pos_t[(size_t)(3 * t + k)] = pm->irr_pos[(size_t)(3 * s + k)];
      ext_t[(size_t)(3 * t + k)] = ext[(size_t)(3 * s + k)];
      int_t[(size_t)(3 * t + k)] = intr[(size_t)(3 * s + k)];
    }
    nrm_t[(size_t)t] = pm->irr_nrm[(size_t)s];
  }
  pm->irr_pos.swap(pos_t);
  pm->irr_nrm.swap(nrm_t);
  pm->irr_ext.swap(ext_t);
  pm->irr_int.swap(int_t);
  pm->n_irr = nq;
  e = upload(pm->irr_ext, &pm->d_irr_ext);
  if (e == cudaSuccess) e = upload(pm->irr_int, &pm->d_irr_int);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "irradiance map upload");
  std::vector<double> d2((size_t)ns, 0.0);
  for (int64_t i = 0; i < ns; ++i) {
    const int32_t t = nearest[(size_t)i];
    if (t < 0) continue;  // no irradiance photon: 0 keeps it out of the percentile
    double s = 0.0;
    for (int k = 0; k < 3; ++k) {
      const double d = sq[(size_t)(3 * i + k)] - (double)pm->irr_pos[(size_t)(3 * t + k)];
      s += d * d;
    }
    d2[(size_t)i] = s;
  }
  const size_t index = d2.size() <= 1 ? 0 : std::max(d2.size() / 1000, (size_t)1);
  std::nth_element(d2.begin(), d2.begin() + (ptrdiff_t)index, d2.end(), std::greater<double>());
  pm->max_irr_dist = d2[index] == 0.0 ? std::numeric_limits<double>::infinity() : std::sqrt(d2[index]);
  return SKW_OK;
}

int finish_map(skw_photon_map *pm, cudaStream_t st) {
  const auto t0 = std::chrono::steady_clock::now();
  cudaError_t e = cudaSetDevice(pm->ctx->device);
  const std::vector<double> &dirs = skw::direction_table_device();
  if (e == cudaSuccess) e = upload(dirs, &pm->d_dirs);
  if (e == cudaSuccess) e = cudaMalloc(&pm->d_status, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemset(pm->d_status, 0, sizeof(unsigned));
  if (e != cudaSuccess) return cuda_fail(pm->ctx, e, "photon map upload");
  int rc = build_maps(pm, st);
  pm->build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}

}  // namespace

extern "C" {

int skw_photon_map_create(skw_ctx *ctx, const skw_photon *const *photons, const int64_t *n, const int64_t *paths,
                          double scene_area, skw_photon_map **out) {
  if (!ctx || !photons || !n || !paths || !out) return fail(ctx, SKW_ERR_ARG, "null argument");
  *out = nullptr;
  if (!(scene_area >= 0.0)) return fail(ctx, SKW_ERR_ARG, "scene_area must be >= 0");
  for (int i = 0; i < 3; ++i) {
    if (n[i] < 0 || n[i] > kMaxPhotonsInMap || (n[i] > 0 && !photons[i]) || paths[i] < 0)
      return fail(ctx, SKW_ERR_ARG, "bad photon array");
  }
  if (n[2] > 0 && n[1] == 0) return fail(ctx, SKW_ERR_ARG, "an indirect map needs a direct map");
  auto *pm = new (std::nothrow) skw_photon_map();
  if (!pm) return fail(ctx, SKW_ERR_OOM, "host allocation");
  pm->ctx = ctx;
  pm->scene_area = scene_area;
  for (int i = 0; i < 3; ++i) {
    const PhotonRec *p = reinterpret_cast<const PhotonRec *>(photons[i]);
    pm->maps[i].input.assign(p, p + n[i]);
    pm->maps[i].paths = paths[i];
  }
  int rc = finish_map(pm, nullptr);
  if (rc != SKW_OK) {
    skw_photon_map_destroy(pm);
    return rc;
  }
  *out = pm;
  return SKW_OK;
}

int skw_photon_shoot(skw_scene *s, const skw_photon_params *params, skw_photon_map **out) {
  if (!s || !params || !out) return fail(s ? s->ctx : nullptr, SKW_ERR_ARG, "null argument");
  skw_ctx *ctx = s->ctx;
  *out = nullptr;
  if (params->paths <= 0 || params->paths > ((int64_t)1 << 31) || params->max_bounces < 1 ||
      params->max_bounces > 1024 || !(params->rr_probability >= 0.0f) || params->rr_probability > 1.0f)
    return fail(ctx, SKW_ERR_ARG, "bad photon parameters");
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaSetDevice");
  const auto t0 = std::chrono::steady_clock::now();
  // Lights by the luminance of their power (PhotonLTEIntegrator.cpp:80-125):
  // PointLight::Power = 4 pi I, DiffuseAreaLightSource::Power = pi A L.
  const skw::SceneDev &S = s->dev;
  std::vector<skw::PointLightDev> pls((size_t)S.n_point_lights);
  std::vector<skw::AreaLight> als((size_t)S.n_area_lights);
  if (!pls.empty()) e = cudaMemcpy(pls.data(), S.point_lights, pls.size() * sizeof(pls[0]), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && !als.empty())
    e = cudaMemcpy(als.data(), S.area_lights, als.size() * sizeof(als[0]), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "light table");
  const double lw[3] = {0.05316285, 0.58515348, 0.36168367};
  std::vector<skw::PhotonLight> lights;
  std::vector<double> power;
  for (size_t i = 0; i < pls.size(); ++i) {
    double p = 0;
    for (int k = 0; k < 3; ++k) p += lw[k] * 4.0 * M_PI * pls[i].intensity[k];
    lights.push_back({0.0, 0, (int32_t)i});
    power.push_back(p);
  }
  for (size_t i = 0; i < als.size(); ++i) {
    double p = 0;
    for (int k = 0; k < 3; ++k) p += lw[k] * M_PI * als[i].area * als[i].radiance[k] * S.emission_scale;
    lights.push_back({0.0, 1, (int32_t)i});
    power.push_back(p);
  }
  if (lights.empty()) return fail(ctx, SKW_ERR_ARG, "the scene has no lights");
  for (size_t i = 1; i < power.size(); ++i) power[i] += power[i - 1];
  const double total = power.back();
  for (size_t i = 0; i < power.size(); ++i) lights[i].cdf = total > 2.220446049250313e-16 ? power[i] / total : 0.0;
  if (!(total > 2.220446049250313e-16)) lights.back().cdf = 1.0;
  skw::PhotonLight *d_lights = nullptr;
  if ((e = upload(lights, &d_lights)) != cudaSuccess) return cuda_fail(ctx, e, "light table");
  // Indirect photons are staged in per-path slots, so that the chunk's
  // photons come out in path order; 63 slots cover every path of a scene
  // whose paths end by Russian roulette (a path of 64 bounces survives with
  // probability ~p^63).  A chunk where a path needs more is shot again in
  // sub-chunks with a slot for every bounce.
  const int full_slots = std::max(params->max_bounces - 1, 1);
  const int slots = std::min(full_slots, 63);
  skw::PhotonShootArgs A{d_lights, (int32_t)lights.size(), params->max_bounces, params->rr_probability, params->seed,
                         slots, nullptr};
  skw_accel *a = s->accel;
  skw::TraceFn trace = [a](const void *rays, int64_t n, const int *n_dev, void *hits, cudaStream_t st, int *work) {
    return skw::launch_traversal(true, a->stack_cap, a->d_nodes, a->d_tris, rays, n, n_dev, a->scene_abs, nullptr,
                                 hits, a->d_status, st, 0, work, true);
  };
  // 2^20 paths per chunk with 63 indirect slots each; a re-shot chunk (every
  // slot) runs in sub-chunks of the same workspace size
  const int64_t chunk = std::min<int64_t>(
      params->paths, std::max<int64_t>((int64_t)1 << 12, ((int64_t)1 << 26) / std::max(slots + 1, 64)));
  const int64_t sub = std::max<int64_t>((int64_t)1 << 12, ((int64_t)1 << 26) / std::max(full_slots + 1, 64));
  const int64_t B1 = std::max<int64_t>(std::max((int64_t)chunk * slots, std::min(chunk, sub) * full_slots), 1);
  void *ws = nullptr;
  PhotonRec *d_dir = nullptr, *d_ind = nullptr, *d_cau = nullptr;
  int *d_tot = nullptr;
  cudaStream_t st = nullptr;
  e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
  const size_t wsb = std::max(skw::photon_chunk_bytes(chunk, slots), skw::photon_chunk_bytes(std::min(chunk, sub), full_slots));
  if (e == cudaSuccess) e = cudaMalloc(&ws, wsb);
  if (e == cudaSuccess) e = cudaMalloc((void **)&d_dir, (size_t)chunk * sizeof(PhotonRec));
  if (e == cudaSuccess) e = cudaMalloc((void **)&d_ind, (size_t)B1 * sizeof(PhotonRec));
  if (e == cudaSuccess) e = cudaMalloc((void **)&d_cau, (size_t)chunk * sizeof(PhotonRec));
  if (e == cudaSuccess) e = cudaMalloc(&d_tot, 4 * sizeof(int));
  A.overflow = d_tot + 3;
  auto *pm = new (std::nothrow) skw_photon_map();
  if (!pm) e = cudaErrorMemoryAllocation;
  int64_t launches = 0;
  // One chunk [p0, p0 + n) with the given slots; its photons appended to the
  // maps unless a path overflowed its slots (*overflowed set, nothing kept).
  auto shoot = [&](int64_t p0, int n, int sl, bool *overflowed) -> cudaError_t {
    skw::PhotonShootArgs a = A;
    a.slots = sl;
    cudaError_t r = cudaMemsetAsync(d_tot + 3, 0, sizeof(int), st);
    if (r == cudaSuccess) r = skw::photon_shoot_chunk(S, a, trace, p0, n, ws, d_dir, d_ind, d_cau, d_tot, st);
    int tot[4] = {0, 0, 0, 0};
    if (r == cudaSuccess) r = cudaMemcpyAsync(tot, d_tot, sizeof(tot), cudaMemcpyDeviceToHost, st);
    if (r == cudaSuccess) r = cudaStreamSynchronize(st);
    if (r != cudaSuccess) return r;
    launches += 1 + 2 * params->max_bounces + 9;
    *overflowed = tot[3] != 0;
    if (*overflowed) return cudaSuccess;
    Map &cm = pm->maps[0], &dm = pm->maps[1], &im = pm->maps[2];
    const size_t oc = cm.input.size(), od = dm.input.size(), oi = im.input.size();
    cm.input.resize(oc + (size_t)tot[2]);
    dm.input.resize(od + (size_t)tot[0]);
    im.input.resize(oi + (size_t)tot[1]);
    if (tot[0] > 0) r = cudaMemcpy(dm.input.data() + od, d_dir, (size_t)tot[0] * sizeof(PhotonRec), cudaMemcpyDeviceToHost);
    if (r == cudaSuccess && tot[1] > 0)
      r = cudaMemcpy(im.input.data() + oi, d_ind, (size_t)tot[1] * sizeof(PhotonRec), cudaMemcpyDeviceToHost);
    if (r == cudaSuccess && tot[2] > 0)
      r = cudaMemcpy(cm.input.data() + oc, d_cau, (size_t)tot[2] * sizeof(PhotonRec), cudaMemcpyDeviceToHost);
    cm.paths += n;
    dm.paths += n;
    im.paths += n;
    return r;
  };
  for (int64_t p0 = 0; p0 < params->paths && e == cudaSuccess; p0 += chunk) {
    const int n = (int)std::min(chunk, params->paths - p0);
    bool over = false;
    e = shoot(p0, n, slots, &over);
    // a path deposited more than `slots` indirect photons: the chunk again,
    // in sub-chunks with a slot for every bounce
    for (int64_t q0 = p0; over && e == cudaSuccess && q0 < p0 + n; q0 += sub) {
      bool again = false;
      e = shoot(q0, (int)std::min<int64_t>(sub, p0 + n - q0), full_slots, &again);
    }
  }
  cudaFree(ws);
  cudaFree(d_dir);
  cudaFree(d_ind);
  cudaFree(d_cau);
  cudaFree(d_tot);
  cudaFree(d_lights);
  if (e != cudaSuccess) {
    if (st) cudaStreamDestroy(st);
    skw_photon_map_destroy(pm);
    return cuda_fail(ctx, e, "photon shooting");
  }
  ctx->launches.fetch_add(launches);
  pm->ctx = ctx;
  pm->scene_area = s->total_area;
  pm->shoot_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  for (int i = 0; i < 3; ++i)
    if ((int64_t)pm->maps[i].input.size() > kMaxPhotonsInMap) {
      cudaStreamDestroy(st);
      skw_photon_map_destroy(pm);
      return fail(ctx, SKW_ERR_BUDGET, "a photon map exceeds 40M photons (the reference's MAX_PHOTONS_IN_MAP)");
    }
  for (int i = 0; i < 3; ++i)
    if (pm->maps[i].input.empty()) pm->maps[i].paths = 0;
  int rc = finish_map(pm, st);
  cudaStreamDestroy(st);
  if (rc != SKW_OK) {
    skw_photon_map_destroy(pm);
    return rc;
  }
  *out = pm;
  return SKW_OK;
}

void skw_photon_map_destroy(skw_photon_map *pm) {
  if (!pm) return;
  for (Map &m : pm->maps) free_map(m);
  cudaFree(pm->d_irr_nodes);
  cudaFree(pm->d_irr_nids);
  cudaFree(pm->d_irr_ext);
  cudaFree(pm->d_irr_int);
  cudaFree(pm->d_dirs);
  cudaFree(pm->d_status);
  delete pm;
}

int skw_photon_map_get_info(const skw_photon_map *pm, skw_photon_map_info *out) {
  if (!pm || !out) return SKW_ERR_ARG;
  std::memset(out, 0, sizeof(*out));
  out->n_caustic = pm->maps[0].n;
  out->n_direct = pm->maps[1].n;
  out->n_indirect = pm->maps[2].n;
  out->n_irradiance = pm->n_irr;
  out->paths_caustic = pm->maps[0].paths;
  out->paths_direct = pm->maps[1].paths;
  out->paths_indirect = pm->maps[2].paths;
  out->max_irradiance_lookup_dist = pm->max_irr_dist;
  out->scene_area = pm->scene_area;
  out->shoot_ms = pm->shoot_ms;
  out->build_ms = pm->build_ms;
  out->trees_on_gpu = 0;
  for (int i = 0; i < 3; ++i)
    if (pm->maps[i].built_on_gpu) out->trees_on_gpu |= 1 << i;
  return SKW_OK;
}

int skw_photon_map_export(const skw_photon_map *pm, int32_t which, skw_photon *out) {
  if (!pm || which < 0 || which > 2 || (!out && pm->maps[which].n > 0)) return SKW_ERR_ARG;
  const Map &m = pm->maps[which];
  if (m.n > 0) std::memcpy(out, m.input.data(), (size_t)m.n * sizeof(PhotonRec));
  return SKW_OK;
}

int skw_photon_map_export_irradiance(const skw_photon_map *pm, float *pos, float *ext, float *intr, uint16_t *nrm) {
  if (!pm) return SKW_ERR_ARG;
  const size_t n = (size_t)pm->n_irr;
  if (n == 0) return SKW_OK;
  if (!pos || !ext || !intr || !nrm) return SKW_ERR_ARG;
  std::memcpy(pos, pm->irr_pos.data(), n * 12);
  std::memcpy(ext, pm->irr_ext.data(), n * 12);
  std::memcpy(intr, pm->irr_int.data(), n * 12);
  std::memcpy(nrm, pm->irr_nrm.data(), n * 2);
  return SKW_OK;
}

}  // extern "C"
