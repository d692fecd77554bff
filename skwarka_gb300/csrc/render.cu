// Wavefront direct-lighting renderer on sm_103a.
//
// Restates the reference's sampler-based direct-lighting render
// (Renderers/SamplerBasedRenderer.cpp:419-491,
// LTEIntegrators/DirectLightingLTEIntegrator.cpp:33-60,
// Core/DirectLightingIntegrator.cpp:54-366) as stages over ray queues:
//
//   k_camera   pinhole camera rays (Cameras/PerspectiveCamera.cpp:36-65),
//              stratified pixel samples (Samplers/StratifiedSampler.cpp:57-100)
//   k_trace    closest hit (traverse.cu)
//   k_shade    differential geometry of the hit (TriangleMesh.cpp:439-561,
//              shading normal interpolated from vertex normals), BSDF
//              assembly (Materials), emission of a hit area light, light
//              sampling (DiffuseAreaLightSource::SampleLighting,
//              PointLight::Lighting) and BSDF sampling (BSDF::Sample), each
//              weighted with the power heuristic; shadow rays and BSDF rays
//              are appended to compacted queues (one atomic per warp)
//   k_trace    any hit for the shadow queue, closest hit for the BSDF queue
//   k_resolve_shadow / k_resolve_bsdf  write each contribution to its own
//              slot (emission, light samples, point lights, BSDF samples)
//   k_film     per pixel: each sample's slots are summed in a fixed order,
//              a NaN, negative or infinite sample counts as black
//              (SamplerBasedRenderer.cpp:458-478), and the box-filtered film
//              (ImageFilm.cpp:32-57, BoxFilter width 0.5: every sample lands
//              in its own pixel with weight 1) averages them.
//
// Arithmetic is float; the reference computes in double.  The estimator
// (sampling densities, MIS weights, BSDF and light formulas) is the same, so
// the images agree in expectation; the random numbers differ (a
// counter-based hash of seed, sample and dimension replaces the reference's
// per-thread Mersenne Twister), so parity is statistical.
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>

#include "kernels.h"
#include "render_device.cuh"
#include "render_scene.h"

namespace skw {
namespace {


// The view holding global pixel P: the last view whose first pixel is <= P.
__device__ __forceinline__ int find_view(const ViewDev *__restrict__ views, int n_views, int64_t P) {
  int lo = 0, hi = n_views - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (views[mid].px_begin <= P) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Camera rays for the samples of global pixels [px_begin, px_begin + n_px):
// PerspectiveCamera::GenerateRay (PerspectiveCamera.cpp:36-65; pinhole) in
// float -- the rays are stored as floats, so double arithmetic would only
// round differently, and GB300 runs it at ~1/64 of the float rate -- with
// 32-bit index arithmetic (a pass holds fewer than 2^31 samples).
__global__ void k_camera(const ViewDev *__restrict__ views, int n_views, int64_t px_begin, int n_px, int sppx,
                         int sppy, int ld, float4 *__restrict__ rays) {
  const uint32_t spp = (uint32_t)(sppx * sppy);
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= (uint32_t)n_px * spp) return;
  const uint32_t pl = s / spp, j = s - pl * spp;
  const int64_t P = px_begin + pl;
  const int v = find_view(views, n_views, P);
  const CameraDev &cam = views[v].cam;
  const uint32_t px = (uint32_t)(P - views[v].px_begin), w = (uint32_t)cam.width;
  const uint32_t y = px / w, x = px - y * w;
  const uint64_t gid = (uint64_t)px * spp + j, seed = views[v].seed;
  float ix, iy;
  if (ld) {
    // LDSampler image points: one scrambled (0,2)-sequence point per sample
    float u0, u1;
    ld_2d(seed, (uint64_t)px, 0, j, spp, 0, 1, u0, u1);
    ix = (float)x + u0;
    iy = (float)y + u1;
  } else {
    // stratified, jittered pixel sample (StratifiedSampling2D)
    const uint32_t jy = j / (uint32_t)sppx, jx = j - jy * (uint32_t)sppx;
    ix = (float)x + ((float)jx + rnd(seed, gid, 0)) / (float)sppx;
    iy = (float)y + ((float)jy + rnd(seed, gid, 1)) / (float)sppy;
  }
  const float cx = cam.sx * (ix - 0.5f * (float)cam.width);
  const float cy = cam.sy * (iy - 0.5f * (float)cam.height);
  const float *m = cam.m;
  float dx = m[0] * cx + m[1] * cy + m[2];
  float dy = m[4] * cx + m[5] * cy + m[6];
  float dz = m[8] * cx + m[9] * cy + m[10];
  const float il = 1.0f / sqrtf(dx * dx + dy * dy + dz * dz);
  dx *= il;
  dy *= il;
  dz *= il;
  rays[2 * (uint64_t)s] = make_float4(m[3], m[7], m[11], dx);
  rays[2 * (uint64_t)s + 1] = make_float4(dy, dz, 0.0f, __int_as_float(0x7f800000));
}

// The specular tree of a camera sample (LTEIntegrator::_SpecularReflect /
// _SpecularTransmit, Core/LTEIntegrator.cpp:66-126, called from
// DirectLightingLTEIntegrator::_SurfaceRadiance while the ray's specular
// depth <= m_max_specular_depth): a hit on a specular material sends a
// reflected and a transmitted ray, each weighted by its BxDF value.  The
// rays of one depth form a queue (ray, RGB weight, camera sample, node); a
// node numbers the ray in the sample's binary tree (camera ray 1, children
// 2k and 2k + 1) and selects its random stream.  Shading a queue entry
// adds weight x (emission + direct lighting) to the sample's specular slot
// with atomics (so the last bits of that slot depend on the order).
// Grid of the kernels of a specular level (grid-stride loops over the
// level's queue, whose capacity is far above its usual length).
constexpr int64_t kStrideBlocks = 2048;

struct SpecArgs {
  // input (SPEC): entries [0, min(*in_count, n)) of a level
  const float *in_w;
  const int *in_sample;
  const int *in_node;
  const int *in_count;
  // output: the children of the shaded rays (null out_count: none)
  float4 *out_rays;
  float *out_w;
  int *out_sample;
  int *out_node;
  int *out_count;
  int depth;      // specular depth of the rays shaded here (camera rays: 0)
  int spec_slot;  // slot of a sample that the specular levels add into
};

__device__ __forceinline__ void atomic_add_rgb(float *c, int64_t slot, V3 v) {
  if (v.x != 0.0f) atomicAdd(c + 3 * slot, v.x);
  if (v.y != 0.0f) atomicAdd(c + 3 * slot + 1, v.y);
  if (v.z != 0.0f) atomicAdd(c + 3 * slot + 2, v.z);
}

struct ShadeArgs {
  int n;               // samples in this pass
  int64_t px_begin;    // global pixel of the pass's first sample
  int spp;
  int slots;           // contribution slots per sample
  int n_light_samples;
  const ViewDev *views;
  int n_views;
  const float *tcam;   // per sample: transmittance of the camera ray's medium segment (null: no medium)
  int ld;              // camera level: light and BSDF samples from the LDSampler's sequences
};

// The random numbers of light sample k (light choice uc, position u0, u1)
// or BSDF sample k (component uc, direction u0, u1) of a camera-level
// entry: the LDSampler's four sequences (light 1D, light 2D, BSDF 1D, BSDF
// 2D; DirectLightingIntegrator.cpp:41-50) or the counter-based stream.
__device__ __forceinline__ void direct_sample(const ShadeArgs &A, bool ld, uint64_t seed, uint64_t gid, bool bsdf,
                                              int k, float &uc, float &u0, float &u1) {
  const int nl = A.n_light_samples;
  if (ld) {
    const uint32_t spp = (uint32_t)A.spp, j = (uint32_t)(gid % spp);
    const uint64_t px = gid / spp;
    uc = ld_1d(seed, px, bsdf ? 3 : 1, j, spp, (uint32_t)k, (uint32_t)nl);
    ld_2d(seed, px, bsdf ? 4 : 2, j, spp, (uint32_t)k, (uint32_t)nl, u0, u1);
    return;
  }
  const uint32_t d = bsdf ? 2 + 3 * nl + 3 * k : 2 + 3 * k;
  uc = rnd(seed, gid, d);
  u0 = rnd(seed, gid, d + 1);
  u1 = rnd(seed, gid, d + 2);
}

// Adjoint pass (ADJ = true).  The same rays as the forward pass are traced
// (same random numbers), but instead of radiance each queued ray carries the
// derivatives of its contribution, already multiplied by dL/dI of its pixel
// divided by spp:
//   shadow entry q: s_tri[q] (global triangle of the shading point),
//     s_dkd[3q..] = dI * d(contribution)/d(kd), s_dem[q] = dI . d(contribution)/d(emission scale);
//   BSDF entry q: b_tri[q], b_dkd[3q..] = dI * d(f |cos| / (pdf n))/d(kd),
//     brgb[4q..] = (dI * f |cos| / (pdf n), pdf); the light's radiance and
//     MIS weight multiply both when the ray is resolved.
struct AdjointArgs {
  const float *dfilm;   // dL/dI, 3 floats per global pixel
  float *g_albedo;      // accumulated dL/d(triangle albedo), 3 floats per global triangle
  double *g_emission;   // accumulated dL/d(emission scale)
  float *s_dkd, *s_dem, *b_dkd;
};

__device__ __forceinline__ void add_emission_grad(double *g, float v) {
  // warp sum, then one atomic per warp
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v != 0.0f) atomicAdd(g, (double)v);
}

// Per camera hit: emission, light samples, point lights and BSDF samples
// (DirectLightingLTEIntegrator::_SurfaceRadiance with
// DirectLightingIntegrator::ComputeDirectLighting).
// SPEC = false: the camera rays of a pass (entry i = sample i, each term in
// its own slot); SPEC = true: a specular level (entry i of the level's
// queue, every term weighted and added into its sample's specular slot).
// KIDS: queue the specular children of the shaded hits into Q.out_*.
template <bool ADJ, bool SPEC, bool KIDS>
__global__ void __launch_bounds__(128) k_shade(SceneDev S, ShadeArgs A, AdjointArgs J, SpecArgs Q,
                                               const float4 *__restrict__ rays, const int4 *__restrict__ hits,
                                               float *__restrict__ contrib, float4 *__restrict__ srays,
                                               int *__restrict__ starget, float *__restrict__ srgb,
                                               int *__restrict__ scount, float4 *__restrict__ brays,
                                               int *__restrict__ btarget, float *__restrict__ brgb,
                                               int *__restrict__ bcount, float *__restrict__ bnrm) {
  // One entry per thread and iteration; a specular level's grid is capped
  // and strides over the level (the trip count is uniform in a block).
  const int n_eff = SPEC ? min(*Q.in_count, A.n) : A.n;
  for (int i0 = blockIdx.x * blockDim.x; i0 < n_eff; i0 += gridDim.x * blockDim.x) {
  const int i = i0 + threadIdx.x;
  const bool valid = i < n_eff;
  int4 hit = make_int4(0x7f800000, -1, -1, 0);
  float4 ra = make_float4(0, 0, 0, 0), rb = make_float4(0, 0, 0, 0);
  int si = valid ? i : 0;  // camera sample of the entry
  unsigned node = 1;       // the entry's node in its sample's specular tree
  V3 wt = v3(1.0f, 1.0f, 1.0f);
  if (valid) {
    hit = hits[i];
    ra = rays[2 * i];
    rb = rays[2 * i + 1];
    if (SPEC) {
      si = Q.in_sample[i];
      node = (unsigned)Q.in_node[i];
      wt = load3(Q.in_w + 3 * (int64_t)i);
    }
  }
  const bool surface = valid && hit.y >= 0;
  const int nl = A.n_light_samples;
  const int64_t slot0 = (int64_t)si * A.slots;
  const int64_t tslot = slot0 + Q.spec_slot;  // SPEC: every term's slot
  uint64_t gid = 0, seed = 0;
  V3 dI = v3(0, 0, 0);  // adjoint: dL/dI of this sample's pixel / spp
  {
    const int64_t P = A.px_begin + si / A.spp;
    const int v = find_view(A.views, A.n_views, P);
    gid = (uint64_t)((P - A.views[v].px_begin) * A.spp + si % A.spp);
    seed = A.views[v].seed;
    if (SPEC) seed ^= 0xA0761D6478BD642Full * (uint64_t)node;  // a stream per tree node
    if (ADJ && valid) {
      dI = load3(J.dfilm + 3 * P) * (1.0f / A.spp);
      if (A.tcam) dI = mul(dI, load3(A.tcam + 3 * (int64_t)si));  // the camera ray's medium segment
      if (SPEC) dI = mul(dI, wt);  // a specular level's terms carry the entry's weight
    }
  }
  const float escale = S.emission_scale;
  float g_em = 0.0f;  // adjoint: this thread's direct emission-gradient terms

  Hit h{};
  Bsdf b{};
  V3 wo = v3(0, 0, 0);
  if (surface) {
    const V3 o = v3(ra.x, ra.y, ra.z), d = v3(ra.w, rb.x, rb.y);
    h = make_hit(S, o, d, __int_as_float(hit.x), hit.y, hit.z);
    b = make_bsdf(S, h, hit.y);
    wo = d * -1.0f;
    // Area light emission towards the viewer (DiffuseAreaLightSource::Radiance).
    const int li = S.prim_light[hit.y];
    if (li >= 0 && dot(wo, h.ng) > 0.0f) {
      const V3 le = load3(S.area_lights[li].radiance);
      if (ADJ) g_em += dot(dI, le);
      else if (SPEC) atomic_add_rgb(contrib, tslot, mul(le * escale, wt));
      else store_rgb(contrib, slot0, le * escale);
    }
  }
  const V3 shading_n = b.n;
  const V3 n_view = dot(wo, b.n) >= 0.0f ? b.n : b.n * -1.0f;

  // Light samples (DirectLightingIntegrator::_SampleLights, :158-262).
  for (int k = 0; k < nl; ++k) {
    bool want = false;
    V3 val = v3(0, 0, 0), dir = v3(0, 0, 0), dkd = v3(0, 0, 0);
    float dem = 0.0f;
    float tmin = 0.0f, tmax = 0.0f;
    if (surface && S.n_area_lights > 0) {
      float uc, u0, u1;
      direct_sample(A, !SPEC && A.ld, seed, gid, false, k, uc, u0, u1);
      // the light by IrradianceLightsSamplingStrategy at this point, with
      // the shading normal turned to the viewer (reflection-only BSDFs,
      // DirectLightingIntegrator.cpp:107-111)
      float lcp, tri_u;
      const int li = choose_light(S, uc, h.p, n_view, lcp, tri_u);
      const AreaLight L = S.area_lights[li];
      // BinarySearchCDF over the light's area CDF (MathRoutines.h:191-218)
      int lo = 0, hi = L.tri_count - 1;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (S.light_cdf[L.tri_begin + mid] <= tri_u) lo = mid + 1; else hi = mid;
      }
      const int lg = S.light_tri[L.tri_begin + lo];
      const int j0 = S.tri_vidx[3 * lg], j1 = S.tri_vidx[3 * lg + 1], j2 = S.tri_vidx[3 * lg + 2];
      const V3 q0 = load3(S.vpos + 3 * j0), q1 = load3(S.vpos + 3 * j1), q2 = load3(S.vpos + 3 * j2);
      const V3 ln = normalized(cross(q1 - q0, q2 - q0));
      // UniformTriangleSampling (SamplingRoutines.h:318-324)
      const float sq = sqrtf(u0), b1 = 1.0f - sq, b2 = u1 * sq;
      const V3 sp = q0 * b1 + q1 * b2 + q2 * (1.0f - b1 - b2);
      const V3 lv = sp - h.p;
      const float dist = len(lv);
      dir = lv * (1.0f / dist);
      const float cosl = fabsf(dot(dir, ln));
      const float light_pdf = cosl > kEps ? dist * dist / (L.area * cosl) : 0.0f;
      if (light_pdf > 0.0f && dot(ln, dir) < 0.0f) {
        const V3 f = bsdf_eval(b, wo, dir);
        if (!black(f)) {
          const float bpdf = bsdf_pdf(b, wo, dir);
          const float w = power_heuristic(nl, light_pdf * lcp, nl, bpdf) * fabsf(dot(dir, shading_n)) /
                          (light_pdf * lcp);
          tmin = next_min_t(S, h, dir);
          tmax = dist - 1e-4f;  // to avoid hitting the light itself (:237)
          const V3 le = mul(load3(L.radiance), medium_tr(S.medium, h.p, dir, tmin, tmax));
          val = mul(f, le) * (escale * w / nl);
          if (ADJ) {
            dkd = mul(dI, mul(bsdf_eval_dkd(b, wo, dir), le)) * (escale * w / nl);
            dem = dot(dI, mul(f, le)) * (w / nl);
          }
          want = tmax > tmin;
        }
      }
    }
    const int q = queue_append(want, scount);
    if (want) {
      store_ray(srays, q, h.p, dir, tmin, tmax);
      if (ADJ) {
        starget[q] = h.g;
        store_rgb(J.s_dkd, q, dkd);
        J.s_dem[q] = dem;
      } else {
        starget[q] = (int)(SPEC ? tslot : slot0 + 1 + k);
        store_rgb(srgb, q, SPEC ? mul(val, wt) : val);
      }
    }
  }
  // Point lights (delta lights, :91-107).
  for (int k = 0; k < S.n_point_lights; ++k) {
    bool want = false;
    V3 val = v3(0, 0, 0), dir = v3(0, 0, 0), dkd = v3(0, 0, 0);
    float tmin = 0.0f, tmax = 0.0f;
    if (surface) {
      const PointLightDev P = S.point_lights[k];
      const V3 lv = load3(P.position) - h.p;
      const float dist = len(lv), inv = 1.0f / dist;
      dir = lv * inv;
      const V3 f = bsdf_eval(b, dir, wo);
      if (!black(f)) {
        tmin = next_min_t(S, h, dir);
        tmax = dist;
        const V3 li = mul(load3(P.intensity), medium_tr(S.medium, h.p, dir, tmin, tmax));
        val = mul(f, li) * (inv * inv * fabsf(dot(dir, shading_n)));
        if (ADJ) dkd = mul(dI, mul(bsdf_eval_dkd(b, dir, wo), li)) * (inv * inv * fabsf(dot(dir, shading_n)));
        want = tmax > tmin;
      }
    }
    const int q = queue_append(want, scount);
    if (want) {
      store_ray(srays, q, h.p, dir, tmin, tmax);
      if (ADJ) {
        starget[q] = h.g;
        store_rgb(J.s_dkd, q, dkd);
        J.s_dem[q] = 0.0f;
      } else {
        starget[q] = (int)(SPEC ? tslot : slot0 + 1 + nl + k);
        store_rgb(srgb, q, SPEC ? mul(val, wt) : val);
      }
    }
  }
  // BSDF samples (DirectLightingIntegrator::_SampleBSDF, :264-366).
  for (int k = 0; k < nl; ++k) {
    bool want = false;
    V3 val = v3(0, 0, 0), dir = v3(0, 0, 0), dkd = v3(0, 0, 0);
    float pdf = 0.0f, tmin = 0.0f;
    if (surface && S.n_area_lights > 0) {
      float uc, u0, u1;
      direct_sample(A, !SPEC && A.ld, seed, gid, true, k, uc, u0, u1);
      const V3 f = bsdf_sample(b, wo, uc, u0, u1, dir, pdf);
      if (pdf > 0.0f && !black(f)) {
        val = f * (fabsf(dot(dir, shading_n)) / (pdf * nl));
        if (ADJ) {
          dkd = mul(dI, bsdf_eval_dkd(b, wo, dir)) * (fabsf(dot(dir, shading_n)) / (pdf * nl));
          val = mul(dI, val);
        }
        tmin = next_min_t(S, h, dir);
        want = true;
      }
    }
    const int q = queue_append(want, bcount);
    if (want) {
      store_ray(brays, q, h.p, dir, tmin, __int_as_float(0x7f800000));
      btarget[q] = ADJ ? h.g : (int)(SPEC ? tslot : slot0 + 1 + nl + S.n_point_lights + k);
      if (ADJ) store_rgb(J.b_dkd, q, dkd);
      if (SPEC) val = mul(val, wt);
      if (bnrm) store_rgb(bnrm, q, n_view);
      brgb[4 * q] = val.x;
      brgb[4 * q + 1] = val.y;
      brgb[4 * q + 2] = val.z;
      brgb[4 * q + 3] = pdf;
    }
  }
  if (ADJ) add_emission_grad(J.g_emission, g_em);
  // Specular children (reflection, then transmission) while the depth allows.
  if (KIDS) {
    const bool deeper = surface && bsdf_nspec(b) > 0 && Q.depth <= S.max_spec_depth;
    for (int c = 0; c < 2; ++c) {
      V3 dir = v3(0, 0, 0), val = v3(0, 0, 0);
      const bool want = deeper && (c == 0 ? specular_reflect(b, wo, dir, val) : specular_transmit(b, wo, dir, val));
      const int q = queue_append(want, Q.out_count);
      if (want) {
        store_ray(Q.out_rays, q, h.p, dir, next_min_t(S, h, dir), __int_as_float(0x7f800000));
        store_rgb(Q.out_w, q, mul(wt, val));
        Q.out_sample[q] = si;
        Q.out_node[q] = (int)(2u * node + (unsigned)c);
      }
    }
  }
  }  // entries
}

// accumulate: add into the target (the targets of a specular level repeat)
// instead of storing.
__global__ void k_resolve_shadow(const uint8_t *__restrict__ occ, const int *__restrict__ starget,
                                 const float *__restrict__ srgb, const int *__restrict__ scount,
                                 float *__restrict__ contrib, bool accumulate) {
  const int n = *scount;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (occ[i]) continue;
    const int64_t t = starget[i];
    if (accumulate) {
      atomic_add_rgb(contrib, t, v3(srgb[3 * i], srgb[3 * i + 1], srgb[3 * i + 2]));
      continue;
    }
    contrib[3 * t] = srgb[3 * i];
    contrib[3 * t + 1] = srgb[3 * i + 1];
    contrib[3 * t + 2] = srgb[3 * i + 2];
  }
}

// A BSDF ray that hits the front of an area light adds its MIS-weighted
// emission (:300-318); the light density is DiffuseAreaLightSource::
// LightingPDF (:104-116).
__device__ __forceinline__ void resolve_bsdf_entry(const SceneDev &S, int n_light_samples, int i,
                                                   const float4 *__restrict__ brays, const int4 *__restrict__ bhits,
                                                   const int *__restrict__ btarget, const float *__restrict__ brgb,
                                                   const float *__restrict__ bnrm, float *__restrict__ contrib,
                                                   bool accumulate) {
  const int4 hit = bhits[i];
  if (hit.y < 0) return;
  const int li = S.prim_light[hit.y];
  if (li < 0) return;
  const float4 ra = brays[2 * i], rb = brays[2 * i + 1];
  const V3 d = v3(ra.w, rb.x, rb.y);
  const int g = S.prim_tri_offset[hit.y] + hit.z;
  const int j0 = S.tri_vidx[3 * g], j1 = S.tri_vidx[3 * g + 1], j2 = S.tri_vidx[3 * g + 2];
  const V3 q0 = load3(S.vpos + 3 * j0), q1 = load3(S.vpos + 3 * j1), q2 = load3(S.vpos + 3 * j2);
  const V3 ln = normalized(cross(q1 - q0, q2 - q0));
  if (!(dot(d * -1.0f, ln) > 0.0f)) return;  // back side emits nothing
  const AreaLight L = S.area_lights[li];
  const float dist = __int_as_float(hit.x) - rb.z;  // ray max_t - min_t
  const float cosl = fabsf(dot(d, ln));
  const float light_pdf = cosl > kEps ? dist * dist / (L.area * cosl) : 0.0f;
  const float lcp = light_choice_pdf(S, li, v3(ra.x, ra.y, ra.z), load3(bnrm + 3 * (int64_t)i));
  const float bpdf = brgb[4 * i + 3];
  const float w = power_heuristic(n_light_samples, bpdf, n_light_samples, light_pdf * lcp);
  const int64_t t = btarget[i];
  const float sw = S.emission_scale * w;
  const V3 tr = medium_tr(S.medium, v3(ra.x, ra.y, ra.z), d, rb.z, __int_as_float(hit.x));
  if (accumulate) {
    atomic_add_rgb(contrib, t,
                   v3(brgb[4 * i] * L.radiance[0] * tr.x * sw, brgb[4 * i + 1] * L.radiance[1] * tr.y * sw,
                      brgb[4 * i + 2] * L.radiance[2] * tr.z * sw));
    return;
  }
  contrib[3 * t] = brgb[4 * i] * L.radiance[0] * tr.x * sw;
  contrib[3 * t + 1] = brgb[4 * i + 1] * L.radiance[1] * tr.y * sw;
  contrib[3 * t + 2] = brgb[4 * i + 2] * L.radiance[2] * tr.z * sw;
}

__global__ void k_resolve_bsdf(SceneDev S, int n_light_samples, const float4 *__restrict__ brays,
                               const int4 *__restrict__ bhits, const int *__restrict__ btarget,
                               const float *__restrict__ brgb, const int *__restrict__ bcount,
                               const float *__restrict__ bnrm, float *__restrict__ contrib, bool accumulate) {
  const int n = *bcount;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    resolve_bsdf_entry(S, n_light_samples, i, brays, bhits, btarget, brgb, bnrm, contrib, accumulate);
}

// Adjoint of k_resolve_shadow: an unoccluded shadow ray adds its derivative
// terms to its triangle's albedo gradient and to the emission gradient.
__global__ void k_resolve_shadow_adj(const uint8_t *__restrict__ occ, const int *__restrict__ stri,
                                     const int *__restrict__ scount, AdjointArgs J) {
  const int n = *scount;
  for (int i0 = blockIdx.x * blockDim.x; i0 < n; i0 += gridDim.x * blockDim.x) {  // block-uniform trip count
    const int i = i0 + threadIdx.x;
    float dem = 0.0f;
    if (i < n && !occ[i]) {
      const int64_t g = stri[i];
      const float *d = J.s_dkd + 3 * (int64_t)i;
      if (d[0] != 0.0f) atomicAdd(J.g_albedo + 3 * g, d[0]);
      if (d[1] != 0.0f) atomicAdd(J.g_albedo + 3 * g + 1, d[1]);
      if (d[2] != 0.0f) atomicAdd(J.g_albedo + 3 * g + 2, d[2]);
      dem = J.s_dem[i];
    }
    add_emission_grad(J.g_emission, dem);
  }
}

// Adjoint of k_resolve_bsdf (same light density and MIS weight).
__global__ void k_resolve_bsdf_adj(SceneDev S, int n_light_samples, const float4 *__restrict__ brays,
                                   const int4 *__restrict__ bhits, const int *__restrict__ btri,
                                   const float *__restrict__ brgb, const int *__restrict__ bcount,
                                   const float *__restrict__ bnrm, AdjointArgs J) {
  const int n = *bcount;
  for (int i0 = blockIdx.x * blockDim.x; i0 < n; i0 += gridDim.x * blockDim.x) {  // block-uniform trip count
  const int i = i0 + threadIdx.x;
  float dem = 0.0f;
  if (i < n) {
    const int4 hit = bhits[i];
    const int li = hit.y >= 0 ? S.prim_light[hit.y] : -1;
    if (li >= 0) {
      const float4 ra = brays[2 * i], rb = brays[2 * i + 1];
      const V3 d = v3(ra.w, rb.x, rb.y);
      const int g = S.prim_tri_offset[hit.y] + hit.z;
      const int j0 = S.tri_vidx[3 * g], j1 = S.tri_vidx[3 * g + 1], j2 = S.tri_vidx[3 * g + 2];
      const V3 q0 = load3(S.vpos + 3 * j0), q1 = load3(S.vpos + 3 * j1), q2 = load3(S.vpos + 3 * j2);
      const V3 ln = normalized(cross(q1 - q0, q2 - q0));
      if (dot(d * -1.0f, ln) > 0.0f) {
        const AreaLight L = S.area_lights[li];
        const float dist = __int_as_float(hit.x) - rb.z;
        const float cosl = fabsf(dot(d, ln));
        const float light_pdf = cosl > kEps ? dist * dist / (L.area * cosl) : 0.0f;
        const float lcp = light_choice_pdf(S, li, v3(ra.x, ra.y, ra.z), load3(bnrm + 3 * (int64_t)i));
        const float w = power_heuristic(n_light_samples, brgb[4 * i + 3], n_light_samples, light_pdf * lcp);
        const V3 le = mul(load3(L.radiance), medium_tr(S.medium, v3(ra.x, ra.y, ra.z), d, rb.z, __int_as_float(hit.x)));
        const V3 dk = mul(load3(J.b_dkd + 3 * (int64_t)i), le) * (S.emission_scale * w);
        const int64_t t = btri[i];
        if (dk.x != 0.0f) atomicAdd(J.g_albedo + 3 * t, dk.x);
        if (dk.y != 0.0f) atomicAdd(J.g_albedo + 3 * t + 1, dk.y);
        if (dk.z != 0.0f) atomicAdd(J.g_albedo + 3 * t + 2, dk.z);
        dem = dot(v3(brgb[4 * i], brgb[4 * i + 1], brgb[4 * i + 2]), le) * w;
      }
    }
  }
  add_emission_grad(J.g_emission, dem);
  }
}

// Double-precision vectors with every product and sum rounded separately
// (no contraction), as the reference's x86-64 build computes them.
struct D3 {
  double x, y, z;
};
__device__ __forceinline__ D3 d3sub(D3 a, D3 b) { return D3{__dsub_rn(a.x, b.x), __dsub_rn(a.y, b.y), __dsub_rn(a.z, b.z)}; }
__device__ __forceinline__ D3 d3cross(D3 a, D3 b) {
  return D3{__dsub_rn(__dmul_rn(a.y, b.z), __dmul_rn(a.z, b.y)), __dsub_rn(__dmul_rn(a.z, b.x), __dmul_rn(a.x, b.z)),
            __dsub_rn(__dmul_rn(a.x, b.y), __dmul_rn(a.y, b.x))};
}
__device__ __forceinline__ double d3dot(D3 a, D3 b) {
  return __dadd_rn(__dadd_rn(__dmul_rn(a.x, b.x), __dmul_rn(a.y, b.y)), __dmul_rn(a.z, b.z));
}
__device__ __forceinline__ D3 d3scale(D3 a, double s) { return D3{__dmul_rn(a.x, s), __dmul_rn(a.y, s), __dmul_rn(a.z, s)}; }
__device__ __forceinline__ D3 d3normalized(D3 a) {
  const double l2 = d3dot(a, a);
  return l2 > 0.0 ? d3scale(a, __ddiv_rn(1.0, __dsqrt_rn(l2))) : a;
}
__device__ __forceinline__ D3 d3load(const float *p) { return D3{(double)p[0], (double)p[1], (double)p[2]}; }

// The reference's medium march samples an area light with the lighting ray
// of DiffuseAreaLightSource::SampleLighting (DiffuseAreaLightSource.cpp:
// 77-98, _SampleArea :149-175): the sampled point p = b1 v0 + b2 v1 +
// (1 - b1 - b2) v2 with b1 = 1 - sqrt(u0), b2 = u1 sqrt(u0)
// (SamplingRoutines::UniformTriangleSampling), the ray (x, (p - x) / |p - x|,
// 0, |p - x|), and tests it as is (DirectLightingLTEIntegrator.cpp:149-156,
// without the surface path's 1e-4 pull-back).  The ray ends exactly on the
// light, so whether the light's own triangle occludes it is decided by the
// double rounding of the ray, of the slab test and of the Moller-Trumbore t
// (TriangleAccelerator.cpp:354-462).  This restates that decision on the
// same double arithmetic: the reference reaches the leaf holding the light
// triangle exactly when the leaf's own slab test passes (every ancestor's
// box contains the leaf's, and (b - o) * (1/d) is monotone in b, so an
// ancestor's slab interval contains the leaf's), and then tests the leaf's
// triangles.  Only triangles whose box contains p are tested here: the ray
// reaches any other triangle of the leaf before p, and the float shadow ray
// (whose tmax stops short of the light) decides those.  Returns true when
// the light's leaf occludes the ray; p_out, len_out give the sampled point
// and the ray length.
__device__ bool own_light_leaf_occludes(const SceneDev &S, int j, D3 x, double u0, double u1, D3 &p_out,
                                        double &len_out) {
  const int g = S.light_tri[j];
  const int j0 = S.tri_vidx[3 * g], j1 = S.tri_vidx[3 * g + 1], j2 = S.tri_vidx[3 * g + 2];
  const D3 v0 = d3load(S.vpos + 3 * j0), v1 = d3load(S.vpos + 3 * j1), v2 = d3load(S.vpos + 3 * j2);
  const double sq = __dsqrt_rn(u0);
  const double b1 = __dsub_rn(1.0, sq), b2 = __dmul_rn(u1, sq);
  const double b0 = __dsub_rn(__dsub_rn(1.0, b1), b2);
  const D3 a = d3scale(v0, b1), b = d3scale(v1, b2), c = d3scale(v2, b0);
  const D3 p{__dadd_rn(__dadd_rn(a.x, b.x), c.x), __dadd_rn(__dadd_rn(a.y, b.y), c.y),
             __dadd_rn(__dadd_rn(a.z, b.z), c.z)};
  const D3 lv = d3sub(p, x);
  const double len = __dsqrt_rn(d3dot(lv, lv));
  const D3 dir = d3scale(lv, __ddiv_rn(1.0, len));
  p_out = p;
  len_out = len;
  const float *lb = S.light_leaf + 8 * (int64_t)j;
  // the leaf's slab test (TriangleAccelerator.cpp:373-390)
  const double inv[3] = {__ddiv_rn(1.0, dir.x), __ddiv_rn(1.0, dir.y), __ddiv_rn(1.0, dir.z)};
  const double org[3] = {x.x, x.y, x.z};
  double tn[3], tf[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    tn[k] = __dmul_rn(__dsub_rn((double)lb[k], org[k]), inv[k]);
    tf[k] = __dmul_rn(__dsub_rn((double)lb[3 + k], org[k]), inv[k]);
    if (tn[k] > tf[k]) {
      const double tmp = tn[k];
      tn[k] = tf[k];
      tf[k] = tmp;
    }
  }
  const double tmin = 0.0, tmax = len;
  if (tmin > tf[0] || tn[0] > tf[1] || tn[1] > tf[0] || tn[2] > tf[0] || tmin > tf[1] || tn[0] > tf[2] ||
      tn[1] > tf[2] || tn[2] > tf[1] || tmin > tf[2] || tn[0] > tmax || tn[1] > tmax || tn[2] > tmax)
    return false;
  const int first = __float_as_int(lb[6]), count = __float_as_int(lb[7]);
  const float pf[3] = {(float)p.x, (float)p.y, (float)p.z};
  for (int k = 0; k < count; ++k) {
    const float4 ta = S.accel_tris[3 * (first + k)], tb = S.accel_tris[3 * (first + k) + 1],
                 tc = S.accel_tris[3 * (first + k) + 2];
    // the triangle's box, widened by a few float ulps of the point, must hold p
    bool near = true;
    const float va[3] = {ta.x, ta.y, ta.z}, vb[3] = {tb.x, tb.y, tb.z}, vc[3] = {tc.x, tc.y, tc.z};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
      const float w = 4.0f * 1.1920929e-7f * (fabsf(pf[q]) + 1e-30f);
      near = near && pf[q] >= fminf(fminf(va[q], vb[q]), vc[q]) - w && pf[q] <= fmaxf(fmaxf(va[q], vb[q]), vc[q]) + w;
    }
    if (!near) continue;
    // Moller-Trumbore in double (TriangleAccelerator.cpp:419-452)
    const D3 w0{(double)ta.x, (double)ta.y, (double)ta.z};
    const D3 e1 = d3sub(D3{(double)tb.x, (double)tb.y, (double)tb.z}, w0);
    const D3 e2 = d3sub(D3{(double)tc.x, (double)tc.y, (double)tc.z}, w0);
    const D3 s1 = d3cross(dir, e2);
    const double idv = __ddiv_rn(1.0, d3dot(s1, e1));
    const D3 dd = d3sub(x, w0);
    const double c1 = __dmul_rn(d3dot(dd, s1), idv);
    if (!(c1 > -2.220446049250313e-16 && c1 < 1.0 + 2.220446049250313e-16)) continue;
    const D3 s2 = d3cross(dd, e1);
    const double c2 = __dmul_rn(d3dot(dir, s2), idv);
    if (!(c2 > -2.220446049250313e-16 && __dadd_rn(c1, c2) < 1.0 + 2.220446049250313e-16)) continue;
    const double t = __dmul_rn(d3dot(e2, s2), idv);
    if (t >= tmin && t <= tmax) return true;
  }
  return false;
}

// Single scattering along the camera ray's segment in the medium
// (DirectLightingLTEIntegrator::_MediaRadianceAndTranmsittance,
// LTEIntegrators/DirectLightingLTEIntegrator.cpp:62-175): march with step
// base / luminance(transmittance) from a random offset, add the medium's
// emission, and at every step one light sample (light chosen uniformly with
// the radical inverse of the step in base 2, area-light position from bases
// 3 and 5) whose shadow ray goes to the media queue.  Writes the segment's
// transmittance (it multiplies the surface radiance, LTEIntegrator.cpp:28-55)
// and the emission term (the sample's medium slot).
struct MediaArgs {
  int n;
  int64_t px_begin;
  int spp;
  int slots;
  int media_slot;
  const ViewDev *views;
  int n_views;
  // A specular level's entries instead of camera rays (in_sample non-null):
  // entry i's sample, weight (multiplied by the segment's transmittance in
  // place) and tree node; its emission and in-scattering go, weighted, into
  // its sample's slot spec_slot (adjoint: only the weight and the
  // in-scattering's emission-scale derivative).
  const int *in_sample;
  float *in_w;
  const int *in_node;
  int spec_slot;
  // Device-counted chunk of a level (off_dev non-null): entries
  // [*off_dev, *off_dev + n) of the level, clipped to min(*count_dev,
  // capacity); the arrays are the level's own, indexed by entry.
  const int *off_dev;
  const int *count_dev;
  int64_t capacity;
  // Adjoint of a specular level: the samples' camera-segment transmittance
  // (it scales the whole specular slot in the film, so dL/dI too).
  const float *tcam_in;
};

__device__ __forceinline__ double radical_inverse_r(unsigned n, unsigned base) {
  double ret = 0.0;
  const double inv_base = 1.0 / base;
  double inv = inv_base;
  while (n > 0) {
    ret += (double)(n % base) * inv;
    n /= base;
    inv *= inv_base;
  }
  return ret;
}

template <bool ADJ>
__global__ void __launch_bounds__(128) k_media(SceneDev S, MediaArgs A, AdjointArgs J, const float4 *__restrict__ rays,
                                               const int4 *__restrict__ hits, float *__restrict__ contrib,
                                               float *__restrict__ tcam, float4 *__restrict__ mrays,
                                               int *__restrict__ mtarget, float *__restrict__ mval,
                                               float *__restrict__ mdem, int *__restrict__ mcount,
                                               unsigned *__restrict__ status) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= A.n) return;
  if (A.off_dev) {  // a device-counted chunk of a specular level
    const int64_t e = (int64_t)*A.off_dev + i;
    if (e >= min((int64_t)*A.count_dev, A.capacity)) return;
    i = (int)e;
  }
  const bool spec = A.in_sample != nullptr;  // a specular level's entry
  const int si = spec ? A.in_sample[i] : i;
  const V3 wt = spec ? load3(A.in_w + 3 * (int64_t)i) : v3(1.0f, 1.0f, 1.0f);
  const MediumDev &M = S.medium;
  const float4 ra = rays[2 * i], rb = rays[2 * i + 1];
  const V3 o = v3(ra.x, ra.y, ra.z), d = v3(ra.w, rb.x, rb.y);
  const int4 hit = hits[i];
  float t0 = 0.0f, t1 = hit.y >= 0 ? __int_as_float(hit.x) : __int_as_float(0x7f800000);
  V3 T = v3(1.0f, 1.0f, 1.0f);
  if (!medium_segment(M, o, d, t0, t1) || fabsf(t0 - t1) < kEps) {
    if (!spec) store_rgb(tcam, i, T);
    return;
  }
  const int64_t P = A.px_begin + si / A.spp;
  int lo = 0, hi = A.n_views - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (A.views[mid].px_begin <= P) lo = mid; else hi = mid - 1;
  }
  const uint64_t gid = (uint64_t)((P - A.views[lo].px_begin) * A.spp + si % A.spp);
  uint64_t seed = A.views[lo].seed;
  if (spec) seed ^= 0xA0761D6478BD642Full * (uint64_t)A.in_node[i];  // the entry's stream, as in k_shade
  V3 dI = v3(0, 0, 0);
  if (ADJ) {
    dI = load3(J.dfilm + 3 * P) * (1.0f / A.spp);
    if (spec && A.tcam_in) dI = mul(dI, load3(A.tcam_in + 3 * (int64_t)si));
  }
  const double offset1 = rnd(seed, gid, 62);
  const V3 ss = load3(M.sigma_s), st = load3(M.sigma_t), em = load3(M.emission);
  const bool scatters = !black(ss);
  const int nlights = S.n_point_lights + S.n_area_lights;
  const V3 dirv = d * -1.0f;
  double tb = t0;
  const double te = t1;
  V3 point = o + d * t0, rad = v3(0, 0, 0);
  double step = M.step;
  int steps = 0;
  for (unsigned k = 0; tb < te - 2.220446049250313e-16; ++k) {
    if (steps == M.max_steps) {  // the media queue is sized for max_steps per ray
      atomicOr(status, 4u);
      break;
    }
    ++steps;
    step = fmin(step, te - tb);
    const double s1 = radical_inverse_r(k + 1, 2);
    const double s2ad = radical_inverse_r(k + 1, 3), s2bd = radical_inverse_r(k + 1, 5);
    const V3 prev = point;
    const double tp = tb + offset1 * step;
    point = o + d * (float)tp;
    tb += step;
    const float seg = len(point - prev);
    T = v3(T.x * expf(-st.x * seg), T.y * expf(-st.y * seg), T.z * expf(-st.z * seg));
    rad = rad + mul(T, em) * (float)step;
    if (scatters && nlights > 0) {
      const int li = min((int)(s1 * nlights), nlights - 1);
      V3 lv = v3(0, 0, 0), ldir = v3(0, 0, 0);
      float dist = 0.0f, pdf = 1.0f;
      bool area = false, self_occ = false;
      if (li < S.n_point_lights) {
        const PointLightDev PL = S.point_lights[li];
        const V3 to = load3(PL.position) - point;
        dist = len(to);
        ldir = to * (1.0f / dist);
        lv = load3(PL.intensity) * (1.0f / (dist * dist));
      } else {
        const AreaLight L = S.area_lights[li - S.n_point_lights];
        // the reference draws the triangle choice from the thread's generator
        const float tri_u = rnd(seed ^ 0xD1B54A32D192ED03ull, gid * 4096ull + (k >> 6), k & 63u);
        int a = 0, b = L.tri_count - 1;
        while (a < b) {
          const int mid = (a + b) >> 1;
          if (S.light_cdf[L.tri_begin + mid] <= tri_u) a = mid + 1; else b = mid;
        }
        const int g = S.light_tri[L.tri_begin + a];
        const int j0 = S.tri_vidx[3 * g], j1 = S.tri_vidx[3 * g + 1], j2 = S.tri_vidx[3 * g + 2];
        const V3 q0 = load3(S.vpos + 3 * j0), q1 = load3(S.vpos + 3 * j1), q2 = load3(S.vpos + 3 * j2);
        const V3 ln = normalized(cross(q1 - q0, q2 - q0));
        D3 spd;
        double lend;
        // the march point in double, o + d t as the reference's Ray::operator()
        // computes it from its double ray (a float point would round the
        // light ray differently from the reference's double one)
        const D3 xd{__dadd_rn((double)o.x, __dmul_rn((double)d.x, tp)), __dadd_rn((double)o.y, __dmul_rn((double)d.y, tp)),
                    __dadd_rn((double)o.z, __dmul_rn((double)d.z, tp))};
        self_occ = own_light_leaf_occludes(S, L.tri_begin + a, xd, s2ad, s2bd, spd, lend);
        const V3 sp = v3((float)spd.x, (float)spd.y, (float)spd.z);
        const V3 to = sp - point;
        dist = len(to);
        ldir = to * (1.0f / dist);
        const float cosl = fabsf(dot(ldir, ln));
        pdf = cosl > kEps ? dist * dist / (L.area * cosl) : 0.0f;
        if (dot(ln, ldir) < 0.0f) lv = load3(L.radiance) * S.emission_scale;
        area = true;
      }
      const bool want = !black(lv) && pdf > 0.0f && !self_occ;
      V3 val = v3(0, 0, 0);
      if (want) {
        // HGPhaseFunction::ScatteringPDF(incoming = -light direction, outgoing = -ray direction)
        const float g = M.g, c = dot(ldir, d);
        const float ph = (float)(1.0 / (4.0 * 3.14159265358979323846)) * (1.0f - g * g) *
                         powf(1.0f + g * g - 2.0f * g * c, -1.5f);
        const V3 tr = medium_tr(M, point, ldir, 0.0f, dist);
        val = mul(mul(mul(T, ss), lv), tr) * (ph * (float)step * nlights / pdf);
      }
      const int q = queue_append(want, mcount);
      if (want) {
        // An area light's own leaf was decided above; the float ray stops
        // short of the light so that it tests everything in front of it.
        store_ray(mrays, q, point, ldir, 0.0f, area ? dist * (1.0f - 1e-4f) : dist);
        mtarget[q] = spec ? (int)((int64_t)si * A.slots + A.spec_slot) : i;
        if (spec) val = mul(val, wt);
        if (ADJ) {
          mdem[q] = area && S.emission_scale > 0.0f ? dot(dI, val) / S.emission_scale : 0.0f;
        } else {
          store_rgb(mval, q, val);
        }
      }
    }
    const float lum = 0.05316285f * T.x + 0.58515348f * T.y + 0.36168367f * T.z;
    if (lum < kEps) break;
    step = M.step / lum;
  }
  if (spec) {
    // LTEIntegrator::Radiance of the specular ray: its surface radiance
    // (shaded next, with the weight) times T, plus the medium's radiance
    // (the medium's own emission is no parameter of the adjoint)
    if (!ADJ) atomic_add_rgb(contrib, (int64_t)si * A.slots + A.spec_slot, mul(rad, wt));
    store_rgb(A.in_w, i, mul(wt, T));
    return;
  }
  store_rgb(tcam, i, T);
  if (!ADJ) store_rgb(contrib, (int64_t)i * A.slots + A.media_slot, rad);
}

// An unoccluded media shadow ray adds its in-scattered radiance to its
// sample's medium slot (adjoint: its emission-scale derivative).
template <bool ADJ>
__global__ void k_resolve_media(const uint8_t *__restrict__ occ, const int *__restrict__ mtarget,
                                const float *__restrict__ mval, const float *__restrict__ mdem,
                                const int *__restrict__ mcount, int slots, int media_slot, float *__restrict__ contrib,
                                double *__restrict__ g_emission) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float dem = 0.0f;
  if (i < *mcount && !occ[i]) {
    if (ADJ) {
      dem = mdem[i];
    } else {
      const int64_t t = (int64_t)mtarget[i] * slots + media_slot;
      atomicAdd(contrib + 3 * t, mval[3 * i]);
      atomicAdd(contrib + 3 * t + 1, mval[3 * i + 1]);
      atomicAdd(contrib + 3 * t + 2, mval[3 * i + 2]);
    }
  }
  if (ADJ) {
    for (int o = 16; o > 0; o >>= 1) dem += __shfl_xor_sync(0xffffffffu, dem, o);
    if ((threadIdx.x & 31) == 0 && dem != 0.0f) atomicAdd(g_emission, (double)dem);
  }
}

// Luminance weights of the reference's RGB spectrum (row Y of its
// Spectrum-to-XYZ matrix, Core/SpectrumRoutines.cpp:20-64), used by the
// renderer's negative-sample check.
__constant__ float kLumW[3] = {0.05316285f, 0.58515348f, 0.36168367f};

__global__ void k_film(const float *__restrict__ contrib, int64_t px_begin, int n_px, int spp, int slots,
                       const float *__restrict__ tcam, int media_slot, float *__restrict__ film) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_px) return;
  float r = 0.0f, g = 0.0f, bb = 0.0f;
  for (int j = 0; j < spp; ++j) {
    const int64_t base = ((int64_t)p * spp + j) * slots;
    float sr = 0.0f, sg = 0.0f, sb = 0.0f;
    const int surface_slots = tcam ? media_slot : slots;
    for (int k = 0; k < surface_slots; ++k) {
      sr += contrib[3 * (base + k)];
      sg += contrib[3 * (base + k) + 1];
      sb += contrib[3 * (base + k) + 2];
    }
    if (tcam) {
      // LTEIntegrator::Radiance: surface * transmittance + medium radiance
      const int64_t si = (int64_t)p * spp + j;
      sr = sr * tcam[3 * si] + contrib[3 * (base + media_slot)];
      sg = sg * tcam[3 * si + 1] + contrib[3 * (base + media_slot) + 1];
      sb = sb * tcam[3 * si + 2] + contrib[3 * (base + media_slot) + 2];
    }
    const bool bad = !(sr == sr && sg == sg && sb == sb) ||
                     (kLumW[0] * sr + kLumW[1] * sg + kLumW[2] * sb) < -1e-16f || isinf(sr) || isinf(sg) ||
                     isinf(sb);
    if (!bad) {
      r += sr;
      g += sg;
      bb += sb;
    }
  }
  const float inv = 1.0f / spp;
  const int64_t o = 3 * (int64_t)(px_begin + p);
  film[o] = r * inv;
  film[o + 1] = g * inv;
  film[o + 2] = bb * inv;
}

// TriangleMesh::ComputeDifferentialGeometry's point, barycentrics and
// normals (Core/TriangleMesh.cpp:414-484) for closest hits of a render
// scene, in double with the reference's operation order (no contraction):
// Moller-Trumbore against the world triangle (_ComputeIntersectionPoint),
// the point o + d t, the geometric normal (v1 - v0) x (v2 - v0) normalised
// as Vector3D::Normalize does (times 1 / sqrt of the squared length), and the
// shading normal b0 n0 + b1 n1 + b2 n2 normalised (the geometric normal
// without vertex normals).  Out per hit: point, geometric normal, shading
// normal, b1, b2, t (12 doubles); NaN for a miss.
__global__ void k_hit_geometry(SceneDev S, const float4 *__restrict__ rays, const int4 *__restrict__ hits, int n,
                               double *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double *o = out + 12 * (int64_t)i;
  const int4 hit = hits[i];
  if (hit.y < 0) {
    for (int k = 0; k < 12; ++k) o[k] = __longlong_as_double(0x7ff8000000000000ll);
    return;
  }
  const int g = S.prim_tri_offset[hit.y] + hit.z;
  const int j0 = S.tri_vidx[3 * g], j1 = S.tri_vidx[3 * g + 1], j2 = S.tri_vidx[3 * g + 2];
  const D3 v0 = d3load(S.vpos + 3 * j0), v1 = d3load(S.vpos + 3 * j1), v2 = d3load(S.vpos + 3 * j2);
  const float4 ra = rays[2 * i], rb = rays[2 * i + 1];
  const D3 org{(double)ra.x, (double)ra.y, (double)ra.z}, dir{(double)ra.w, (double)rb.x, (double)rb.y};
  const D3 e1 = d3sub(v1, v0), e2 = d3sub(v2, v0);
  const D3 s1 = d3cross(dir, e2);
  const double inv = __ddiv_rn(1.0, d3dot(s1, e1));
  const D3 dd = d3sub(org, v0);
  const double b1 = __dmul_rn(d3dot(dd, s1), inv);
  const D3 s2 = d3cross(dd, e1);
  const double b2 = __dmul_rn(d3dot(dir, s2), inv);
  const double t = __dmul_rn(d3dot(e2, s2), inv);
  const D3 p{__dadd_rn(org.x, __dmul_rn(dir.x, t)), __dadd_rn(org.y, __dmul_rn(dir.y, t)),
             __dadd_rn(org.z, __dmul_rn(dir.z, t))};
  const D3 ng = d3normalized(d3cross(e1, e2));
  D3 ns = ng;
  if (S.prim_has_normals[hit.y]) {
    const double b0 = __dsub_rn(__dsub_rn(1.0, b1), b2);
    const D3 n0 = d3load(S.vnrm + 3 * j0), n1 = d3load(S.vnrm + 3 * j1), n2 = d3load(S.vnrm + 3 * j2);
    const D3 a = d3scale(n0, b0), b = d3scale(n1, b1), c = d3scale(n2, b2);
    ns = d3normalized(D3{__dadd_rn(__dadd_rn(a.x, b.x), c.x), __dadd_rn(__dadd_rn(a.y, b.y), c.y),
                         __dadd_rn(__dadd_rn(a.z, b.z), c.z)});
  }
  const double v[12] = {p.x, p.y, p.z, ng.x, ng.y, ng.z, ns.x, ns.y, ns.z, b1, b2, t};
  for (int k = 0; k < 12; ++k) o[k] = v[k];
}

// ---------------------------------------------- the whole Intersection --
// TriangleAccelerator::Intersect's Intersection for ray differentials
// (TriangleAccelerator.cpp:295-347 with TriangleMesh::
// ComputeDifferentialGeometry, TriangleMesh.cpp:414-561), in double with
// every operation rounded separately as the reference's x86-64 build does.
// Identity-transform primitives reproduce the reference bit for bit,
// including the identity Transform's own arithmetic on the way into and out
// of mesh space (1 x + 0 y + 0 z + 0 turns a -0 into +0; TransformNormal
// normalises again).  A transformed primitive is evaluated on its
// world-space triangle (same formulas, not the reference's rounding).
// The meshes here carry no uv coordinates (the reference's default: all
// zero) and no tangents, so the tangent comes from CoordinateSystem around
// the shading normal, as the reference's zero-determinant branch does.

__device__ __forceinline__ D3 d3add(D3 a, D3 b) { return D3{__dadd_rn(a.x, b.x), __dadd_rn(a.y, b.y), __dadd_rn(a.z, b.z)}; }

// Transform::operator() of the identity matrix on a point / vector and
// TransformNormal (Math/Transform.h:223-292).
__device__ __forceinline__ double id_row(double a, double b, double c, int r) {
  const double m0 = r == 0 ? 1.0 : 0.0, m1 = r == 1 ? 1.0 : 0.0, m2 = r == 2 ? 1.0 : 0.0;
  return __dadd_rn(__dadd_rn(__dmul_rn(m0, a), __dmul_rn(m1, b)), __dmul_rn(m2, c));
}
__device__ __forceinline__ D3 id_point(D3 p) {
  return D3{__dadd_rn(id_row(p.x, p.y, p.z, 0), 0.0), __dadd_rn(id_row(p.x, p.y, p.z, 1), 0.0),
            __dadd_rn(id_row(p.x, p.y, p.z, 2), 0.0)};
}
__device__ __forceinline__ D3 id_vector(D3 v) { return D3{id_row(v.x, v.y, v.z, 0), id_row(v.x, v.y, v.z, 1), id_row(v.x, v.y, v.z, 2)}; }

// TriangleMesh::_ComputeIntersectionPoint (TriangleMesh.cpp:414-437).
__device__ __forceinline__ bool plane_point(D3 v0, D3 v1, D3 v2, D3 o, D3 d, double &b1, double &b2, double &t) {
  const D3 e1 = d3sub(v1, v0), e2 = d3sub(v2, v0);
  const D3 s1 = d3cross(d, e2);
  const double div = d3dot(s1, e1);
  if (div == 0.0) return false;
  const double inv = __ddiv_rn(1.0, div);
  const D3 dd = d3sub(o, v0);
  b1 = __dmul_rn(d3dot(dd, s1), inv);
  const D3 s2 = d3cross(dd, e1);
  b2 = __dmul_rn(d3dot(d, s2), inv);
  t = __dmul_rn(d3dot(e2, s2), inv);
  return true;
}

// MathRoutines::CoordinateSystem (Math/MathRoutines.h:298-313): e2.
__device__ __forceinline__ D3 coordinate_e2(D3 e1) {
  if (fabs(e1.x) > fabs(e1.y)) {
    const double il = __ddiv_rn(1.0, __dsqrt_rn(__dadd_rn(__dmul_rn(e1.x, e1.x), __dmul_rn(e1.z, e1.z))));
    return D3{__dmul_rn(-e1.z, il), 0.0, __dmul_rn(e1.x, il)};
  }
  const double il = __ddiv_rn(1.0, __dsqrt_rn(__dadd_rn(__dmul_rn(e1.y, e1.y), __dmul_rn(e1.z, e1.z))));
  return D3{0.0, __dmul_rn(e1.z, il), __dmul_rn(-e1.y, il)};
}

// b0 a + b1 b + b2 c (uv interpolation with the all-zero uv of the meshes:
// the sign of each zero product is kept, as the reference computes it).
__device__ __forceinline__ double lerp0(double b0, double b1, double b2) {
  return __dadd_rn(__dadd_rn(__dmul_rn(b0, 0.0), __dmul_rn(b1, 0.0)), __dmul_rn(b2, 0.0));
}

__global__ void k_intersection(SceneDev S, const double *__restrict__ rays, const int4 *__restrict__ hits, int n,
                               double *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double *o = out + 36 * (int64_t)i;
  const int4 hit = hits[i];
  const int prim = hit.z, tri = hit.w;
  const double nan = __longlong_as_double(0x7ff8000000000000ll);
  if (prim < 0) {
    for (int k = 0; k < 35; ++k) o[k] = nan;
    ((int *)(o + 35))[0] = -1;
    ((int *)(o + 35))[1] = -1;
    return;
  }
  const double *r = rays + 21 * (int64_t)i;
  const bool ident = S.prim_xform == nullptr || S.prim_xform[prim] == 0;
  const int g = S.prim_tri_offset[prim] + tri;
  const int j0 = S.tri_vidx[3 * g], j1 = S.tri_vidx[3 * g + 1], j2 = S.tri_vidx[3 * g + 2];
  const D3 v0 = d3load(S.vpos + 3 * j0), v1 = d3load(S.vpos + 3 * j1), v2 = d3load(S.vpos + 3 * j2);
  // world_to_mesh of the base ray and of the differentials
  auto pt = [&](D3 p) { return ident ? id_point(p) : p; };
  auto vc = [&](D3 v) { return ident ? id_vector(v) : v; };
  const D3 org = pt(D3{r[0], r[1], r[2]}), dir = vc(D3{r[3], r[4], r[5]});
  const bool has_diff = __double_as_longlong(r[20]) & 1;
  double b1 = nan, b2 = nan, t = nan;
  plane_point(v0, v1, v2, org, dir, b1, b2, t);
  const D3 point = d3add(org, d3scale(dir, t));  // Ray::operator()(t)
  const double b0 = __dsub_rn(__dsub_rn(1.0, b1), b2);
  const double uv[2] = {lerp0(b0, b1, b2), lerp0(b0, b1, b2)};
  const bool use_sn = S.prim_has_normals[prim] != 0;
  D3 n0{0, 0, 0}, n1{0, 0, 0}, n2{0, 0, 0};
  if (use_sn) {
    n0 = d3load(S.vnrm + 3 * j0);
    n1 = d3load(S.vnrm + 3 * j1);
    n2 = d3load(S.vnrm + 3 * j2);
  }
  const D3 gn = d3normalized(d3cross(d3sub(v1, v0), d3sub(v2, v0)));
  const D3 sn = use_sn ? d3normalized(d3add(d3add(d3scale(n0, b0), d3scale(n1, b1)), d3scale(n2, b2))) : gn;
  // tangent: zero uv determinant -> CoordinateSystem(shading normal)
  D3 tangent = coordinate_e2(sn);
  const D3 t2 = d3cross(sn, tangent);
  if (d3dot(t2, t2) > 2.220446049250313e-16) {
    const D3 tt = d3cross(t2, sn);
    const double l2 = d3dot(tt, tt);
    tangent = l2 > 0.0 ? d3scale(tt, __ddiv_rn(1.0, __dsqrt_rn(l2))) : tt;
  }
  // screen-space differentials
  D3 pdx = point, pdy = point, ndx = sn, ndy = sn;
  double duv[4] = {0.0, 0.0, 0.0, 0.0};
  double b1x, b2x, tx, b1y, b2y, ty;
  if (has_diff && plane_point(v0, v1, v2, pt(D3{r[8], r[9], r[10]}), vc(D3{r[11], r[12], r[13]}), b1x, b2x, tx) &&
      plane_point(v0, v1, v2, pt(D3{r[14], r[15], r[16]}), vc(D3{r[17], r[18], r[19]}), b1y, b2y, ty)) {
    const double b0x = __dsub_rn(__dsub_rn(1.0, b1x), b2x), b0y = __dsub_rn(__dsub_rn(1.0, b1y), b2y);
    pdx = d3add(pt(D3{r[8], r[9], r[10]}), d3scale(vc(D3{r[11], r[12], r[13]}), tx));
    pdy = d3add(pt(D3{r[14], r[15], r[16]}), d3scale(vc(D3{r[17], r[18], r[19]}), ty));
    duv[0] = __dsub_rn(lerp0(b0x, b1x, b2x), uv[0]);
    duv[1] = __dsub_rn(lerp0(b0x, b1x, b2x), uv[1]);
    duv[2] = __dsub_rn(lerp0(b0y, b1y, b2y), uv[0]);
    duv[3] = __dsub_rn(lerp0(b0y, b1y, b2y), uv[1]);
    if (use_sn) {
      ndx = d3normalized(d3add(d3add(d3scale(n0, b0x), d3scale(n1, b1x)), d3scale(n2, b2x)));
      ndy = d3normalized(d3add(d3add(d3scale(n0, b0y), d3scale(n1, b1y)), d3scale(n2, b2y)));
    } else {
      ndx = ndy = gn;
    }
  }
  // back to world space (identity: the Transform's own arithmetic)
  auto nrm = [&](D3 v) { return ident ? d3normalized(id_vector(v)) : v; };
  const D3 wp = pt(point);
  const D3 out3[9] = {wp, nrm(gn), nrm(sn), pt(pdx), pt(pdy), nrm(ndx), nrm(ndy), vc(tangent),
                      d3cross(d3sub(v1, v0), d3sub(v2, v0))};
  // m_dot uses world_to_mesh of the world point (TriangleAccelerator.cpp:345)
  const double mdot = d3dot(d3cross(d3sub(v0, pt(wp)), d3sub(v1, v0)), d3sub(v2, v0));
  // layout: point, geometric normal, shading normal, uv, point_dx, point_dy,
  // normal_dx, normal_dy, duv_dx, duv_dy, tangent, cross, dot, t
  const int at[9] = {0, 3, 6, 11, 14, 17, 20, 27, 30};
  for (int k = 0; k < 9; ++k) {
    o[at[k]] = out3[k].x;
    o[at[k] + 1] = out3[k].y;
    o[at[k] + 2] = out3[k].z;
  }
  o[9] = uv[0];
  o[10] = uv[1];
  for (int k = 0; k < 4; ++k) o[23 + k] = duv[k];
  o[33] = mdot;
  o[34] = __hiloint2double(hit.y, hit.x);
  ((int *)(o + 35))[0] = prim;
  ((int *)(o + 35))[1] = tri;
}

// Outgoing rays as the renders make them: from the float hit point of each
// closest hit in direction dirs[i], tmin = GetNextMinT (next_min_t), tmax =
// +inf; NaN rays for misses.
__global__ void k_next_rays(SceneDev S, const float4 *__restrict__ rays, const int4 *__restrict__ hits,
                            const float *__restrict__ dirs, int n, float4 *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int4 hit = hits[i];
  const V3 w = load3(dirs + 3 * (int64_t)i);
  if (hit.y < 0) {
    const float nanf_ = __int_as_float(0x7fc00000);
    out[2 * i] = make_float4(nanf_, nanf_, nanf_, nanf_);
    out[2 * i + 1] = make_float4(nanf_, nanf_, nanf_, nanf_);
    return;
  }
  const float4 ra = rays[2 * i], rb = rays[2 * i + 1];
  const Hit h = make_hit(S, v3(ra.x, ra.y, ra.z), v3(ra.w, rb.x, rb.y), __int_as_float(hit.x), hit.y, hit.z);
  store_ray(out, i, h.p, w, next_min_t(S, h, w), __int_as_float(0x7f800000));
}

}  // namespace

cudaError_t launch_hit_geometry(const SceneDev &S, const void *rays, const void *hits, int64_t n, double *out,
                                cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_hit_geometry<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(S, (const float4 *)rays, (const int4 *)hits, (int)n,
                                                              out);
  return cudaGetLastError();
}

cudaError_t launch_intersection(const SceneDev &S, const void *rays, const void *hits, int64_t n, double *out,
                                cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_intersection<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(S, (const double *)rays, (const int4 *)hits, (int)n,
                                                              out);
  return cudaGetLastError();
}

cudaError_t launch_next_rays(const SceneDev &S, const void *rays, const void *hits, const float *dirs, int64_t n,
                             void *out, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_next_rays<<<(unsigned)((n + 127) / 128), 128, 0, s>>>(S, (const float4 *)rays, (const int4 *)hits, dirs, (int)n,
                                                          (float4 *)out);
  return cudaGetLastError();
}

cudaError_t launch_camera(const ViewDev *views, int n_views, int64_t px_begin, int n_px, int sppx, int sppy,
                          void *rays, cudaStream_t s, int ld) {
  const int64_t n = (int64_t)n_px * sppx * sppy;
  if (n <= 0) return cudaSuccess;
  k_camera<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(views, n_views, px_begin, n_px, sppx, sppy, ld,
                                                       (float4 *)rays);
  return cudaGetLastError();
}

cudaError_t launch_shade(const SceneDev &S, const ViewDev *views, int n_views, int n, int64_t px_begin, int spp,
                         int slots, int n_light_samples, const void *rays, const void *hits, float *contrib,
                         void *srays, int *starget, float *srgb, int *scount, void *brays, int *btarget, float *brgb,
                         int *bcount, float *bnrm, int block, cudaStream_t s, const SpecQueues *spec, int ld) {
  if (n <= 0) return cudaSuccess;
  if (block != 64) block = 128;
  ShadeArgs A{n, px_begin, spp, slots, n_light_samples, views, n_views, nullptr, ld};
  SpecArgs Q{};
  if (spec) {
    Q.out_rays = (float4 *)spec->out_rays;
    Q.out_w = spec->out_w;
    Q.out_sample = spec->out_sample;
    Q.out_node = spec->out_node;
    Q.out_count = spec->out_count;
    Q.depth = 0;
    Q.spec_slot = spec->spec_slot;
  }
  if (spec)
    k_shade<false, false, true><<<(unsigned)((n + block - 1) / block), (unsigned)block, 0, s>>>(
        S, A, AdjointArgs{}, Q, (const float4 *)rays, (const int4 *)hits, contrib, (float4 *)srays, starget, srgb,
        scount, (float4 *)brays, btarget, brgb, bcount, bnrm);
  else
    k_shade<false, false, false><<<(unsigned)((n + block - 1) / block), (unsigned)block, 0, s>>>(
        S, A, AdjointArgs{}, Q, (const float4 *)rays, (const int4 *)hits, contrib, (float4 *)srays, starget, srgb,
        scount, (float4 *)brays, btarget, brgb, bcount, bnrm);
  return cudaGetLastError();
}

cudaError_t launch_shade_specular(const SceneDev &S, const ViewDev *views, int n_views, int64_t capacity,
                                  int64_t px_begin, int spp, int slots, int n_light_samples, const SpecQueues &spec,
                                  int depth, const void *hits, float *contrib, void *srays, int *starget, float *srgb,
                                  int *scount, void *brays, int *btarget, float *brgb, int *bcount, float *bnrm,
                                  cudaStream_t s) {
  if (capacity <= 0) return cudaSuccess;
  ShadeArgs A{(int)capacity, px_begin, spp, slots, n_light_samples, views, n_views, nullptr, 0};
  SpecArgs Q{spec.in_w,      spec.in_sample, spec.in_node,  spec.in_count, (float4 *)spec.out_rays,
             spec.out_w,     spec.out_sample, spec.out_node, spec.out_count, depth,
             spec.spec_slot};
  const unsigned grid = (unsigned)std::min<int64_t>((capacity + 127) / 128, kStrideBlocks);
  if (spec.out_count)
    k_shade<false, true, true><<<grid, 128, 0, s>>>(
        S, A, AdjointArgs{}, Q, (const float4 *)spec.in_rays, (const int4 *)hits, contrib, (float4 *)srays, starget,
        srgb, scount, (float4 *)brays, btarget, brgb, bcount, bnrm);
  else
    k_shade<false, true, false><<<grid, 128, 0, s>>>(
        S, A, AdjointArgs{}, Q, (const float4 *)spec.in_rays, (const int4 *)hits, contrib, (float4 *)srays, starget,
        srgb, scount, (float4 *)brays, btarget, brgb, bcount, bnrm);
  return cudaGetLastError();
}

cudaError_t launch_shade_adjoint(const SceneDev &S, const ViewDev *views, int n_views, int n, int64_t px_begin, int spp,
                                 int n_light_samples, const float *dfilm, float *g_albedo, double *g_emission,
                                 const void *rays, const void *hits, void *srays, int *stri, float *s_dkd,
                                 float *s_dem, int *scount, void *brays, int *btri, float *b_dkd, float *brgb,
                                 int *bcount, float *bnrm, const float *tcam, cudaStream_t s, int ld,
                                 const SpecQueues *spec) {
  if (n <= 0) return cudaSuccess;
  ShadeArgs A{n, px_begin, spp, 0, n_light_samples, views, n_views, tcam, ld};
  AdjointArgs J{dfilm, g_albedo, g_emission, s_dkd, s_dem, b_dkd};
  SpecArgs Q{};
  if (spec) {
    Q.out_rays = (float4 *)spec->out_rays;
    Q.out_w = spec->out_w;
    Q.out_sample = spec->out_sample;
    Q.out_node = spec->out_node;
    Q.out_count = spec->out_count;
  }
  if (spec)
    k_shade<true, false, true><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(
        S, A, J, Q, (const float4 *)rays, (const int4 *)hits, nullptr, (float4 *)srays, stri, nullptr, scount,
        (float4 *)brays, btri, brgb, bcount, bnrm);
  else
    k_shade<true, false, false><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(
        S, A, J, Q, (const float4 *)rays, (const int4 *)hits, nullptr, (float4 *)srays, stri, nullptr, scount,
        (float4 *)brays, btri, brgb, bcount, bnrm);
  return cudaGetLastError();
}

cudaError_t launch_shade_specular_adjoint(const SceneDev &S, const ViewDev *views, int n_views, int64_t capacity,
                                          int64_t px_begin, int spp, int n_light_samples, const float *dfilm,
                                          float *g_albedo, double *g_emission, const SpecQueues &spec, int depth,
                                          const void *hits, void *srays, int *stri, float *s_dkd, float *s_dem,
                                          int *scount, void *brays, int *btri, float *b_dkd, float *brgb,
                                          int *bcount, float *bnrm, cudaStream_t s, const float *tcam) {
  if (capacity <= 0) return cudaSuccess;
  ShadeArgs A{(int)capacity, px_begin, spp, 0, n_light_samples, views, n_views, tcam, 0};
  AdjointArgs J{dfilm, g_albedo, g_emission, s_dkd, s_dem, b_dkd};
  SpecArgs Q{spec.in_w,      spec.in_sample, spec.in_node,  spec.in_count, (float4 *)spec.out_rays,
             spec.out_w,     spec.out_sample, spec.out_node, spec.out_count, depth,
             0};
  const unsigned grid = (unsigned)std::min<int64_t>((capacity + 127) / 128, kStrideBlocks);
  if (spec.out_count)
    k_shade<true, true, true><<<grid, 128, 0, s>>>(
        S, A, J, Q, (const float4 *)spec.in_rays, (const int4 *)hits, nullptr, (float4 *)srays, stri, nullptr, scount,
        (float4 *)brays, btri, brgb, bcount, bnrm);
  else
    k_shade<true, true, false><<<grid, 128, 0, s>>>(
        S, A, J, Q, (const float4 *)spec.in_rays, (const int4 *)hits, nullptr, (float4 *)srays, stri, nullptr, scount,
        (float4 *)brays, btri, brgb, bcount, bnrm);
  return cudaGetLastError();
}

cudaError_t launch_resolve_adjoint(const SceneDev &S, int capacity, int n_light_samples, const uint8_t *occ,
                                   const int *stri, const float *s_dkd, const float *s_dem, const int *scount,
                                   const void *brays, const void *bhits, const int *btri, const float *b_dkd,
                                   const float *brgb, const int *bcount, const float *bnrm, float *g_albedo,
                                   double *g_emission, cudaStream_t s, bool capped) {
  if (capacity <= 0) return cudaSuccess;
  AdjointArgs J{nullptr, g_albedo, g_emission, const_cast<float *>(s_dkd), const_cast<float *>(s_dem),
                const_cast<float *>(b_dkd)};
  const unsigned grid = (unsigned)(capped ? std::min<int64_t>((capacity + 255) / 256, kStrideBlocks)
                                          : (capacity + 255) / 256);
  k_resolve_shadow_adj<<<grid, 256, 0, s>>>(occ, stri, scount, J);
  k_resolve_bsdf_adj<<<grid, 256, 0, s>>>(S, n_light_samples, (const float4 *)brays, (const int4 *)bhits, btri, brgb,
                                          bcount, bnrm, J);
  return cudaGetLastError();
}

cudaError_t launch_resolve(const SceneDev &S, int capacity, int n_light_samples, const uint8_t *occ,
                           const int *starget, const float *srgb, const int *scount, const void *brays,
                           const void *bhits, const int *btarget, const float *brgb, const int *bcount,
                           const float *bnrm, float *contrib, cudaStream_t s, bool accumulate) {
  if (capacity <= 0) return cudaSuccess;
  // a specular level (accumulate) strides with a capped grid over its queue
  const unsigned grid = (unsigned)(accumulate ? std::min<int64_t>((capacity + 255) / 256, kStrideBlocks)
                                              : (capacity + 255) / 256);
  k_resolve_shadow<<<grid, 256, 0, s>>>(occ, starget, srgb, scount, contrib, accumulate);
  k_resolve_bsdf<<<grid, 256, 0, s>>>(S, n_light_samples, (const float4 *)brays, (const int4 *)bhits, btarget, brgb,
                                      bcount, bnrm, contrib, accumulate);
  return cudaGetLastError();
}

cudaError_t launch_film(const float *contrib, int64_t px_begin, int n_px, int spp, int slots, float *film,
                        cudaStream_t s, const float *tcam, int media_slot) {
  if (n_px <= 0) return cudaSuccess;
  k_film<<<(unsigned)((n_px + 127) / 128), 128, 0, s>>>(contrib, px_begin, n_px, spp, slots, tcam, media_slot, film);
  return cudaGetLastError();
}

cudaError_t launch_media(bool adjoint, const SceneDev &S, const ViewDev *views, int n_views, int n, int64_t px_begin,
                         int spp, int slots, int media_slot, const float *dfilm, const void *rays, const void *hits,
                         float *contrib, float *tcam, void *mrays, int *mtarget, float *mval, float *mdem,
                         int *mcount, unsigned *status, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  MediaArgs A{n, px_begin, spp, slots, media_slot, views, n_views, nullptr, nullptr, nullptr, 0, nullptr, nullptr, 0,
              nullptr};
  AdjointArgs J{dfilm, nullptr, nullptr, nullptr, nullptr, nullptr};
  const unsigned grid = (unsigned)((n + 127) / 128);
  if (adjoint)
    k_media<true><<<grid, 128, 0, s>>>(S, A, J, (const float4 *)rays, (const int4 *)hits, contrib, tcam,
                                       (float4 *)mrays, mtarget, mval, mdem, mcount, status);
  else
    k_media<false><<<grid, 128, 0, s>>>(S, A, J, (const float4 *)rays, (const int4 *)hits, contrib, tcam,
                                        (float4 *)mrays, mtarget, mval, mdem, mcount, status);
  return cudaGetLastError();
}

cudaError_t launch_media_specular(bool adjoint, const SceneDev &S, const ViewDev *views, int n_views, int n,
                                  int64_t px_begin, int spp, int slots, int spec_slot, const void *rays,
                                  const void *hits, const int *in_sample, float *in_w, const int *in_node,
                                  const MediaChunk &chunk, const float *dfilm, const float *tcam, float *contrib,
                                  void *mrays, int *mtarget, float *mval, float *mdem, int *mcount,
                                  unsigned *status, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  MediaArgs A{n,         px_begin, spp,    slots,         0,          views,       n_views,
              in_sample, in_w,     in_node, spec_slot, chunk.off_dev, chunk.count_dev, chunk.capacity, tcam};
  AdjointArgs J{dfilm, nullptr, nullptr, nullptr, nullptr, nullptr};
  const unsigned grid = (unsigned)((n + 127) / 128);
  if (adjoint)
    k_media<true><<<grid, 128, 0, s>>>(S, A, J, (const float4 *)rays, (const int4 *)hits, contrib, nullptr,
                                       (float4 *)mrays, mtarget, mval, mdem, mcount, status);
  else
    k_media<false><<<grid, 128, 0, s>>>(S, A, J, (const float4 *)rays, (const int4 *)hits, contrib, nullptr,
                                        (float4 *)mrays, mtarget, mval, mdem, mcount, status);
  return cudaGetLastError();
}

// The end of a device-counted chunk loop: the next chunk's offset, and the
// loop's condition (another chunk remains).
__global__ void k_media_advance(cudaGraphConditionalHandle h, int *off, const int *count, int chunk, int64_t capacity) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int64_t o = (int64_t)*off + chunk;
  *off = (int)min(o, (int64_t)INT32_MAX);
  cudaGraphSetConditional(h, o < min((int64_t)*count, capacity) ? 1u : 0u);
}

cudaError_t launch_media_advance(cudaGraphConditionalHandle h, int *off, const int *count, int chunk,
                                 int64_t capacity, cudaStream_t s) {
  k_media_advance<<<1, 32, 0, s>>>(h, off, count, chunk, capacity);
  return cudaGetLastError();
}

cudaError_t launch_resolve_media(bool adjoint, int64_t capacity, const uint8_t *occ, const int *mtarget,
                                 const float *mval, const float *mdem, const int *mcount, int slots, int media_slot,
                                 float *contrib, double *g_emission, cudaStream_t s) {
  if (capacity <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)((capacity + 255) / 256);
  if (adjoint)
    k_resolve_media<true><<<grid, 256, 0, s>>>(occ, mtarget, mval, mdem, mcount, slots, media_slot, contrib,
                                               g_emission);
  else
    k_resolve_media<false><<<grid, 256, 0, s>>>(occ, mtarget, mval, mdem, mcount, slots, media_slot, contrib,
                                                g_emission);
  return cudaGetLastError();
}

}  // namespace skw
