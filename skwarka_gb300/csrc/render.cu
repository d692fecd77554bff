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
#include <cstdint>

#include "kernels.h"
#include "render_scene.h"

namespace skw {
namespace {

constexpr float kPi = 3.14159265358979f;
constexpr float kInvPi = 0.318309886183791f;
constexpr float kEps = 2.220446e-16f;  // the reference's DBL_EPS thresholds, kept as tiny floats

// ---------------------------------------------------------------- random --
// SplitMix64 finaliser (Steele, Lea, Flood 2014) over (seed, sample, dim).
__device__ __forceinline__ float rnd(uint64_t seed, uint64_t sample, uint32_t dim) {
  uint64_t z = seed + 0x9E3779B97F4A7C15ull * (sample * 64ull + dim + 1ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  return (float)(z >> 40) * (1.0f / 16777216.0f);  // 24 bits: in [0, 1)
}

// ----------------------------------------------------------------- vectors --
struct V3 {
  float x, y, z;
};
__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
__device__ __forceinline__ V3 mul(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return v3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float len(V3 a) { return sqrtf(dot(a, a)); }
__device__ __forceinline__ V3 normalized(V3 a) {
  const float l2 = dot(a, a);
  return l2 > 0.0f ? a * (1.0f / sqrtf(l2)) : a;
}
__device__ __forceinline__ V3 load3(const float *p) { return v3(p[0], p[1], p[2]); }
__device__ __forceinline__ bool black(V3 a) { return a.x == 0.0f && a.y == 0.0f && a.z == 0.0f; }

// ------------------------------------------------------------ sampling --
// SamplingRoutines::ConcentricDiskSampling (Math/SamplingRoutines.h:197-241).
__device__ __forceinline__ void concentric_disk(float u0, float u1, float &dx, float &dy) {
  const float sx = 2.0f * u0 - 1.0f, sy = 2.0f * u1 - 1.0f;
  if (sx == 0.0f && sy == 0.0f) {
    dx = dy = 0.0f;
    return;
  }
  float r, theta;
  if (sx >= -sy) {
    if (sx > sy) {
      r = sx;
      theta = sy > 0.0f ? sy / r : 8.0f + sy / r;
    } else {
      r = sy;
      theta = 2.0f - sx / r;
    }
  } else {
    if (sx <= sy) {
      r = -sx;
      theta = 4.0f - sy / r;
    } else {
      r = -sy;
      theta = 6.0f + sx / r;
    }
  }
  theta *= kPi / 4.0f;
  dx = r * cosf(theta);
  dy = r * sinf(theta);
}

// CosineHemisphereSampling (SamplingRoutines.h:282-291).
__device__ __forceinline__ V3 cosine_hemisphere(float u0, float u1) {
  float x, y;
  concentric_disk(u0, u1, x, y);
  return v3(x, y, sqrtf(fmaxf(0.0f, 1.0f - x * x - y * y)));
}

// PowerHeuristic (SamplingRoutines.h:449-455).
__device__ __forceinline__ float power_heuristic(int n1, float p1, int n2, float p2) {
  const float f = n1 * p1, g = n2 * p2;
  return (f * f) / (f * f + g * g);
}

// ------------------------------------------------------------------- BSDF --
struct Bsdf {
  V3 n, e1, e2, ng;  // shading frame and geometric normal
  int kind;
  V3 kd, ks;
  float exponent, on_a, on_b;
  V3 eta, k2;
  __device__ __forceinline__ V3 local(V3 w) const { return v3(dot(w, e1), dot(w, e2), dot(w, n)); }
  __device__ __forceinline__ V3 world(V3 l) const { return e1 * l.x + e2 * l.y + n * l.z; }
  __device__ __forceinline__ int components() const { return kind == kPlastic ? 2 : 1; }
};

// FresnelDielectric (Core/Fresnel.h:96-124), inner 1.5, outer 1.0.
__device__ __forceinline__ float fresnel_dielectric(float c) {
  c = fminf(1.0f, fmaxf(-1.0f, c));
  float ni = 1.5f, no = 1.0f;
  if (c < 0.0f) {
    ni = 1.0f;
    no = 1.5f;
  }
  const float st = no / ni * sqrtf(fmaxf(0.0f, 1.0f - c * c));
  if (st >= 1.0f) return 1.0f;
  const float ct = sqrtf(fmaxf(0.0f, 1.0f - st * st));
  c = fabsf(c);
  const float rpar = (ni * c - no * ct) / (ni * c + no * ct);
  const float rper = (no * c - ni * ct) / (no * c + ni * ct);
  return (rpar * rpar + rper * rper) * 0.5f;
}

// FresnelConductor (Core/Fresnel.h:132-145), per channel.
__device__ __forceinline__ float fresnel_conductor1(float c, float eta, float k2) {
  c = fabsf(c);
  const float t1 = eta * eta + k2, t2 = t1 * (c * c);
  const float rpar = (t2 - (2.0f * c) * eta + 1.0f) / (t2 + (2.0f * c) * eta + 1.0f);
  const float rper = (t1 - (2.0f * eta * c) + c * c) / (t1 + (2.0f * eta * c) + c * c);
  return (rpar + rper) * 0.5f;
}

// Microfacet<Fresnel, Blinn>::Evaluate (BxDFs/Microfacet.h:86-104) for the
// glossy component of plastic (ks, dielectric) or metal (1, conductor).
__device__ V3 microfacet_eval(const Bsdf &b, V3 wi, V3 wo) {
  const float ci = fabsf(wi.z), co = fabsf(wo.z);
  if (ci < kEps || co < kEps) return v3(0, 0, 0);
  V3 h = wi + wo;
  if (fabsf(h.x) < kEps && fabsf(h.y) < kEps && fabsf(h.z) < kEps) return v3(0, 0, 0);
  h = normalized(h);
  const float ch = dot(wo, h);
  const float d = (b.exponent + 2.0f) * (0.5f * kInvPi) * powf(fabsf(h.z), b.exponent);
  const float tmp = 2.0f * fabsf(h.z) / fabsf(dot(wi, h));
  const float g = fminf(1.0f, fminf(ci * tmp, co * tmp));
  const float s = d * g / (4.0f * ci * co);
  if (b.kind == kPlastic) return b.ks * (fresnel_dielectric(ch) * s);
  return v3(fresnel_conductor1(ch, b.eta.x, b.k2.x) * s, fresnel_conductor1(ch, b.eta.y, b.k2.y) * s,
            fresnel_conductor1(ch, b.eta.z, b.k2.z) * s);
}

// BlinnDistribution::PDF (MicrofacetDistributions/BlinnDistribution.h:104-111)
// inside Microfacet::PDF (Microfacet.h:125-134).
__device__ float microfacet_pdf(const Bsdf &b, V3 wi, V3 wo) {
  if (wi.z * wo.z < 0.0f) return 0.0f;
  const V3 h = normalized(wi + wo);
  return ((b.exponent + 1.0f) * powf(fabsf(h.z), b.exponent)) / (2.0f * kPi * 4.0f * fabsf(dot(wi, h)));
}

// Diffuse component: Lambertian (BxDFs/Lambertian.cpp:18-30) or the
// reference's Oren-Nayar (BxDFs/OrenNayar.cpp:19-42).
__device__ __forceinline__ V3 diffuse_eval(const Bsdf &b, V3 wi, V3 wo) {
  if (b.kind != kOrenNayar) return b.kd * kInvPi;
  const float dcos = fmaxf(0.0f, wi.x * wo.x + wi.y * wo.y);
  const float denom = fmaxf(fabsf(wi.z), fabsf(wo.z));
  return b.kd * (kInvPi * (b.on_a + b.on_b * dcos / denom));
}
__device__ __forceinline__ float diffuse_pdf(V3 wi, V3 wo) {  // BxDF::PDF (Core/BxDF.cpp:33-37)
  return wi.z * wo.z > 0.0f ? fabsf(wo.z) * kInvPi : 0.0f;
}

// BSDF::Evaluate (Core/BSDF.cpp:22-40): every component is a reflection, so
// directions on opposite sides of the geometric normal give zero.
__device__ V3 bsdf_eval(const Bsdf &b, V3 wi_w, V3 wo_w) {
  if (!(dot(wi_w, b.ng) * dot(wo_w, b.ng) > 0.0f)) return v3(0, 0, 0);
  const V3 wi = b.local(wi_w), wo = b.local(wo_w);
  if (b.kind == kMetal) return microfacet_eval(b, wi, wo);
  V3 f = diffuse_eval(b, wi, wo);
  if (b.kind == kPlastic) f = f + microfacet_eval(b, wi, wo);
  return f;
}

// The derivative of bsdf_eval with respect to kd (per channel): the diffuse
// component evaluated with kd = 1 (zero for metal, whose BSDF has no kd).
__device__ V3 bsdf_eval_dkd(const Bsdf &b, V3 wi_w, V3 wo_w) {
  if (b.kind == kMetal || !(dot(wi_w, b.ng) * dot(wo_w, b.ng) > 0.0f)) return v3(0, 0, 0);
  Bsdf u = b;
  u.kd = v3(1.0f, 1.0f, 1.0f);
  return diffuse_eval(u, b.local(wi_w), b.local(wo_w));
}

// BSDF::PDF (Core/BSDF.cpp:42-58): average of the component densities.
__device__ float bsdf_pdf(const Bsdf &b, V3 wi_w, V3 wo_w) {
  const V3 wi = b.local(wi_w), wo = b.local(wo_w);
  if (b.kind == kMetal) return microfacet_pdf(b, wi, wo);
  if (b.kind == kPlastic) return 0.5f * (diffuse_pdf(wi, wo) + microfacet_pdf(b, wi, wo));
  return diffuse_pdf(wi, wo);
}

// BSDF::Sample (Core/BSDF.cpp:110-168) over the non-specular components:
// pick a component uniformly, sample it, average the densities of all
// components at the sampled direction, evaluate the whole BSDF.
__device__ V3 bsdf_sample(const Bsdf &b, V3 wi_w, float uc, float u0, float u1, V3 &wo_w, float &pdf) {
  const V3 wi = b.local(wi_w);
  const int nc = b.components();
  const int comp = min((int)(uc * nc), nc - 1);
  V3 wo;
  const bool glossy = b.kind == kMetal || (b.kind == kPlastic && comp == 1);
  if (glossy) {
    // BlinnDistribution::Sample (BlinnDistribution.h:86-101)
    const float ct = powf(u0, 1.0f / (b.exponent + 1.0f));
    const float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
    const float phi = u1 * 2.0f * kPi;
    V3 h = v3(st * cosf(phi), st * sinf(phi), ct);
    if (wi.z * h.z < 0.0f) h.z = -h.z;
    wo = h * (2.0f * dot(wi, h)) - wi;
    if (wi.z * wo.z < 0.0f) {  // Microfacet::Sample rejects the wrong hemisphere
      pdf = 0.0f;
      wo_w = b.world(wo);
      return v3(0, 0, 0);
    }
  } else {
    // BxDF::Sample (Core/BxDF.cpp:20-31): cosine hemisphere on the incident side
    wo = cosine_hemisphere(u0, u1);
    if (wi.z < 0.0f) wo.z = -wo.z;
  }
  wo_w = b.world(wo);
  if (b.kind == kMetal) {
    pdf = microfacet_pdf(b, wi, wo);
  } else if (b.kind == kPlastic) {
    pdf = 0.5f * (diffuse_pdf(wi, wo) + microfacet_pdf(b, wi, wo));
  } else {
    pdf = diffuse_pdf(wi, wo);
  }
  return bsdf_eval(b, wi_w, wo_w);
}

// ------------------------------------------------------------------ shading --
struct Hit {
  V3 p, ng, ns;
  V3 v0, cr;  // triangle vertex 0 and (v1 - v0) x (v2 - v0), for the next ray's tmin
  int g;      // global triangle
};

// Ray start offset for leaving a surface: past the point where the ray
// crosses the triangle's plane (CoreUtils::GetNextMinT, CoreUtils.h:139-149),
// plus a margin for the float hit point.
__device__ __forceinline__ float next_min_t(const Hit &h, V3 w, float scene_abs) {
  const float den = dot(w, h.cr);
  float t = 0.0f;
  if (den != 0.0f) t = fmaxf(0.0f, dot(h.v0 - h.p, h.cr) / den);
  return t + 2.0e-6f * (1.0f + scene_abs);
}

__device__ Bsdf make_bsdf(const SceneDev &S, const Hit &h, int prim) {
  const DevMaterial m = S.materials[S.prim_material[prim]];
  Bsdf b;
  b.ng = h.ng;
  b.n = h.ns;
  // Any frame around the shading normal: all the BxDFs here are isotropic.
  const V3 a = fabsf(b.n.x) > 0.9f ? v3(0, 1, 0) : v3(1, 0, 0);
  b.e1 = normalized(cross(a, b.n));
  b.e2 = cross(b.n, b.e1);
  b.kind = m.kind;
  b.kd = load3(m.kd);
  if (S.tri_albedo) {
    const float *ta = S.tri_albedo + 3 * (int64_t)h.g;
    if (ta[0] == ta[0]) b.kd = v3(fminf(1.0f, fmaxf(0.0f, ta[0])), fminf(1.0f, fmaxf(0.0f, ta[1])),
                                  fminf(1.0f, fmaxf(0.0f, ta[2])));
  }
  b.ks = load3(m.ks);
  b.exponent = m.exponent;
  b.on_a = m.on_a;
  b.on_b = m.on_b;
  b.eta = load3(m.eta);
  b.k2 = load3(m.k2);
  return b;
}

__device__ Hit make_hit(const SceneDev &S, V3 o, V3 d, float t, int prim, int tri) {
  Hit h;
  h.g = S.prim_tri_offset[prim] + tri;
  const int i0 = S.tri_vidx[3 * h.g], i1 = S.tri_vidx[3 * h.g + 1], i2 = S.tri_vidx[3 * h.g + 2];
  const V3 p0 = load3(S.vpos + 3 * i0), p1 = load3(S.vpos + 3 * i1), p2 = load3(S.vpos + 3 * i2);
  h.p = o + d * t;
  h.v0 = p0;
  h.cr = cross(p1 - p0, p2 - p0);
  h.ng = normalized(h.cr);
  h.ns = h.ng;
  if (S.prim_has_normals[prim]) {
    // barycentrics of the hit point (Moller-Trumbore), then the
    // interpolated vertex normal (TriangleMesh.cpp:478-484)
    const V3 e1 = p1 - p0, e2 = p2 - p0, s1 = cross(d, e2);
    const float inv = 1.0f / dot(s1, e1);
    const V3 dd = o - p0;
    const float b1 = dot(dd, s1) * inv;
    const float b2 = dot(d, cross(dd, e1)) * inv;
    const float b0 = 1.0f - b1 - b2;
    const V3 n = load3(S.vnrm + 3 * i0) * b0 + load3(S.vnrm + 3 * i1) * b1 + load3(S.vnrm + 3 * i2) * b2;
    h.ns = normalized(n);
  }
  return h;
}

// Warp-aggregated append: one atomic per warp for the lanes with `want`.
__device__ __forceinline__ int queue_append(bool want, int *count) {
  const unsigned mask = __ballot_sync(__activemask(), want);
  if (!want) return -1;
  const int leader = __ffs(mask) - 1;
  const int lane = threadIdx.x & 31;
  int base = 0;
  if (lane == leader) base = atomicAdd(count, __popc(mask));
  base = __shfl_sync(mask, base, leader);
  return base + __popc(mask & ((1u << lane) - 1u));
}

__device__ __forceinline__ void store_ray(float4 *rays, int i, V3 o, V3 d, float tmin, float tmax) {
  rays[2 * i] = make_float4(o.x, o.y, o.z, d.x);
  rays[2 * i + 1] = make_float4(d.y, d.z, tmin, tmax);
}

__device__ __forceinline__ void store_rgb(float *c, int64_t slot, V3 v) {
  c[3 * slot] = v.x;
  c[3 * slot + 1] = v.y;
  c[3 * slot + 2] = v.z;
}

// The view holding global pixel P: the last view whose first pixel is <= P.
__device__ __forceinline__ int find_view(const ViewDev *__restrict__ views, int n_views, int64_t P) {
  int lo = 0, hi = n_views - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (views[mid].px_begin <= P) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Camera rays for the samples of global pixels [px_begin, px_begin + n_px).
__global__ void k_camera(const ViewDev *__restrict__ views, int n_views, int64_t px_begin, int n_px, int sppx,
                         int sppy, float4 *__restrict__ rays) {
  const int spp = sppx * sppy;
  const int64_t s = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= (int64_t)n_px * spp) return;
  const int64_t P = px_begin + s / spp;
  const int j = (int)(s % spp);
  const int v = find_view(views, n_views, P);
  const CameraDev &cam = views[v].cam;
  const int64_t px = P - views[v].px_begin;
  const int x = (int)(px % cam.width), y = (int)(px / cam.width);
  const uint64_t gid = (uint64_t)px * spp + j, seed = views[v].seed;
  // stratified, jittered pixel sample (StratifiedSampling2D)
  const double ix = x + ((j % sppx) + (double)rnd(seed, gid, 0)) / sppx;
  const double iy = y + ((j / sppx) + (double)rnd(seed, gid, 1)) / sppy;
  // PerspectiveCamera::GenerateRay (pinhole)
  const double cx = 2.0 * cam.x_tan * (ix - cam.width * 0.5) / cam.width;
  const double cy = 2.0 * cam.y_tan * (iy - cam.height * 0.5) / cam.height;
  const double *m = cam.c2w;
  const double ox = m[3], oy = m[7], oz = m[11];
  double dx = m[0] * cx + m[1] * cy + m[2];
  double dy = m[4] * cx + m[5] * cy + m[6];
  double dz = m[8] * cx + m[9] * cy + m[10];
  const double il = 1.0 / sqrt(dx * dx + dy * dy + dz * dz);
  dx *= il;
  dy *= il;
  dz *= il;
  rays[2 * s] = make_float4((float)ox, (float)oy, (float)oz, (float)dx);
  rays[2 * s + 1] = make_float4((float)dy, (float)dz, 0.0f, __int_as_float(0x7f800000));
}

struct ShadeArgs {
  int n;               // samples in this pass
  int64_t px_begin;    // global pixel of the pass's first sample
  int spp;
  int slots;           // contribution slots per sample
  int n_light_samples;
  const ViewDev *views;
  int n_views;
};

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
template <bool ADJ>
__global__ void __launch_bounds__(128) k_shade(SceneDev S, ShadeArgs A, AdjointArgs J, const float4 *__restrict__ rays,
                                               const int4 *__restrict__ hits, float *__restrict__ contrib,
                                               float4 *__restrict__ srays, int *__restrict__ starget,
                                               float *__restrict__ srgb, int *__restrict__ scount,
                                               float4 *__restrict__ brays, int *__restrict__ btarget,
                                               float *__restrict__ brgb, int *__restrict__ bcount) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = i < A.n;
  int4 hit = make_int4(0x7f800000, -1, -1, 0);
  float4 ra = make_float4(0, 0, 0, 0), rb = make_float4(0, 0, 0, 0);
  if (valid) {
    hit = hits[i];
    ra = rays[2 * i];
    rb = rays[2 * i + 1];
  }
  const bool surface = valid && hit.y >= 0;
  const int nl = A.n_light_samples;
  const int64_t slot0 = (int64_t)i * A.slots;
  uint64_t gid = 0, seed = 0;
  V3 dI = v3(0, 0, 0);  // adjoint: dL/dI of this sample's pixel / spp
  {
    const int64_t P = A.px_begin + (valid ? i : 0) / A.spp;
    const int v = find_view(A.views, A.n_views, P);
    gid = (uint64_t)((P - A.views[v].px_begin) * A.spp + (valid ? i : 0) % A.spp);
    seed = A.views[v].seed;
    if (ADJ && valid) dI = load3(J.dfilm + 3 * P) * (1.0f / A.spp);
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
      else store_rgb(contrib, slot0, le * escale);
    }
  }
  const V3 shading_n = b.n;

  // Light samples (DirectLightingIntegrator::_SampleLights, :158-262).  The
  // light is chosen uniformly among the area lights (any density gives the
  // same expectation; a single light -- all configurations -- has pdf 1).
  for (int k = 0; k < nl; ++k) {
    bool want = false;
    V3 val = v3(0, 0, 0), dir = v3(0, 0, 0), dkd = v3(0, 0, 0);
    float dem = 0.0f;
    float tmin = 0.0f, tmax = 0.0f;
    if (surface && S.n_area_lights > 0) {
      const float uc = rnd(seed, gid, 2 + 3 * k), u0 = rnd(seed, gid, 3 + 3 * k),
                  u1 = rnd(seed, gid, 4 + 3 * k);
      const int nls = S.n_area_lights;
      const int li = min((int)(uc * nls), nls - 1);
      const float lcp = 1.0f / nls;
      const float tri_u = uc * nls - li;  // the remaining fraction selects the triangle
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
          const V3 le = load3(L.radiance);
          val = mul(f, le) * (escale * w / nl);
          if (ADJ) {
            dkd = mul(dI, mul(bsdf_eval_dkd(b, wo, dir), le)) * (escale * w / nl);
            dem = dot(dI, mul(f, le)) * (w / nl);
          }
          tmin = next_min_t(h, dir, S.scene_abs);
          tmax = dist - 1e-4f;  // to avoid hitting the light itself (:237)
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
        starget[q] = (int)(slot0 + 1 + k);
        store_rgb(srgb, q, val);
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
        val = mul(f, load3(P.intensity)) * (inv * inv * fabsf(dot(dir, shading_n)));
        if (ADJ)
          dkd = mul(dI, mul(bsdf_eval_dkd(b, dir, wo), load3(P.intensity))) * (inv * inv * fabsf(dot(dir, shading_n)));
        tmin = next_min_t(h, dir, S.scene_abs);
        tmax = dist;
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
        starget[q] = (int)(slot0 + 1 + nl + k);
        store_rgb(srgb, q, val);
      }
    }
  }
  // BSDF samples (DirectLightingIntegrator::_SampleBSDF, :264-366).
  for (int k = 0; k < nl; ++k) {
    bool want = false;
    V3 val = v3(0, 0, 0), dir = v3(0, 0, 0), dkd = v3(0, 0, 0);
    float pdf = 0.0f, tmin = 0.0f;
    if (surface && S.n_area_lights > 0) {
      const float uc = rnd(seed, gid, 2 + 3 * nl + 3 * k), u0 = rnd(seed, gid, 3 + 3 * nl + 3 * k),
                  u1 = rnd(seed, gid, 4 + 3 * nl + 3 * k);
      const V3 f = bsdf_sample(b, wo, uc, u0, u1, dir, pdf);
      if (pdf > 0.0f && !black(f)) {
        val = f * (fabsf(dot(dir, shading_n)) / (pdf * nl));
        if (ADJ) {
          dkd = mul(dI, bsdf_eval_dkd(b, wo, dir)) * (fabsf(dot(dir, shading_n)) / (pdf * nl));
          val = mul(dI, val);
        }
        tmin = next_min_t(h, dir, S.scene_abs);
        want = true;
      }
    }
    const int q = queue_append(want, bcount);
    if (want) {
      store_ray(brays, q, h.p, dir, tmin, __int_as_float(0x7f800000));
      btarget[q] = ADJ ? h.g : (int)(slot0 + 1 + nl + S.n_point_lights + k);
      if (ADJ) store_rgb(J.b_dkd, q, dkd);
      brgb[4 * q] = val.x;
      brgb[4 * q + 1] = val.y;
      brgb[4 * q + 2] = val.z;
      brgb[4 * q + 3] = pdf;
    }
  }
  if (ADJ) add_emission_grad(J.g_emission, g_em);
}

__global__ void k_resolve_shadow(const uint8_t *__restrict__ occ, const int *__restrict__ starget,
                                 const float *__restrict__ srgb, const int *__restrict__ scount,
                                 float *__restrict__ contrib) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *scount || occ[i]) return;
  const int64_t t = starget[i];
  contrib[3 * t] = srgb[3 * i];
  contrib[3 * t + 1] = srgb[3 * i + 1];
  contrib[3 * t + 2] = srgb[3 * i + 2];
}

// A BSDF ray that hits the front of an area light adds its MIS-weighted
// emission (:300-318); the light density is DiffuseAreaLightSource::
// LightingPDF (:104-116).
__global__ void k_resolve_bsdf(SceneDev S, int n_light_samples, const float4 *__restrict__ brays,
                               const int4 *__restrict__ bhits, const int *__restrict__ btarget,
                               const float *__restrict__ brgb, const int *__restrict__ bcount,
                               float *__restrict__ contrib) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= *bcount) return;
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
  const float lcp = 1.0f / S.n_area_lights;
  const float bpdf = brgb[4 * i + 3];
  const float w = power_heuristic(n_light_samples, bpdf, n_light_samples, light_pdf * lcp);
  const int64_t t = btarget[i];
  const float sw = S.emission_scale * w;
  contrib[3 * t] = brgb[4 * i] * L.radiance[0] * sw;
  contrib[3 * t + 1] = brgb[4 * i + 1] * L.radiance[1] * sw;
  contrib[3 * t + 2] = brgb[4 * i + 2] * L.radiance[2] * sw;
}

// Adjoint of k_resolve_shadow: an unoccluded shadow ray adds its derivative
// terms to its triangle's albedo gradient and to the emission gradient.
__global__ void k_resolve_shadow_adj(const uint8_t *__restrict__ occ, const int *__restrict__ stri,
                                     const int *__restrict__ scount, AdjointArgs J) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float dem = 0.0f;
  if (i < *scount && !occ[i]) {
    const int64_t g = stri[i];
    const float *d = J.s_dkd + 3 * (int64_t)i;
    if (d[0] != 0.0f) atomicAdd(J.g_albedo + 3 * g, d[0]);
    if (d[1] != 0.0f) atomicAdd(J.g_albedo + 3 * g + 1, d[1]);
    if (d[2] != 0.0f) atomicAdd(J.g_albedo + 3 * g + 2, d[2]);
    dem = J.s_dem[i];
  }
  add_emission_grad(J.g_emission, dem);
}

// Adjoint of k_resolve_bsdf (same light density and MIS weight).
__global__ void k_resolve_bsdf_adj(SceneDev S, int n_light_samples, const float4 *__restrict__ brays,
                                   const int4 *__restrict__ bhits, const int *__restrict__ btri,
                                   const float *__restrict__ brgb, const int *__restrict__ bcount, AdjointArgs J) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float dem = 0.0f;
  if (i < *bcount) {
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
        const float lcp = 1.0f / S.n_area_lights;
        const float w = power_heuristic(n_light_samples, brgb[4 * i + 3], n_light_samples, light_pdf * lcp);
        const V3 le = load3(L.radiance);
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

// Luminance weights of the reference's RGB spectrum (row Y of its
// Spectrum-to-XYZ matrix, Core/SpectrumRoutines.cpp:20-64), used by the
// renderer's negative-sample check.
__constant__ float kLumW[3] = {0.05316285f, 0.58515348f, 0.36168367f};

__global__ void k_film(const float *__restrict__ contrib, int64_t px_begin, int n_px, int spp, int slots,
                       float *__restrict__ film) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_px) return;
  float r = 0.0f, g = 0.0f, bb = 0.0f;
  for (int j = 0; j < spp; ++j) {
    const int64_t base = ((int64_t)p * spp + j) * slots;
    float sr = 0.0f, sg = 0.0f, sb = 0.0f;
    for (int k = 0; k < slots; ++k) {
      sr += contrib[3 * (base + k)];
      sg += contrib[3 * (base + k) + 1];
      sb += contrib[3 * (base + k) + 2];
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

}  // namespace

cudaError_t launch_camera(const ViewDev *views, int n_views, int64_t px_begin, int n_px, int sppx, int sppy,
                          void *rays, cudaStream_t s) {
  const int64_t n = (int64_t)n_px * sppx * sppy;
  if (n <= 0) return cudaSuccess;
  k_camera<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(views, n_views, px_begin, n_px, sppx, sppy, (float4 *)rays);
  return cudaGetLastError();
}

cudaError_t launch_shade(const SceneDev &S, const ViewDev *views, int n_views, int n, int64_t px_begin, int spp,
                         int slots, int n_light_samples, const void *rays, const void *hits, float *contrib,
                         void *srays, int *starget, float *srgb, int *scount, void *brays, int *btarget, float *brgb,
                         int *bcount, int block, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  if (block != 64) block = 128;
  ShadeArgs A{n, px_begin, spp, slots, n_light_samples, views, n_views};
  k_shade<false><<<(unsigned)((n + block - 1) / block), (unsigned)block, 0, s>>>(
      S, A, AdjointArgs{}, (const float4 *)rays, (const int4 *)hits, contrib, (float4 *)srays, starget, srgb, scount,
      (float4 *)brays, btarget, brgb, bcount);
  return cudaGetLastError();
}

cudaError_t launch_shade_adjoint(const SceneDev &S, const ViewDev *views, int n_views, int n, int64_t px_begin, int spp,
                                 int n_light_samples, const float *dfilm, float *g_albedo, double *g_emission,
                                 const void *rays, const void *hits, void *srays, int *stri, float *s_dkd,
                                 float *s_dem, int *scount, void *brays, int *btri, float *b_dkd, float *brgb,
                                 int *bcount, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  ShadeArgs A{n, px_begin, spp, 0, n_light_samples, views, n_views};
  AdjointArgs J{dfilm, g_albedo, g_emission, s_dkd, s_dem, b_dkd};
  k_shade<true><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(S, A, J, (const float4 *)rays, (const int4 *)hits,
                                                             nullptr, (float4 *)srays, stri, nullptr, scount,
                                                             (float4 *)brays, btri, brgb, bcount);
  return cudaGetLastError();
}

cudaError_t launch_resolve_adjoint(const SceneDev &S, int capacity, int n_light_samples, const uint8_t *occ,
                                   const int *stri, const float *s_dkd, const float *s_dem, const int *scount,
                                   const void *brays, const void *bhits, const int *btri, const float *b_dkd,
                                   const float *brgb, const int *bcount, float *g_albedo, double *g_emission,
                                   cudaStream_t s) {
  if (capacity <= 0) return cudaSuccess;
  AdjointArgs J{nullptr, g_albedo, g_emission, const_cast<float *>(s_dkd), const_cast<float *>(s_dem),
                const_cast<float *>(b_dkd)};
  const unsigned grid = (unsigned)((capacity + 255) / 256);
  k_resolve_shadow_adj<<<grid, 256, 0, s>>>(occ, stri, scount, J);
  k_resolve_bsdf_adj<<<grid, 256, 0, s>>>(S, n_light_samples, (const float4 *)brays, (const int4 *)bhits, btri, brgb,
                                          bcount, J);
  return cudaGetLastError();
}

cudaError_t launch_resolve(const SceneDev &S, int capacity, int n_light_samples, const uint8_t *occ,
                           const int *starget, const float *srgb, const int *scount, const void *brays,
                           const void *bhits, const int *btarget, const float *brgb, const int *bcount,
                           float *contrib, cudaStream_t s) {
  if (capacity <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)((capacity + 255) / 256);
  k_resolve_shadow<<<grid, 256, 0, s>>>(occ, starget, srgb, scount, contrib);
  k_resolve_bsdf<<<grid, 256, 0, s>>>(S, n_light_samples, (const float4 *)brays, (const int4 *)bhits, btarget, brgb,
                                      bcount, contrib);
  return cudaGetLastError();
}

cudaError_t launch_film(const float *contrib, int64_t px_begin, int n_px, int spp, int slots, float *film,
                        cudaStream_t s) {
  if (n_px <= 0) return cudaSuccess;
  k_film<<<(unsigned)((n_px + 127) / 128), 128, 0, s>>>(contrib, px_begin, n_px, spp, slots, film);
  return cudaGetLastError();
}

}  // namespace skw
