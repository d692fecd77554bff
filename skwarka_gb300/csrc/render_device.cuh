// Device helpers shared by the wavefront kernels (render.cu, photon.cu):
// counter-based random numbers, float vectors, the reference's sampling
// routines, BSDFs (Lambertian, Oren-Nayar, Blinn microfacet with dielectric
// or conductor Fresnel), hit differential geometry and queue appends.
// Each translation unit gets its own internal copy.
#pragma once

#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <cstdint>

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

// ------------------------------------------------------ low discrepancy --
// LDSampler (Samplers/LDSampler.cpp:91-190): per pixel and per requested
// sequence, spp groups of L points of one scrambled (0,2)-sequence
// (VanDerCorput x Sobol2, SamplingRoutines.h:468-490), the groups dealt to
// the pixel's samples in a random order and the points of a group in a
// random order.  The scrambles and orders come from a hash of (seed, pixel,
// sequence) instead of the reference's generator; the orders are affine
// permutations j -> (a j + b) mod m (a odd, m a power of two).
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ uint32_t affine_perm(uint32_t j, uint32_t m, uint64_t h) {
  return ((uint32_t)(h | 1u) * j + (uint32_t)(h >> 32)) & (m - 1u);
}
__device__ __forceinline__ float van_der_corput(uint32_t n, uint32_t scramble) {
  return (float)((__brev(n) ^ scramble) >> 8) * (1.0f / 16777216.0f);
}
__device__ __forceinline__ float sobol2(uint32_t n, uint32_t scramble) {
  for (uint32_t v = 1u << 31; n != 0; n >>= 1, v ^= v >> 1)
    if (n & 1u) scramble ^= v;
  return (float)(scramble >> 8) * (1.0f / 16777216.0f);
}
// Point index of element e (of L) of sequence `seq` for sample j (of spp)
// of pixel px, and the sequence's two scrambles.
__device__ __forceinline__ uint32_t ld_index(uint64_t seed, uint64_t px, uint32_t seq, uint32_t j, uint32_t spp,
                                             uint32_t e, uint32_t L, uint32_t &s1, uint32_t &s2) {
  const uint64_t h = mix64(seed + 0x9E3779B97F4A7C15ull * (px * 16ull + seq + 1ull));
  const uint64_t hs = mix64(h ^ 0x632BE59BD9B4E019ull);
  s1 = (uint32_t)hs;
  s2 = (uint32_t)(hs >> 32);
  const uint32_t group = affine_perm(j, spp, mix64(h + 1ull));
  const uint32_t elem = L > 1u ? affine_perm(e, L, mix64(h + 2ull + j)) : 0u;
  return group * L + elem;
}
__device__ __forceinline__ float ld_1d(uint64_t seed, uint64_t px, uint32_t seq, uint32_t j, uint32_t spp, uint32_t e,
                                       uint32_t L) {
  uint32_t s1, s2;
  return van_der_corput(ld_index(seed, px, seq, j, spp, e, L, s1, s2), s1);
}
__device__ __forceinline__ void ld_2d(uint64_t seed, uint64_t px, uint32_t seq, uint32_t j, uint32_t spp, uint32_t e,
                                      uint32_t L, float &u0, float &u1) {
  uint32_t s1, s2;
  const uint32_t i = ld_index(seed, px, seq, j, spp, e, L, s1, s2);
  u0 = van_der_corput(i, s1);
  u1 = sobol2(i, s2);
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
// A BSDF is one or two layers (two for MixMaterial: each layer one of the
// other materials' BxDF sets, scaled -- ScaledBxDF, BxDFs/ScaledBxDF.cpp).
// A layer's non-specular components, in the order its material adds them:
//   kLambert, kOrenNayar: the diffuse BxDF          (1)
//   kPlastic: Lambertian(kd), Microfacet(ks, dielectric 1.5, Blinn)  (2)
//   kMetal: Microfacet(conductor, Blinn)            (1)
//   kMeasured: MERLMeasured                         (1)
//   kSubstrate: FresnelBlend<Blinn>(kd, ks)         (1)
//   kUber: Lambertian(kd) if kd is not black, Microfacet(ks, dielectric ior,
//          Blinn) if ks is not black                (0-2)
//   kTransparent: none
// and its specular ones: kTransparent SpecularReflection(kd) and
// SpecularTransmission(ks); kUber SpecularReflection(kr) and
// SpecularTransmission(kt) -- each only when its weight is not black.
struct Layer {
  int kind;
  V3 kd, ks, kr, kt;
  float exponent, on_a, on_b;
  float ior;    // dielectric Fresnel (inside index; outside 1)
  float pdiff;  // kSubstrate: probability of sampling the diffuse lobe
  float ev;     // kSubstrate: < 0 Blinn(exponent), else Ashikhmin-Shirley(exponent, ev)
  V3 eta, k2;
  MerlDev merl;
  V3 scale;
};
// The second layer of a mix is kept as its material (read again where it
// is needed, an L1-resident line) so that the common one-layer BSDF stays
// in registers.
struct Bsdf {
  V3 n, e1, e2, ng;  // shading frame and geometric normal
  int nl;            // layers (1, or 2 for a mix)
  Layer L0;
  const DevMaterial *m1;  // nl == 2: the second layer's material
  V3 s1;                  // nl == 2: its scale
  __device__ __forceinline__ V3 local(V3 w) const { return v3(dot(w, e1), dot(w, e2), dot(w, n)); }
  __device__ __forceinline__ V3 world(V3 l) const { return e1 * l.x + e2 * l.y + n * l.z; }
};

// FresnelDielectric(inner, 1)::operator() (Core/Fresnel.h:96-124).
__device__ __forceinline__ float fresnel_dielectric_ior(float c, float inner) {
  c = fminf(1.0f, fmaxf(-1.0f, c));
  float ni = inner, no = 1.0f;
  if (c < 0.0f) {
    ni = 1.0f;
    no = inner;
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

// BlinnDistribution::Evaluate (MicrofacetDistributions/BlinnDistribution.h).
__device__ __forceinline__ float blinn_d(float exponent, V3 h) {
  return (exponent + 2.0f) * (0.5f * kInvPi) * powf(fabsf(h.z), exponent);
}

// Microfacet<Fresnel, Blinn>::Evaluate (BxDFs/Microfacet.h:86-104): the
// glossy component of plastic and uber (ks, dielectric) or metal
// (conductor).
__device__ V3 microfacet_eval(const Layer &b, V3 wi, V3 wo) {
  const float ci = fabsf(wi.z), co = fabsf(wo.z);
  if (ci < kEps || co < kEps) return v3(0, 0, 0);
  V3 h = wi + wo;
  if (fabsf(h.x) < kEps && fabsf(h.y) < kEps && fabsf(h.z) < kEps) return v3(0, 0, 0);
  h = normalized(h);
  const float ch = dot(wo, h);
  const float d = blinn_d(b.exponent, h);
  const float tmp = 2.0f * fabsf(h.z) / fabsf(dot(wi, h));
  const float g = fminf(1.0f, fminf(ci * tmp, co * tmp));
  const float s = d * g / (4.0f * ci * co);
  if (b.kind != kMetal) return b.ks * (fresnel_dielectric_ior(ch, b.ior) * s);
  return v3(fresnel_conductor1(ch, b.eta.x, b.k2.x) * s, fresnel_conductor1(ch, b.eta.y, b.k2.y) * s,
            fresnel_conductor1(ch, b.eta.z, b.k2.z) * s);
}

// BlinnDistribution::PDF (MicrofacetDistributions/BlinnDistribution.h:104-111)
// inside Microfacet::PDF (Microfacet.h:125-134).
__device__ float microfacet_pdf(const Layer &b, V3 wi, V3 wo) {
  if (wi.z * wo.z < 0.0f) return 0.0f;
  const V3 h = normalized(wi + wo);
  return ((b.exponent + 1.0f) * powf(fabsf(h.z), b.exponent)) / (2.0f * kPi * 4.0f * fabsf(dot(wi, h)));
}

// BlinnDistribution::Sample (BlinnDistribution.h:86-101): the mirror of wi
// about a sampled half vector on wi's side; false (pdf 0) when wo falls in
// the other hemisphere, which Microfacet::Sample rejects.
__device__ __forceinline__ bool blinn_sample(float exponent, V3 wi, float u0, float u1, V3 &wo) {
  const float ct = powf(u0, 1.0f / (exponent + 1.0f));
  const float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
  const float phi = u1 * 2.0f * kPi;
  V3 h = v3(st * cosf(phi), st * sinf(phi), ct);
  if (wi.z * h.z < 0.0f) h.z = -h.z;
  wo = h * (2.0f * dot(wi, h)) - wi;
  return !(wi.z * wo.z < 0.0f);
}

// Diffuse component: Lambertian (BxDFs/Lambertian.cpp:18-30) or the
// reference's Oren-Nayar (BxDFs/OrenNayar.cpp:19-42).
__device__ __forceinline__ V3 diffuse_eval(const Layer &b, V3 wi, V3 wo) {
  if (b.kind != kOrenNayar) return b.kd * kInvPi;
  const float dcos = fmaxf(0.0f, wi.x * wo.x + wi.y * wo.y);
  const float denom = fmaxf(fabsf(wi.z), fabsf(wo.z));
  return b.kd * (kInvPi * (b.on_a + b.on_b * dcos / denom));
}
__device__ __forceinline__ float diffuse_pdf(V3 wi, V3 wo) {  // BxDF::PDF (Core/BxDF.cpp:33-37)
  return wi.z * wo.z > 0.0f ? fabsf(wo.z) * kInvPi : 0.0f;
}

// FresnelBlend<BlinnDistribution> (BxDFs/FresnelBlend.h): Ashikhmin and
// Shirley's diffuse substrate under a glossy coat.  Evaluate: the diffuse
// term (28 / 23 pi) kd (1 - ks) (1 - (1 - |cos o| / 2)^5)
// (1 - (1 - |cos i| / 2)^5) plus the Schlick-Fresnel-weighted Blinn term
// D(h) / (4 |o.h| max(|cos o|, |cos i|)).  The lobe is sampled as a mixture:
// the cosine lobe with probability pdiff (on wi's side), the Blinn half
// vector otherwise; the density is the mixture's (0 across hemispheres).
// AnisotropicDistribution (MicrofacetDistributions/AnisotropicDistribution.h):
// Ashikhmin and Shirley's half-vector distribution with exponents eu along
// the shading tangent (x) and ev across it (y).  Evaluate: sqrt((eu + 2)
// (ev + 2)) / 2 pi cos^e, e = (eu hx^2 + ev hy^2) / (1 - cos^2), 0 at the
// pole; PDF: sqrt((eu + 1)(ev + 1)) cos^e / (8 pi |wi.h|); Sample: the
// first quadrant's phi = atan(sqrt((eu + 1) / (ev + 1)) tan(pi u / 2)) (pi u
// / 2 when eu == ev) mirrored into the quadrant u0 selects, cos theta =
// u1^(1 / (eu cos^2 phi + ev sin^2 phi + 1)), the half vector on wi's side.
__device__ __forceinline__ float aniso_d(float eu, float ev, V3 h) {
  const float ct = fabsf(h.z), d = 1.0f - ct * ct;
  if (!(d > 0.0f)) return 0.0f;
  const float e = (eu * h.x * h.x + ev * h.y * h.y) / d;
  return sqrtf((eu + 2.0f) * (ev + 2.0f)) * (0.5f * kInvPi) * powf(ct, e);
}
__device__ __forceinline__ float aniso_pdf(float eu, float ev, V3 wi, V3 wo) {
  const V3 h = normalized(wi + wo);
  const float ct = fabsf(h.z), ds = 1.0f - ct * ct;
  if (!(ds > 0.0f)) return 0.0f;
  const float e = (eu * h.x * h.x + ev * h.y * h.y) / ds;
  return sqrtf((eu + 1.0f) * (ev + 1.0f)) * powf(ct, e) / (2.0f * kPi * 4.0f * fabsf(dot(wi, h)));
}
__device__ __forceinline__ bool aniso_sample(float eu, float ev, V3 wi, float u0, float u1, V3 &wo) {
  float s0;
  int q;
  if (u0 < 0.25f) {
    s0 = 4.0f * u0;
    q = 0;
  } else if (u0 < 0.5f) {
    s0 = 4.0f * (0.5f - u0);
    q = 1;
  } else if (u0 < 0.75f) {
    s0 = 4.0f * (u0 - 0.5f);
    q = 2;
  } else {
    s0 = 4.0f * (1.0f - u0);
    q = 3;
  }
  float phi = eu == ev ? kPi * s0 * 0.5f : atanf(sqrtf((eu + 1.0f) / (ev + 1.0f)) * tanf(kPi * s0 * 0.5f));
  const float cp = cosf(phi), sp = sinf(phi);
  const float ct = powf(u1, 1.0f / (eu * cp * cp + ev * sp * sp + 1.0f));
  if (q == 1) phi = kPi - phi;
  else if (q == 2) phi += kPi;
  else if (q == 3) phi = 2.0f * kPi - phi;
  const float st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
  V3 h = v3(st * cosf(phi), st * sinf(phi), ct);
  if (wi.z * h.z < 0.0f) h.z = -h.z;
  wo = h * (2.0f * dot(wi, h)) - wi;
  return !(wi.z * wo.z < 0.0f);
}

__device__ V3 fb_eval(const Layer &b, V3 wi, V3 wo) {
  const float ci = fabsf(wi.z), co = fabsf(wo.z);
  const V3 h = normalized(wi + wo);
  const float ch = dot(wo, h);
  const float t1 = 1.0f - 0.5f * co, t2 = 1.0f - 0.5f * ci;
  const float p1 = t1 * t1 * t1 * t1 * t1, p2 = t2 * t2 * t2 * t2 * t2;
  const V3 one = v3(1.0f, 1.0f, 1.0f);
  const V3 diffuse = mul(b.kd, one - b.ks) * ((28.0f / (23.0f * kPi)) * (1.0f - p1) * (1.0f - p2));
  const float m = 1.0f - fminf(1.0f, fabsf(ch)), m5 = m * m * m * m * m;
  const V3 schlick = b.ks + (one - b.ks) * m5;
  const float denom = 4.0f * fabsf(ch) * fmaxf(co, ci);
  const float dh = b.ev < 0.0f ? blinn_d(b.exponent, h) : aniso_d(b.exponent, b.ev, h);
  const V3 specular = denom > 0.0f ? schlick * (dh / denom) : v3(0, 0, 0);
  return diffuse + specular;
}
__device__ float fb_pdf(const Layer &b, V3 wi, V3 wo) {
  if (wi.z * wo.z < 0.0f) return 0.0f;
  const float pm = b.ev < 0.0f ? microfacet_pdf(b, wi, wo) : aniso_pdf(b.exponent, b.ev, wi, wo);
  return b.pdiff * fabsf(wo.z) * kInvPi + (1.0f - b.pdiff) * pm;
}
__device__ bool fb_sample(const Layer &b, V3 wi, float u0, float u1, V3 &wo) {
  if (u0 < b.pdiff) {
    wo = cosine_hemisphere(fminf(u0 / b.pdiff, 0.99999994f), u1);
    if (wi.z < 0.0f) wo.z = -wo.z;
    return true;
  }
  const float us = fminf((u0 - b.pdiff) / (1.0f - b.pdiff), 0.99999994f);
  return b.ev < 0.0f ? blinn_sample(b.exponent, wi, us, u1, wo) : aniso_sample(b.exponent, b.ev, wi, us, u1, wo);
}

// ------------------------------------------------------- measured BRDF --
// MERLMeasuredData::GetBRDF / Sample / PDF (BxDFs/MERLMeasured.cpp:254-369)
// in float, over the loader's half table and the sampling segmentations.
__device__ __forceinline__ float sph_theta(V3 v) { return acosf(fminf(1.0f, fmaxf(-1.0f, v.z))); }
__device__ __forceinline__ float sph_phi(V3 v) {
  const float p = atan2f(v.y, v.x);
  return p < 0.0f ? p + 2.0f * kPi : p;
}

__device__ V3 merl_brdf(const MerlDev &m, V3 wi, V3 wo) {
  V3 h = wi + wo;
  if (h.x == 0.0f && h.y == 0.0f && h.z == 0.0f) return v3(0, 0, 0);
  h = normalized(h);
  const float sin_t = sqrtf(h.x * h.x + h.y * h.y), cos_t = h.z;
  float sin_p = 0.0f, cos_p = 1.0f;
  if (sin_t > 1e-10f) {
    sin_p = h.y / sin_t;
    cos_p = h.x / sin_t;
  }
  const V3 whx = v3(cos_p * cos_t, sin_p * cos_t, -sin_t), why = v3(-sin_p, cos_p, 0.0f);
  const V3 diff = v3(dot(wi, whx), dot(wi, why), dot(wi, h));
  const float th = sph_theta(h), td = sph_theta(diff), pd = sph_phi(diff);
  const int ipd = (int)(pd * kInvPi * kMerlPhiD) % kMerlPhiD;
  const int itd = min((int)(td * 2.0f * kInvPi * kMerlThetaD), kMerlThetaD - 1);
  const float ths = sqrtf(th * 2.0f * kInvPi) * kMerlThetaH;
  const int ith = min((int)ths, kMerlThetaH - 1);
  const int idx = ipd + (itd + ith * kMerlThetaD) * kMerlPhiD;
  const uint16_t *t = m.table;
  V3 a = v3(__half2float(__ushort_as_half(t[3 * idx])), __half2float(__ushort_as_half(t[3 * idx + 1])),
            __half2float(__ushort_as_half(t[3 * idx + 2])));
  if (idx < (kMerlThetaH - 1) * kMerlThetaD * kMerlPhiD) {
    const float w = ths - (float)(int)ths;
    const int j = idx + kMerlThetaD * kMerlPhiD;
    const V3 b = v3(__half2float(__ushort_as_half(t[3 * j])), __half2float(__ushort_as_half(t[3 * j + 1])),
                    __half2float(__ushort_as_half(t[3 * j + 2])));
    a = a * (1.0f - w) + b * w;
  }
  return a;
}

__device__ __forceinline__ int merl_incident_bin(V3 wi) {
  return min((int)(sph_theta(wi) * 2.0f * kInvPi * kSegIncident), kSegIncident - 1);
}

__device__ float merl_data_pdf(const MerlDev &m, V3 wi, V3 wo) {
  const float *seg = m.seg + merl_incident_bin(wi) * kSegFloats;
  const float *cols = seg, *rows = seg + kSegTheta * kSegPhi, *gx = rows + kSegTheta, *gy = gx + kSegPhi;
  float dp = fabsf(sph_phi(wi) - sph_phi(wo));
  if (dp > kPi) dp = 2.0f * kPi - dp;
  const float px = dp * kInvPi, py = sph_theta(wo) * 2.0f * kInvPi;
  int ci = 0, ri = 0;  // last grid line <= the point (upper_bound - 1)
  while (ci + 1 < kSegPhi && gx[ci + 1] <= px) ++ci;
  while (ri + 1 < kSegTheta && gy[ri + 1] <= py) ++ri;
  const float bx0 = gx[ci], by0 = gy[ri];
  const float bx1 = ci + 1 < kSegPhi ? gx[ci + 1] : 1.0f, by1 = ri + 1 < kSegTheta ? gy[ri + 1] : 1.0f;
  const float *cc = cols + ri * kSegPhi;
  const float row_pdf = ri > 0 ? rows[ri] - rows[ri - 1] : rows[ri];
  const float col_pdf = ci > 0 ? cc[ci] - cc[ci - 1] : cc[ci];
  const float d_phi = (bx1 - bx0) * kPi, d_cos = cosf(by0 * (0.5f * kPi)) - cosf(by1 * (0.5f * kPi));
  return 0.5f * row_pdf * col_pdf / (d_phi * d_cos);
}

// MERLMeasured::Evaluate / PDF: the incident side's hemisphere folded to +z.
__device__ __forceinline__ V3 merl_eval(const MerlDev &m, V3 wi, V3 wo) {
  if (wi.z * wo.z < 0.0f) return v3(0, 0, 0);
  if (wi.z < 0.0f) {
    wi.z = -wi.z;
    wo.z = -wo.z;
  }
  return merl_brdf(m, wi, wo);
}
__device__ __forceinline__ float merl_pdf(const MerlDev &m, V3 wi, V3 wo) {
  if (wi.z * wo.z < 0.0f) return 0.0f;
  if (wi.z < 0.0f) {
    wi.z = -wi.z;
    wo.z = -wo.z;
  }
  return merl_data_pdf(m, wi, wo);
}

__device__ __forceinline__ int search_cdf_f(const float *cdf, int n, float u, float &pdf) {
  int b = 0, e = n - 1;
  while (b < e) {
    const int mid = b + (e - b) / 2;
    if (cdf[mid] <= u) b = mid + 1; else e = mid;
  }
  pdf = b == 0 ? cdf[0] : cdf[b] - cdf[b - 1];
  return b;
}

__device__ V3 merl_sample(const MerlDev &m, V3 wi, float u0, float u1, V3 &wo, float &pdf) {
  const bool flip = wi.z < 0.0f;
  if (flip) wi.z = -wi.z;
  const float *seg = m.seg + merl_incident_bin(wi) * kSegFloats;
  const float *cols = seg, *rows = seg + kSegTheta * kSegPhi, *gx = rows + kSegTheta, *gy = gx + kSegPhi;
  bool opposite = false;
  if (u0 > 0.5f) {
    opposite = true;
    u0 = (u0 - 0.5f) * 2.0f;
  } else {
    u0 *= 2.0f;
  }
  float rp, cp;
  const int ri = search_cdf_f(rows, kSegTheta, u1, rp);
  const float *cc = cols + ri * kSegPhi;
  const int ci = search_cdf_f(cc, kSegPhi, u0, cp);
  const float r0 = (u0 - (ci > 0 ? cc[ci - 1] : 0.0f)) / cp, r1 = (u1 - (ri > 0 ? rows[ri - 1] : 0.0f)) / rp;
  const float bx0 = gx[ci], by0 = gy[ri];
  const float bx1 = ci + 1 < kSegPhi ? gx[ci + 1] : 1.0f, by1 = ri + 1 < kSegTheta ? gy[ri + 1] : 1.0f;
  const float c1 = cosf(by0 * (0.5f * kPi)), c2 = cosf(by1 * (0.5f * kPi)), d_cos = c1 - c2;
  float phi = (bx0 + (bx1 - bx0) * r0) * kPi;
  if (opposite) phi = 2.0f * kPi - phi;
  phi += sph_phi(wi);
  const float ct = c1 - r1 * d_cos, st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
  wo = v3(st * cosf(phi), st * sinf(phi), ct);
  pdf = 0.5f * rp * cp / ((bx1 - bx0) * kPi * d_cos);
  const V3 f = merl_brdf(m, wi, wo);
  if (flip) wo.z = -wo.z;
  return f;
}

// ------------------------------------------------------------ layers --
// Non-specular component count of a layer, and of the whole BSDF.
__device__ __forceinline__ int layer_ncomp(const Layer &b) {
  switch (b.kind) {
    case kTransparent: return 0;
    case kPlastic: return 2;
    case kUber: return (black(b.kd) ? 0 : 1) + (black(b.ks) ? 0 : 1);
    default: return 1;
  }
}
// Specular component count (reflection + transmission).
__device__ __forceinline__ int layer_nspec(const Layer &b) {
  if (b.kind == kTransparent) return (black(b.kd) ? 0 : 1) + (black(b.ks) ? 0 : 1);
  if (b.kind == kUber) return (black(b.kr) ? 0 : 1) + (black(b.kt) ? 0 : 1);
  return 0;
}
// A material's BxDF set as one layer (scale 1).
__device__ Layer make_layer(const DevMaterial &m) {
  Layer l;
  l.kind = m.kind;
  l.kd = load3(m.kd);
  l.ks = load3(m.ks);
  l.kr = load3(m.kr);
  l.kt = load3(m.kt);
  l.exponent = m.exponent;
  l.on_a = m.on_a;
  l.on_b = m.on_b;
  l.ior = m.ior;
  l.pdiff = m.pdiff;
  l.ev = m.ev;
  l.eta = load3(m.eta);
  l.k2 = load3(m.k2);
  l.merl = m.merl;
  l.scale = v3(1.0f, 1.0f, 1.0f);
  return l;
}
// The second layer of a mix (nl == 2).
__device__ __forceinline__ Layer layer1(const Bsdf &b) {
  Layer l = make_layer(*b.m1);
  l.scale = b.s1;
  return l;
}
__device__ __forceinline__ int bsdf_ncomp(const Bsdf &b) {
  return layer_ncomp(b.L0) + (b.nl == 2 ? layer_ncomp(layer1(b)) : 0);
}
__device__ __forceinline__ int bsdf_nspec(const Bsdf &b) {
  return layer_nspec(b.L0) + (b.nl == 2 ? layer_nspec(layer1(b)) : 0);
}

// A layer's non-specular components summed (local frame, unscaled).
__device__ V3 layer_eval(const Layer &b, V3 wi, V3 wo) {
  switch (b.kind) {
    case kTransparent: return v3(0, 0, 0);
    case kMetal: return microfacet_eval(b, wi, wo);
    case kMeasured: return merl_eval(b.merl, wi, wo);
    case kSubstrate: return fb_eval(b, wi, wo);
    case kPlastic: return diffuse_eval(b, wi, wo) + microfacet_eval(b, wi, wo);
    case kUber: {
      V3 f = v3(0, 0, 0);
      if (!black(b.kd)) f = f + b.kd * kInvPi;
      if (!black(b.ks)) f = f + microfacet_eval(b, wi, wo);
      return f;
    }
    default: return diffuse_eval(b, wi, wo);
  }
}
// The sum of a layer's non-specular component densities.
__device__ float layer_pdf_sum(const Layer &b, V3 wi, V3 wo) {
  switch (b.kind) {
    case kTransparent: return 0.0f;
    case kMetal: return microfacet_pdf(b, wi, wo);
    case kMeasured: return merl_pdf(b.merl, wi, wo);
    case kSubstrate: return fb_pdf(b, wi, wo);
    case kPlastic: return diffuse_pdf(wi, wo) + microfacet_pdf(b, wi, wo);
    case kUber: {
      float p = 0.0f;
      if (!black(b.kd)) p += diffuse_pdf(wi, wo);
      if (!black(b.ks)) p += microfacet_pdf(b, wi, wo);
      return p;
    }
    default: return diffuse_pdf(wi, wo);
  }
}
// Samples non-specular component c of a layer: the exitant direction and
// that component's own density (0: the sample is rejected).
__device__ float layer_sample(const Layer &b, int c, V3 wi, float u0, float u1, V3 &wo) {
  bool glossy = false;
  switch (b.kind) {
    case kMeasured: {  // MERLMeasured::Sample (MERLMeasured.cpp:302-369)
      float pdf = 0.0f;
      merl_sample(b.merl, wi, u0, u1, wo, pdf);
      return pdf;
    }
    case kSubstrate:
      if (!fb_sample(b, wi, u0, u1, wo)) return 0.0f;
      return fb_pdf(b, wi, wo);
    case kMetal: glossy = true; break;
    case kPlastic: glossy = c == 1; break;
    case kUber: glossy = black(b.kd) || c == 1; break;
    default: break;
  }
  if (glossy) {
    if (!blinn_sample(b.exponent, wi, u0, u1, wo)) return 0.0f;
    return microfacet_pdf(b, wi, wo);
  }
  // BxDF::Sample (Core/BxDF.cpp:20-31): cosine hemisphere on the incident side
  wo = cosine_hemisphere(u0, u1);
  if (wi.z < 0.0f) wo.z = -wo.z;
  return diffuse_pdf(wi, wo);
}

// BSDF::Evaluate (Core/BSDF.cpp:22-40): every non-specular component is a
// reflection, so directions on opposite sides of the geometric normal give
// zero; the layers' components are summed, each layer scaled.
__device__ V3 bsdf_eval(const Bsdf &b, V3 wi_w, V3 wo_w) {
  if (!(dot(wi_w, b.ng) * dot(wo_w, b.ng) > 0.0f)) return v3(0, 0, 0);
  const V3 wi = b.local(wi_w), wo = b.local(wo_w);
  const V3 f = mul(b.L0.scale, layer_eval(b.L0, wi, wo));
  if (b.nl == 1) return f;
  const Layer l = layer1(b);
  return f + mul(l.scale, layer_eval(l, wi, wo));
}

// The derivative of bsdf_eval with respect to the per-triangle albedo kd of
// a single-layer matte, plastic or substrate surface (the diffuse term with
// kd = 1); zero for the others, whose reflectance the albedo does not set.
__device__ V3 bsdf_eval_dkd(const Bsdf &b, V3 wi_w, V3 wo_w) {
  const Layer &l = b.L0;
  const bool albedo = b.nl == 1 && (l.kind == kLambert || l.kind == kOrenNayar || l.kind == kPlastic ||
                                    l.kind == kSubstrate);
  if (!albedo || !(dot(wi_w, b.ng) * dot(wo_w, b.ng) > 0.0f)) return v3(0, 0, 0);
  const V3 wi = b.local(wi_w), wo = b.local(wo_w);
  if (l.kind == kSubstrate) {
    const float t1 = 1.0f - 0.5f * fabsf(wo.z), t2 = 1.0f - 0.5f * fabsf(wi.z);
    const float p1 = t1 * t1 * t1 * t1 * t1, p2 = t2 * t2 * t2 * t2 * t2;
    return (v3(1.0f, 1.0f, 1.0f) - l.ks) * ((28.0f / (23.0f * kPi)) * (1.0f - p1) * (1.0f - p2));
  }
  Layer u = l;
  u.kd = v3(1.0f, 1.0f, 1.0f);
  return diffuse_eval(u, wi, wo);
}

// BSDF::PDF (Core/BSDF.cpp:42-58): the average of the non-specular
// component densities.
__device__ float bsdf_pdf(const Bsdf &b, V3 wi_w, V3 wo_w) {
  const int n = bsdf_ncomp(b);
  if (n == 0) return 0.0f;
  const V3 wi = b.local(wi_w), wo = b.local(wo_w);
  float p = layer_pdf_sum(b.L0, wi, wo);
  if (b.nl == 2) p += layer_pdf_sum(layer1(b), wi, wo);
  return n == 1 ? p : p / n;
}

// BSDF::Sample (Core/BSDF.cpp:110-168) over the non-specular components:
// sample component comp (0 .. bsdf_ncomp - 1; the caller picks it
// uniformly), add the other components' densities at the sampled direction
// and average over n_all (the non-specular count for direct lighting;
// every component, specular ones included, when the caller samples
// BSDF_ALL), evaluate the whole BSDF.
__device__ V3 bsdf_sample_c(const Bsdf &b, int comp, V3 wi_w, float u0, float u1, V3 &wo_w, float &pdf, int n_all) {
  const int n = bsdf_ncomp(b);
  pdf = 0.0f;
  wo_w = wi_w;
  if (n == 0) return v3(0, 0, 0);
  const V3 wi = b.local(wi_w);
  V3 wo;
  float pc;
  int kind;
  MerlDev merl;
  const int n0 = layer_ncomp(b.L0);
  if (comp < n0 || b.nl == 1) {
    pc = layer_sample(b.L0, comp, wi, u0, u1, wo);
    kind = b.L0.kind;
    merl = b.L0.merl;
  } else {
    const Layer l = layer1(b);
    pc = layer_sample(l, comp - n0, wi, u0, u1, wo);
    kind = l.kind;
    merl = l.merl;
  }
  wo_w = b.world(wo);
  if (!(pc > 0.0f)) return v3(0, 0, 0);
  if (n == 1 && n_all == 1) {
    pdf = pc;
  } else {
    // the sampled component's own density, plus the others' at wo
    float p = layer_pdf_sum(b.L0, wi, wo) + (b.nl == 2 ? layer_pdf_sum(layer1(b), wi, wo) : 0.0f);
    if (kind == kMeasured) p += pc - merl_pdf(merl, wi, wo);  // MERL's sample density as it returned it
    pdf = p / n_all;
  }
  return bsdf_eval(b, wi_w, wo_w);
}
// The direct-lighting form: a non-specular component picked uniformly with uc.
__device__ __forceinline__ V3 bsdf_sample(const Bsdf &b, V3 wi_w, float uc, float u0, float u1, V3 &wo_w,
                                          float &pdf) {
  const int n = bsdf_ncomp(b);
  return bsdf_sample_c(b, min((int)(uc * n), max(n - 1, 0)), wi_w, u0, u1, wo_w, pdf, n);
}

// ------------------------------------------------------------------ shading --
struct Hit {
  V3 p, ng, ns;
  int g;      // global triangle
  int prim;   // primitive
  float b1, b2;  // barycentrics of vertices 1 and 2 (where the primitive interpolates vertex data)
};

// CoreUtils::GetNextMinT (CoreUtils.h:139-149) for a ray leaving the hit
// point p in direction w: max(0, m_dot / (w . m_cross) + 1e-14), with the
// Intersection's m_cross = (v1 - v0) x (v2 - v0) and m_dot = ((v0 - p) x
// (v1 - v0)) . (v2 - v0) = (v0 - p) . m_cross (TriangleAccelerator.cpp:
// 341-345): the ray's own crossing of the triangle's plane plus 1e-14.
//
// next_min_t_exact evaluates that in double with every operation rounded
// separately, as the reference does, for the float point p the ray actually
// starts from, rounded up to float.  On GB300 a double operation costs
// about 64 float ones, so the renders use next_min_t: the same quantity in
// float with a rigorous bound on its error, E; the returned tmin is an upper
// bound of the reference's value that exceeds it by at most 2E (a few float
// roundings of the hit point's distance to the plane, the precision of a
// float ray anyway), so the outgoing ray never re-hits its own triangle and
// skips no geometry farther than that from its plane.  Where the direction
// is nearly parallel to the plane (the bound on the denominator covers zero)
// the double evaluation decides.  World-space triangle: for a transformed
// primitive the reference evaluates the same quantity in mesh space (t is
// the same parameter in both spaces).
__device__ __noinline__ float next_min_t_exact(const SceneDev &S, const Hit &h, V3 w) {
  const int i0 = S.tri_vidx[3 * h.g], i1 = S.tri_vidx[3 * h.g + 1], i2 = S.tri_vidx[3 * h.g + 2];
  const double ax = S.vpos[3 * i0], ay = S.vpos[3 * i0 + 1], az = S.vpos[3 * i0 + 2];
  const double e1x = __dsub_rn(S.vpos[3 * i1], ax), e1y = __dsub_rn(S.vpos[3 * i1 + 1], ay),
               e1z = __dsub_rn(S.vpos[3 * i1 + 2], az);
  const double e2x = __dsub_rn(S.vpos[3 * i2], ax), e2y = __dsub_rn(S.vpos[3 * i2 + 1], ay),
               e2z = __dsub_rn(S.vpos[3 * i2 + 2], az);
  const double cx = __dsub_rn(__dmul_rn(e1y, e2z), __dmul_rn(e1z, e2y));
  const double cy = __dsub_rn(__dmul_rn(e1z, e2x), __dmul_rn(e1x, e2z));
  const double cz = __dsub_rn(__dmul_rn(e1x, e2y), __dmul_rn(e1y, e2x));
  const double qx = __dsub_rn(ax, (double)h.p.x), qy = __dsub_rn(ay, (double)h.p.y), qz = __dsub_rn(az, (double)h.p.z);
  const double sx = __dsub_rn(__dmul_rn(qy, e1z), __dmul_rn(qz, e1y));
  const double sy = __dsub_rn(__dmul_rn(qz, e1x), __dmul_rn(qx, e1z));
  const double sz = __dsub_rn(__dmul_rn(qx, e1y), __dmul_rn(qy, e1x));
  const double mdot = __dadd_rn(__dadd_rn(__dmul_rn(sx, e2x), __dmul_rn(sy, e2y)), __dmul_rn(sz, e2z));
  const double div = __dadd_rn(__dadd_rn(__dmul_rn((double)w.x, cx), __dmul_rn((double)w.y, cy)),
                               __dmul_rn((double)w.z, cz));
  if (div == 0.0) return 0.0f;
  const double t = fmax(0.0, __dadd_rn(__dmul_rn(mdot, __ddiv_rn(1.0, div)), 1e-14));
  return __double2float_ru(t);
}

// A primitive whose mesh is shared is traced in mesh space (the ray taken
// there by its world-to-mesh matrix in double), so its outgoing rays get
// GetNextMinT exactly as the reference computes it: in mesh space, for the
// ray's origin and direction transformed with the same double operations
// as the traversal uses, rounded up to float.
__device__ __noinline__ float next_min_t_instance(const SceneDev &S, const Hit &h, V3 w) {
  const double *m = S.prim_w2m + 16 * h.prim;
  auto row = [&](int r, double x, double y, double z) {
    return __dadd_rn(__dadd_rn(__dmul_rn(m[4 * r], x), __dmul_rn(m[4 * r + 1], y)), __dmul_rn(m[4 * r + 2], z));
  };
  double o[3] = {__dadd_rn(row(0, h.p.x, h.p.y, h.p.z), m[3]), __dadd_rn(row(1, h.p.x, h.p.y, h.p.z), m[7]),
                 __dadd_rn(row(2, h.p.x, h.p.y, h.p.z), m[11])};
  const double wq = __dadd_rn(row(3, h.p.x, h.p.y, h.p.z), m[15]);
  if (wq != 1.0) {
    const double inv = __ddiv_rn(1.0, wq);
    for (int k = 0; k < 3; ++k) o[k] = __dmul_rn(o[k], inv);
  }
  const double d[3] = {row(0, w.x, w.y, w.z), row(1, w.x, w.y, w.z), row(2, w.x, w.y, w.z)};
  const int i0 = S.tri_vidx[3 * h.g], i1 = S.tri_vidx[3 * h.g + 1], i2 = S.tri_vidx[3 * h.g + 2];
  const float *vm = S.vpos_mesh;
  const double ax = vm[3 * i0], ay = vm[3 * i0 + 1], az = vm[3 * i0 + 2];
  const double e1x = __dsub_rn(vm[3 * i1], ax), e1y = __dsub_rn(vm[3 * i1 + 1], ay), e1z = __dsub_rn(vm[3 * i1 + 2], az);
  const double e2x = __dsub_rn(vm[3 * i2], ax), e2y = __dsub_rn(vm[3 * i2 + 1], ay), e2z = __dsub_rn(vm[3 * i2 + 2], az);
  const double cx = __dsub_rn(__dmul_rn(e1y, e2z), __dmul_rn(e1z, e2y));
  const double cy = __dsub_rn(__dmul_rn(e1z, e2x), __dmul_rn(e1x, e2z));
  const double cz = __dsub_rn(__dmul_rn(e1x, e2y), __dmul_rn(e1y, e2x));
  const double qx = __dsub_rn(ax, o[0]), qy = __dsub_rn(ay, o[1]), qz = __dsub_rn(az, o[2]);
  const double sx = __dsub_rn(__dmul_rn(qy, e1z), __dmul_rn(qz, e1y));
  const double sy = __dsub_rn(__dmul_rn(qz, e1x), __dmul_rn(qx, e1z));
  const double sz = __dsub_rn(__dmul_rn(qx, e1y), __dmul_rn(qy, e1x));
  const double mdot = __dadd_rn(__dadd_rn(__dmul_rn(sx, e2x), __dmul_rn(sy, e2y)), __dmul_rn(sz, e2z));
  const double div = __dadd_rn(__dadd_rn(__dmul_rn(d[0], cx), __dmul_rn(d[1], cy)), __dmul_rn(d[2], cz));
  if (div == 0.0) return 0.0f;
  return __double2float_ru(fmax(0.0, __dadd_rn(__dmul_rn(mdot, __ddiv_rn(1.0, div)), 1e-14)));
}

__device__ __forceinline__ float next_min_t(const SceneDev &S, const Hit &h, V3 w) {
  if (S.prim_inst && S.prim_inst[h.prim]) return next_min_t_instance(S, h, w);
  const int i0 = S.tri_vidx[3 * h.g], i1 = S.tri_vidx[3 * h.g + 1], i2 = S.tri_vidx[3 * h.g + 2];
  const V3 p0 = load3(S.vpos + 3 * i0), p1 = load3(S.vpos + 3 * i1), p2 = load3(S.vpos + 3 * i2);
  const V3 e1 = p1 - p0, e2 = p2 - p0, n = cross(e1, e2), q = p0 - h.p;
  // componentwise magnitude of the cross product, bounding its terms
  const V3 a1 = v3(fabsf(e1.x), fabsf(e1.y), fabsf(e1.z)), a2 = v3(fabsf(e2.x), fabsf(e2.y), fabsf(e2.z));
  const V3 A = v3(a1.y * a2.z + a1.z * a2.y, a1.z * a2.x + a1.x * a2.z, a1.x * a2.y + a1.y * a2.x);
  const float num = dot(q, n), den = dot(w, n);
  // u = 2^-24: the edges carry <= u relative error, the cross product
  // <= 4u A, q <= u |q|; the dot products add 3u of their magnitude sums
  const float u = 5.9604645e-8f;
  const float en = 9.0f * u * (fabsf(q.x) * A.x + fabsf(q.y) * A.y + fabsf(q.z) * A.z) + 1e-35f;
  const float ed = 8.0f * u * (fabsf(w.x) * A.x + fabsf(w.y) * A.y + fabsf(w.z) * A.z) + 1e-35f;
  const float ad = fabsf(den);
  if (!(ad > 4.0f * ed)) return next_min_t_exact(S, h, w);
  const float t = num / den;
  const float et = 1.01f * (en + fabsf(t) * ed) / (ad - ed) + 4.0f * u * fabsf(t);
  return fmaxf(0.0f, __fadd_ru(__fadd_ru(t, et), 1e-14f));
}

// MathRoutines::CoordinateSystem (Math/MathRoutines.h:298-313): the first
// tangent of the frame it builds around a unit vector.
__device__ __forceinline__ V3 coordinate_tangent(V3 n) {
  if (fabsf(n.x) > fabsf(n.y)) {
    const float il = 1.0f / sqrtf(n.x * n.x + n.z * n.z);
    return v3(-n.z * il, 0.0f, n.x * il);
  }
  const float il = 1.0f / sqrtf(n.y * n.y + n.z * n.z);
  return v3(0.0f, n.z * il, -n.y * il);
}

// The differential geometry's tangent (TriangleMesh::
// ComputeDifferentialGeometry, TriangleMesh.cpp:490-528): interpolated
// vertex tangents; else the direction of increasing u from the triangle's
// uvs; else (no uvs, or degenerate ones) CoordinateSystem of the shading
// normal; then made perpendicular to the shading normal, (n x t) x n.
__device__ V3 shading_tangent(const SceneDev &S, const Hit &h) {
  const V3 n = h.ns;
  const int mode = S.prim_frame ? S.prim_frame[h.prim] : 0;
  V3 t;
  if (mode == 1) {
    const int i0 = S.tri_vidx[3 * h.g], i1 = S.tri_vidx[3 * h.g + 1], i2 = S.tri_vidx[3 * h.g + 2];
    t = load3(S.vtan + 3 * i0) * (1.0f - h.b1 - h.b2) + load3(S.vtan + 3 * i1) * h.b1 +
        load3(S.vtan + 3 * i2) * h.b2;
  } else if (mode == 2) {
    const float *uv = S.tri_uv + 6 * h.g;
    const float du1 = uv[0] - uv[4], du2 = uv[2] - uv[4], dv1 = uv[1] - uv[5], dv2 = uv[3] - uv[5];
    const float det = du1 * dv2 - dv1 * du2;
    if (fabsf(det) < 1e-12f) {
      t = coordinate_tangent(n);
    } else {
      const int i0 = S.tri_vidx[3 * h.g], i1 = S.tri_vidx[3 * h.g + 1], i2 = S.tri_vidx[3 * h.g + 2];
      const V3 p0 = load3(S.vpos + 3 * i0), p1 = load3(S.vpos + 3 * i1), p2 = load3(S.vpos + 3 * i2);
      t = ((p0 - p2) * dv2 - (p1 - p2) * dv1) * (1.0f / det);
    }
  } else {
    t = coordinate_tangent(n);
  }
  const V3 t2 = cross(n, t);
  if (dot(t2, t2) > 1e-20f) return normalized(cross(t2, n));
  return coordinate_tangent(n);
}

// The material's BSDF at a hit (Material::GetBSDF).  MixMaterial
// (Materials/MixMaterial.cpp:29-57): the first material's components scaled
// by the mix's scale s and the second's by 1 - s, a side whose scale is
// black left out.  A per-triangle albedo replaces the diffuse reflectance
// of a single-layer surface other than transparent and uber ones.
__device__ Bsdf make_bsdf(const SceneDev &S, const Hit &h, int prim) {
  const DevMaterial &m = S.materials[S.prim_material[prim]];
  Bsdf b;
  b.ng = h.ng;
  b.n = h.ns;
  b.e1 = shading_tangent(S, h);
  b.e2 = cross(b.n, b.e1);  // BSDF::BSDF (Core/BSDF.h:182-192): e2 = n x tangent
  b.m1 = nullptr;
  b.s1 = v3(0, 0, 0);
  if (m.kind == kMix) {
    const V3 s0 = load3(m.mix_scale), s1 = v3(1.0f - s0.x, 1.0f - s0.y, 1.0f - s0.z);
    const bool has0 = !black(s0), has1 = !black(s1) && m.mix[1] >= 0;
    b.nl = has0 && has1 ? 2 : 1;
    if (has0) {
      b.L0 = make_layer(S.materials[m.mix[0]]);
      b.L0.scale = s0;
      if (has1) {
        b.m1 = S.materials + m.mix[1];
        b.s1 = s1;
      }
    } else if (has1) {
      b.L0 = make_layer(S.materials[m.mix[1]]);
      b.L0.scale = s1;
    } else {  // nothing scatters
      b.L0 = make_layer(m);
      b.L0.kind = kTransparent;
      b.L0.kd = b.L0.ks = v3(0, 0, 0);
    }
    return b;
  }
  b.nl = 1;
  b.L0 = make_layer(m);
  if (S.tri_albedo && m.kind != kTransparent && m.kind != kUber) {
    const float *ta = S.tri_albedo + 3 * (int64_t)h.g;
    if (ta[0] == ta[0]) b.L0.kd = v3(fminf(1.0f, fmaxf(0.0f, ta[0])), fminf(1.0f, fmaxf(0.0f, ta[1])),
                                     fminf(1.0f, fmaxf(0.0f, ta[2])));
  }
  return b;
}

// --------------------------------------------------------------- specular --
// The specular reflection and transmission weights of a layer
// (TransparentMaterial: kd, ks; UberMaterial: kr, 1 - opacity).
__device__ __forceinline__ V3 layer_spec_r(const Layer &l) {
  return l.kind == kTransparent ? l.kd : (l.kind == kUber ? l.kr : v3(0, 0, 0));
}
__device__ __forceinline__ V3 layer_spec_t(const Layer &l) {
  return l.kind == kTransparent ? l.ks : (l.kind == kUber ? l.kt : v3(0, 0, 0));
}

// LTEIntegrator::_SpecularReflect (Core/LTEIntegrator.cpp:66-92) with
// SpecularReflection<FresnelDielectric>::Sample (BxDFs/SpecularReflection.h):
// the mirror direction of wo (towards the viewer) about the shading normal
// and its weight scale * r * F(cos) -- no cosine and no density, the BxDF
// accounts for both.  False when the BSDF has no reflection component, the
// weight is black or the direction grazes the shading plane.  (A BSDF has
// at most one specular reflection: the host refuses mixes of two.)
__device__ __forceinline__ bool specular_reflect(const Bsdf &b, V3 wo_w, V3 &dir, V3 &val) {
  for (int i = 0; i < b.nl; ++i) {
    const Layer l = i == 0 ? b.L0 : layer1(b);
    const V3 r = layer_spec_r(l);
    if (black(r)) continue;
    const V3 wi = b.local(wo_w);
    dir = b.world(v3(-wi.x, -wi.y, wi.z));
    val = mul(l.scale, r) * fresnel_dielectric_ior(wi.z, l.ior);
    return !black(val) && fabsf(dot(dir, b.n)) > kEps;
  }
  return false;
}

// LTEIntegrator::_SpecularTransmit (LTEIntegrator.cpp:94-126) with
// SpecularTransmission::Sample (BxDFs/SpecularTransmission.cpp:33-66): the
// refracted direction (Snell's law, the indices swapped when wo is inside),
// its weight scale * t * (1 - F(cos)) * eta^2 (eta = 1/ior entering, ior
// leaving); false on total internal reflection (black weight), at
// normal-grazing incidence, or when the BSDF has no transmission component.
__device__ __forceinline__ bool specular_transmit(const Bsdf &b, V3 wo_w, V3 &dir, V3 &val) {
  for (int i = 0; i < b.nl; ++i) {
    const Layer l = i == 0 ? b.L0 : layer1(b);
    const V3 t = layer_spec_t(l);
    if (black(t)) continue;
    const float cn = dot(wo_w, b.n);
    if (fabsf(cn) < kEps) return false;
    const V3 wi = b.local(wo_w);
    float zs = -1.0f, ni = l.ior, no = 1.0f;
    if (wi.z < 0.0f) {
      zs = 1.0f;
      ni = 1.0f;
      no = l.ior;
    }
    const float eta = no / ni;
    const float st2 = eta * eta * (1.0f - wi.z * wi.z);
    if (st2 >= 1.0f) return false;
    const float ct = sqrtf(1.0f - st2);
    dir = b.world(v3(-wi.x * eta, -wi.y * eta, ct * zs));
    const float e = cn > 0.0f ? 1.0f / l.ior : l.ior;
    val = mul(l.scale, t) * ((1.0f - fresnel_dielectric_ior(wi.z, l.ior)) * (e * e));
    return !black(val) && fabsf(dot(dir, b.n)) > kEps;
  }
  return false;
}

__device__ Hit make_hit(const SceneDev &S, V3 o, V3 d, float t, int prim, int tri) {
  Hit h;
  h.prim = prim;
  h.g = S.prim_tri_offset[prim] + tri;
  const int i0 = S.tri_vidx[3 * h.g], i1 = S.tri_vidx[3 * h.g + 1], i2 = S.tri_vidx[3 * h.g + 2];
  const V3 p0 = load3(S.vpos + 3 * i0), p1 = load3(S.vpos + 3 * i1), p2 = load3(S.vpos + 3 * i2);
  h.p = o + d * t;
  h.ng = normalized(cross(p1 - p0, p2 - p0));
  h.ns = h.ng;
  h.b1 = h.b2 = 0.0f;
  const bool normals = S.prim_has_normals[prim] != 0;
  if (normals || (S.prim_frame && S.prim_frame[prim] == 1)) {
    // barycentrics of the hit point (Moller-Trumbore)
    const V3 e1 = p1 - p0, e2 = p2 - p0, s1 = cross(d, e2);
    const float inv = 1.0f / dot(s1, e1);
    const V3 dd = o - p0;
    h.b1 = dot(dd, s1) * inv;
    h.b2 = dot(d, cross(dd, e1)) * inv;
  }
  if (normals) {
    // the interpolated vertex normal (TriangleMesh.cpp:478-484)
    const float b0 = 1.0f - h.b1 - h.b2;
    const V3 n = load3(S.vnrm + 3 * i0) * b0 + load3(S.vnrm + 3 * i1) * h.b1 + load3(S.vnrm + 3 * i2) * h.b2;
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

}  // namespace
}  // namespace skw

namespace skw {
namespace {

// ------------------------------------------------------------ light choice --
// MathRoutines::_SubtendedSolidAngle / SubtendedSolidAngle (Math/
// MathRoutines.h:321-391): the box's faces that face the point, as two
// triangles each (Oosterom-Strackee).
__device__ __forceinline__ float tri_solid_angle(V3 a, V3 b, V3 c) {
  const float det = dot(a, cross(b, c));
  const float den = 1.0f + dot(a, b) + dot(a, c) + dot(b, c);
  if (den > 0.0f) return fabsf(atanf(det / den) * 2.0f);
  if (den < 0.0f) return 2.0f * (kPi - fabsf(atanf(det / den)));
  return 2.0f * kPi;
}

__device__ float box_solid_angle(V3 p, const float lo[3], const float hi[3]) {
  V3 d[8];
  for (int i = 0; i < 8; ++i)
    d[i] = normalized(v3((i & 1) ? hi[0] : lo[0], (i & 2) ? hi[1] : lo[1], (i & 4) ? hi[2] : lo[2]) - p);
  bool inside = true;
  float sum = 0.0f;
  if (p.x < lo[0]) {
    sum += tri_solid_angle(d[0], d[2], d[6]) + tri_solid_angle(d[0], d[4], d[6]);
    inside = false;
  } else if (p.x > hi[0]) {
    sum += tri_solid_angle(d[1], d[3], d[7]) + tri_solid_angle(d[1], d[5], d[7]);
    inside = false;
  }
  if (p.y < lo[1]) {
    sum += tri_solid_angle(d[0], d[1], d[5]) + tri_solid_angle(d[0], d[4], d[5]);
    inside = false;
  } else if (p.y > hi[1]) {
    sum += tri_solid_angle(d[2], d[3], d[7]) + tri_solid_angle(d[2], d[6], d[7]);
    inside = false;
  }
  if (p.z < lo[2]) {
    sum += tri_solid_angle(d[0], d[1], d[3]) + tri_solid_angle(d[0], d[2], d[3]);
    inside = false;
  } else if (p.z > hi[2]) {
    sum += tri_solid_angle(d[4], d[5], d[7]) + tri_solid_angle(d[4], d[6], d[7]);
    inside = false;
  }
  return inside ? 4.0f * kPi : sum;
}

// IrradianceLightsSamplingStrategy::GetLightsCDF(point, normal) (:57-113)
// weight of area light `li`: solid angle of its bounds times its intensity
// times the average (clamped) cosine of the bounds' corners, pi * intensity
// inside the bounds.
__device__ float light_weight(const AreaLight &L, V3 p, V3 n) {
  if (p.x >= L.lo[0] && p.y >= L.lo[1] && p.z >= L.lo[2] && p.x <= L.hi[0] && p.y <= L.hi[1] && p.z <= L.hi[2])
    return kPi * L.intensity;
  float avg = 0.0f;
  for (int j = 0; j < 8; ++j) {
    const V3 v = v3((j & 1) ? L.lo[0] : L.hi[0], (j & 2) ? L.lo[1] : L.hi[1], (j & 4) ? L.lo[2] : L.hi[2]);
    avg += fmaxf(0.0f, dot(normalized(v - p), n));
  }
  avg *= 0.125f;
  if (!(avg > 0.0f)) return 0.0f;
  if (avg < 0.1f) avg = 0.1f;
  return box_solid_angle(p, L.lo, L.hi) * L.intensity * avg;
}

// Probability of choosing light `li` at (p, n) among all area lights
// (_Weights_To_CDF: equal probabilities when every weight is 0).
__device__ float light_choice_pdf(const SceneDev &S, int li, V3 p, V3 n) {
  const int nl = S.n_area_lights;
  if (nl <= 1) return 1.0f;
  float tot = 0.0f, mine = 0.0f;
  for (int i = 0; i < nl; ++i) {
    const float w = light_weight(S.area_lights[i], p, n);
    tot += w;
    if (i == li) mine = w;
  }
  return tot > 0.0f ? mine / tot : 1.0f / nl;
}

// Chooses a light with u (BinarySearchCDF over the normalised cumulative
// weights); returns its index, its probability and the remainder of u
// rescaled to [0, 1) for the triangle choice.
__device__ int choose_light(const SceneDev &S, float u, V3 p, V3 n, float &pdf, float &u_rest) {
  const int nl = S.n_area_lights;
  if (nl <= 1) {
    pdf = 1.0f;
    u_rest = u;
    return 0;
  }
  float tot = 0.0f;
  for (int i = 0; i < nl; ++i) tot += light_weight(S.area_lights[i], p, n);
  const bool uniform = !(tot > 0.0f);
  float cum = 0.0f, prev = 0.0f;
  int li = -1, last = 0;
  float last_w = 0.0f, last_prev = 0.0f;
  pdf = 0.0f;
  for (int i = 0; i < nl; ++i) {
    const float w = uniform ? 1.0f / nl : light_weight(S.area_lights[i], p, n) / tot;
    const float c0 = cum;
    cum += w;
    if (w > 0.0f) {
      last = i;
      last_w = w;
      last_prev = c0;
      if (u < cum) {
        li = i;
        pdf = w;
        prev = c0;
        break;
      }
    }
  }
  if (li < 0) {  // u beyond the float sum of the weights: the last light that can be chosen
    li = last;
    pdf = last_w;
    prev = last_prev;
  }
  u_rest = pdf > 0.0f ? fminf(fmaxf((u - prev) / pdf, 0.0f), 0.99999994f) : 0.0f;
  return li;
}

// BBox3D::Intersect (Math/BBox3D.h:150-171) of the ray segment [t0, t1] with
// the medium's box; false if they miss.
__device__ __forceinline__ bool medium_segment(const MediumDev &M, V3 o, V3 d, float &t0, float &t1) {
  const float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
  for (int i = 0; i < 3; ++i) {
    const float inv = 1.0f / dd[i];
    float tn = (M.lo[i] - oo[i]) * inv, tf = (M.hi[i] - oo[i]) * inv;
    if (tn > tf) {
      const float x = tn;
      tn = tf;
      tf = x;
    }
    t0 = tn > t0 ? tn : t0;
    t1 = tf < t1 ? tf : t1;
    if (t0 > t1) return false;
  }
  return true;
}

// _MediaTransmittance of a ray segment: exp(-OpticalThickness), the
// homogeneous region's optical thickness being sigma_t * |box segment|
// (HomogeneousVolumeRegion.cpp:63-73).
__device__ __forceinline__ V3 medium_tr(const MediumDev &M, V3 o, V3 d, float tmin, float tmax) {
  if (!M.on) return v3(1.0f, 1.0f, 1.0f);
  float t0 = tmin, t1 = tmax;
  if (!medium_segment(M, o, d, t0, t1)) return v3(1.0f, 1.0f, 1.0f);
  const float l = fabsf(t1 - t0);
  return v3(expf(-M.sigma_t[0] * l), expf(-M.sigma_t[1] * l), expf(-M.sigma_t[2] * l));
}

}  // namespace
}  // namespace skw
