// Photon mapping on sm_103a: photon shooting as a wavefront over paths,
// deterministic compaction of the deposits, and the irradiance estimate of
// the irradiance photons.
//
// Restates PhotonsShootingFilter::operator()
// (LTEIntegrators/PhotonLTEIntegrator/PhotonShootingPipeline.cpp:110-267):
//
//   k_photon_emit    path i: the light chosen by the power CDF with the
//                    radical inverse of i+1 in base 11, PointLight::SamplePhoton
//                    (LightSources/PointLight.cpp:44-55) or
//                    DiffuseAreaLightSource::SamplePhoton
//                    (LightSources/DiffuseAreaLightSource.cpp:118-150) with
//                    radical inverses in bases 2, 3, 5, 7 and 13, in double
//   k_trace          closest hit of every live path (traverse.cu)
//   k_photon_bounce  deposit at the hit (the first hit into the direct map,
//                    a later hit of a path that has only scattered
//                    specularly so far into the caustic map, other later
//                    hits into the indirect map; no direct or caustic
//                    deposit on a purely specular surface), BSDF sample
//                    (radical inverses in bases 17, 19, 23 at the first hit,
//                    the counter-based generator after it; between two
//                    specular components by their luminance), Russian
//                    roulette with the luminance ratio, next ray
//   k_scan_* / k_gather_photons  per-path deposits -> maps in path order
//
// The deposits of path i land in fixed staging slots (i, bounce), so the maps
// come out in the order of a single-threaded run of the reference: paths in
// order, each path's photons in bounce order.
#include <cuda_runtime.h>
#include <cstdint>

#include "kernels.h"
#include "photon_types.h"
#include "render_device.cuh"
#include "render_scene.h"

namespace skw {
namespace {

// SamplingRoutines::RadicalInverse (Math/SamplingRoutines.h:492-507).
__device__ double radical_inverse(unsigned n, unsigned base) {
  double ret = 0.0;
  const double inv_base = 1.0 / base;
  double inv = inv_base;
  while (n > 0) {
    const unsigned d = n % base;
    ret = __dadd_rn(ret, __dmul_rn((double)d, inv));
    n /= base;
    inv = __dmul_rn(inv, inv_base);
  }
  return ret;
}

// CompressedDirection(Vector3D_d) (Math/CompressedDirection.h:91-110).
__device__ uint16_t compress_dir(double x, double y, double z) {
  unsigned data = 0;
  if (x < 0) {
    data |= 1u << 13;
    x = -x;
  }
  if (y < 0) {
    data |= 1u << 14;
    y = -y;
  }
  if (z < 0) {
    data |= 1u << 15;
    z = -z;
  }
  const double scale = 126.999 / (x + y + z);
  unsigned qx = (unsigned)(uint8_t)(x * scale), qy = (unsigned)(uint8_t)(y * scale);
  if (qy >= 64) {
    qx = (127u - qx) & 0xFFu;
    qy = (127u - qy) & 0xFFu;
  }
  data |= (qx << 6) | qy;
  return (uint16_t)data;
}

__device__ __forceinline__ float luminance(V3 c) {
  return 0.05316285f * c.x + 0.58515348f * c.y + 0.36168367f * c.z;
}

struct Queue {
  float4 *rays;  // 2 per path
  float *w;      // 3 per path
  int *path;     // path index within the chunk | kDiffusePath once a bounce was not specular
  int *count;
};

constexpr int kDiffusePath = 1 << 30;

// The path's random numbers at bounce >= 1: 4 per bounce; bounces 0-15 use
// numbers 0-63 of the path's counter-based stream, later blocks of 16
// bounces re-seeded streams (a path's stream holds 64 numbers).
__device__ __forceinline__ float bounce_rnd(uint64_t seed, uint64_t path, int bounce, int k) {
  const uint64_t s = bounce < 16 ? seed : seed ^ (0xD6E8FEB86659FD93ull * (uint64_t)(bounce >> 4));
  return rnd(s, path, (uint32_t)(4 * (bounce & 15) + k));
}

// The specular components of a BSDF as the photon pipeline samples them
// (SpecularReflection / SpecularTransmission::Sample): the mirror
// direction with scale r F, and the refracted direction with scale t (1 - F)
// (black on total internal reflection, with the mirror direction).  The
// host admits at most one layer with specular components.
__device__ bool specular_parts(const Bsdf &b, V3 inc_w, V3 &dr, V3 &fr, V3 &dt, V3 &ft) {
  for (int i = 0; i < b.nl; ++i) {
    const Layer l = i == 0 ? b.L0 : layer1(b);
    const V3 r = layer_spec_r(l), t = layer_spec_t(l);
    if (black(r) && black(t)) continue;
    const V3 wi = b.local(inc_w);
    const float F = fresnel_dielectric_ior(wi.z, l.ior);
    dr = b.world(v3(-wi.x, -wi.y, wi.z));
    fr = mul(l.scale, r) * F;
    dt = dr;
    ft = v3(0, 0, 0);
    float zs = -1.0f, ni = l.ior, no = 1.0f;
    if (wi.z < 0.0f) {
      zs = 1.0f;
      ni = 1.0f;
      no = l.ior;
    }
    const float eta = no / ni;
    const float st2 = eta * eta * (1.0f - wi.z * wi.z);
    if (st2 < 1.0f) {
      dt = b.world(v3(-wi.x * eta, -wi.y * eta, sqrtf(1.0f - st2) * zs));
      if (!black(t)) ft = mul(l.scale, t) * (1.0f - F);
    }
    if (black(r)) fr = v3(0, 0, 0);
    return true;
  }
  return false;
}

// BSDF::Sample over all components of a specular-only BSDF (Core/BSDF.cpp:
// 72-117, _SampleSpecularOnly): each component's Sample, then one of them
// chosen with probability proportional to its luminance (the 0.999 guard as
// in the reference); pdf = that probability.  A single component is sampled
// with pdf 1.
__device__ V3 specular_sample_photon(const Bsdf &b, V3 inc_w, float uc, V3 &dir, float &pdf) {
  V3 dr, fr, dt, ft;
  pdf = 0.0f;
  dir = inc_w;
  if (!specular_parts(b, inc_w, dr, fr, dt, ft)) return v3(0, 0, 0);
  const bool has_r = !black(layer_spec_r(b.L0)) || (b.nl == 2 && !black(layer_spec_r(layer1(b))));
  const bool has_t = !black(layer_spec_t(b.L0)) || (b.nl == 2 && !black(layer_spec_t(layer1(b))));
  pdf = 1.0f;
  if (has_r && has_t) {
    const float lr = 0.05316285f * fr.x + 0.58515348f * fr.y + 0.36168367f * fr.z;
    const float lt = 0.05316285f * ft.x + 0.58515348f * ft.y + 0.36168367f * ft.z;
    const float sum = lr + lt;
    float c = uc * sum;
    if (c * 0.999f < lr) {
      pdf = lr / sum;
      dir = dr;
      return fr;
    }
    c -= lr;
    if (c * 0.999f < lt) {
      pdf = lt / sum;
      dir = dt;
      return ft;
    }
    pdf = 0.0f;
    dir = dr;
    return v3(0, 0, 0);
  }
  if (has_r) {
    dir = dr;
    return fr;
  }
  if (has_t) {
    dir = dt;
    return ft;
  }
  pdf = 0.0f;
  dir = dr;
  return v3(0, 0, 0);
}

// BSDF::Sample over every component of a BSDF with both kinds (Core/
// BSDF.cpp:119-168): one component chosen uniformly among all; a specular
// one gives its direction and value with pdf 1 / count (`specular` set), a
// non-specular one its direction, the whole BSDF's value there and the sum
// of the non-specular densities over the count.
__device__ V3 bsdf_sample_all(const Bsdf &b, V3 inc_w, float uc, float u0, float u1, V3 &dir, float &pdf,
                              bool &specular) {
  const int nn = bsdf_ncomp(b), ns = bsdf_nspec(b), n = nn + ns;
  specular = false;
  if (ns == 0) return bsdf_sample(b, inc_w, uc, u0, u1, dir, pdf);
  if (nn == 0) {
    specular = true;
    return specular_sample_photon(b, inc_w, uc, dir, pdf);
  }
  const int c = min((int)(uc * n), n - 1);
  if (c < nn) return bsdf_sample_c(b, c, inc_w, u0, u1, dir, pdf, n);
  specular = true;
  V3 dr, fr, dt, ft;
  specular_parts(b, inc_w, dr, fr, dt, ft);
  const bool has_r = !black(layer_spec_r(b.L0)) || (b.nl == 2 && !black(layer_spec_r(layer1(b))));
  const bool refl = has_r && c == nn;  // the reflection comes first when both are present
  dir = refl ? dr : dt;
  pdf = 1.0f / n;
  return refl ? fr : ft;
}

__device__ __forceinline__ void queue_push(const Queue &Q, int q, V3 o, V3 d, float tmin, V3 w, int path) {
  Q.rays[2 * q] = make_float4(o.x, o.y, o.z, d.x);
  Q.rays[2 * q + 1] = make_float4(d.y, d.z, tmin, __int_as_float(0x7f800000));
  Q.w[3 * q] = w.x;
  Q.w[3 * q + 1] = w.y;
  Q.w[3 * q + 2] = w.z;
  Q.path[q] = path;
}

__global__ void k_photon_emit(SceneDev S, PhotonShootArgs A, int64_t path0, int n, Queue out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool ok = false;
  V3 o = v3(0, 0, 0), d = v3(0, 0, 0), w = v3(0, 0, 0);
  float tmin = 0.0f;
  if (i < n) {
    const unsigned pi = (unsigned)(path0 + i) + 1u;
    const double ps0 = radical_inverse(pi, 2), ps1 = radical_inverse(pi, 3);
    const double ds0 = radical_inverse(pi, 5), ds1 = radical_inverse(pi, 7);
    // MathRoutines::BinarySearchCDF (Math/MathRoutines.h:191-218)
    const double u = radical_inverse(pi, 11);
    int lo = 0, hi = A.n_lights - 1;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (A.lights[mid].cdf <= u) lo = mid + 1; else hi = mid;
    }
    const double light_pdf = lo == 0 ? A.lights[0].cdf : A.lights[lo].cdf - A.lights[lo - 1].cdf;
    const PhotonLight L = A.lights[lo];
    double pdf = 0.0, wx = 0, wy = 0, wz = 0, ox = 0, oy = 0, oz = 0, dx = 0, dy = 0, dz = 0;
    if (L.kind == 0) {
      // UniformSphereSampling (SamplingRoutines.h:265-275), pdf 1 / (4 pi)
      const PointLightDev P = S.point_lights[L.index];
      const double z = 1.0 - 2.0 * ds0, r = sqrt(fmax(0.0, 1.0 - z * z)), phi = 2.0 * 3.14159265358979323846 * ds1;
      dx = r * cos(phi);
      dy = r * sin(phi);
      dz = z;
      ox = P.position[0];
      oy = P.position[1];
      oz = P.position[2];
      pdf = 1.0 / (4.0 * 3.14159265358979323846);
      wx = P.intensity[0];
      wy = P.intensity[1];
      wz = P.intensity[2];
    } else {
      const AreaLight AL = S.area_lights[L.index];
      const double ts = radical_inverse(pi, 13);
      int a = 0, b = AL.tri_count - 1;
      while (a < b) {
        const int mid = (a + b) >> 1;
        if ((double)S.light_cdf[AL.tri_begin + mid] <= ts) a = mid + 1; else b = mid;
      }
      const int g = S.light_tri[AL.tri_begin + a];
      const int j0 = S.tri_vidx[3 * g], j1 = S.tri_vidx[3 * g + 1], j2 = S.tri_vidx[3 * g + 2];
      const float *q0 = S.vpos + 3 * j0, *q1 = S.vpos + 3 * j1, *q2 = S.vpos + 3 * j2;
      // triangle normal (TriangleMesh::GetTriangleNormal, float)
      const V3 fn = normalized(cross(load3(q1) - load3(q0), load3(q2) - load3(q0)));
      const double nx = fn.x, ny = fn.y, nz = fn.z;
      const double sq = sqrt(ps0), b1 = 1.0 - sq, b2 = ps1 * sq;
      ox = b1 * q0[0] + b2 * q1[0] + (1.0 - b1 - b2) * q2[0];
      oy = b1 * q0[1] + b2 * q1[1] + (1.0 - b1 - b2) * q2[1];
      oz = b1 * q0[2] + b2 * q1[2] + (1.0 - b1 - b2) * q2[2];
      // MathRoutines::CoordinateSystem (Math/MathRoutines.h:298-312)
      double e2x, e2y, e2z;
      if (fabs(nx) > fabs(ny)) {
        const double il = 1.0 / sqrt(nx * nx + nz * nz);
        e2x = -nz * il;
        e2y = 0.0;
        e2z = nx * il;
      } else {
        const double il = 1.0 / sqrt(ny * ny + nz * nz);
        e2x = 0.0;
        e2y = nz * il;
        e2z = -ny * il;
      }
      const double e3x = ny * e2z - nz * e2y, e3y = nz * e2x - nx * e2z, e3z = nx * e2y - ny * e2x;
      const V3 l = cosine_hemisphere((float)ds0, (float)ds1);
      dx = l.x * e2x + l.y * e3x + l.z * nx;
      dy = l.x * e2y + l.y * e3y + l.z * ny;
      dz = l.x * e2z + l.y * e3z + l.z * nz;
      const double il = 1.0 / sqrt(dx * dx + dy * dy + dz * dz);
      dx *= il;
      dy *= il;
      dz *= il;
      pdf = (double)l.z * 0.31830988618379067154 / AL.area;
      const double c = dx * nx + dy * ny + dz * nz;
      wx = AL.radiance[0] * S.emission_scale * c;
      wy = AL.radiance[1] * S.emission_scale * c;
      wz = AL.radiance[2] * S.emission_scale * c;
      tmin = 1e-4f;
    }
    if (pdf > 0.0 && (wx > 0.0 || wy > 0.0 || wz > 0.0)) {
      const double inv = 1.0 / (pdf * light_pdf);
      w = v3((float)(wx * inv), (float)(wy * inv), (float)(wz * inv));
      o = v3((float)ox, (float)oy, (float)oz);
      d = v3((float)dx, (float)dy, (float)dz);
      ok = true;
    }
  }
  const int q = queue_append(ok, out.count);
  if (ok) queue_push(out, q, o, d, tmin, w, i);
}

// One bounce of every live path.  Deposits go to staging slot (path, bounce):
// the direct map holds bounce 0, the indirect map bounces 1 .. B-1.
__global__ void __launch_bounds__(128) k_photon_bounce(SceneDev S, PhotonShootArgs A, int64_t path0, int bounce,
                                                       int n_cap, Queue in, const int4 *__restrict__ hits, Queue out,
                                                       PhotonRec *__restrict__ st_direct,
                                                       uint8_t *__restrict__ has_direct,
                                                       PhotonRec *__restrict__ st_indirect,
                                                       int *__restrict__ n_indirect,
                                                       PhotonRec *__restrict__ st_caustic,
                                                       uint8_t *__restrict__ has_caustic) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int n = min(n_cap, *in.count);
  bool cont = false;
  V3 o = v3(0, 0, 0), dnew = v3(0, 0, 0), wnew = v3(0, 0, 0);
  float tmin = 0.0f;
  int path = 0, diffuse_path = 0;
  if (i < n) {
    const int4 hit = hits[i];
    path = in.path[i] & ~kDiffusePath;
    diffuse_path = in.path[i] & kDiffusePath;
    if (hit.y >= 0) {
      const float4 ra = in.rays[2 * i], rb = in.rays[2 * i + 1];
      const V3 ro = v3(ra.x, ra.y, ra.z), d = v3(ra.w, rb.x, rb.y);
      const Hit h = make_hit(S, ro, d, __int_as_float(hit.x), hit.y, hit.z);
      const Bsdf b = make_bsdf(S, h, hit.y);
      const V3 w = v3(in.w[3 * i], in.w[3 * i + 1], in.w[3 * i + 2]);
      const V3 inc = d * -1.0f;
      PhotonRec rec;
      rec.p[0] = h.p.x;
      rec.p[1] = h.p.y;
      rec.p[2] = h.p.z;
      rec.w[0] = w.x;
      rec.w[1] = w.y;
      rec.w[2] = w.z;
      rec.dir = compress_dir(inc.x, inc.y, inc.z);
      rec.nrm = compress_dir(h.ng.x, h.ng.y, h.ng.z);
      const bool specular_bsdf = bsdf_ncomp(b) == 0;  // no non-specular component: no photon stored
      if (bounce == 0) {
        if (!specular_bsdf) {
          st_direct[path] = rec;
          has_direct[path] = 1;
        }
      } else if (!diffuse_path) {
        // all bounces so far specular: a caustic photon (at most one per
        // path: the bounce after it is not specular)
        if (!specular_bsdf) {
          st_caustic[path] = rec;
          has_caustic[path] = 1;
        }
      } else {
        // indirect photons also land on specular surfaces (the reference's
        // note at PhotonShootingPipeline.cpp:203-210)
        const int c = n_indirect[path];
        if (c < A.slots) {
          st_indirect[(int64_t)path * A.slots + c] = rec;
          n_indirect[path] = c + 1;
        } else {
          atomicOr(A.overflow, 1);
        }
      }
      // BSDF::Sample over all components
      float uc, u0, u1;
      const uint64_t gp = (uint64_t)(path0 + path);
      if (bounce == 0) {
        const unsigned pi = (unsigned)gp + 1u;
        u0 = (float)radical_inverse(pi, 17);
        u1 = (float)radical_inverse(pi, 19);
        uc = (float)radical_inverse(pi, 23);
      } else {
        u0 = bounce_rnd(A.seed, gp, bounce, 0);
        u1 = bounce_rnd(A.seed, gp, bounce, 1);
        uc = bounce_rnd(A.seed, gp, bounce, 2);
      }
      V3 ex;
      float pdf = 0.0f;
      bool spec_sampled = false;
      const V3 f = bsdf_sample_all(b, inc, uc, u0, u1, ex, pdf, spec_sampled);
      if (pdf > 0.0f && bounce + 1 < A.max_bounces) {
        // no cosine for specular scattering: the BxDF holds it (:229-231)
        wnew = spec_sampled ? mul(w, f) * (1.0f / pdf) : mul(w, f) * (fabsf(dot(ex, b.n)) / pdf);
        if (!spec_sampled) diffuse_path = kDiffusePath;
        float p = A.rr_probability;
        if (!(p > 0.0f)) {
          const float lw = luminance(w);
          p = lw > 0.0f ? fminf(1.0f, luminance(wnew) / lw) : 0.0f;
        }
        const float r = bounce_rnd(A.seed, gp, bounce, 3);
        if (!(r > p) && p > 0.0f) {
          wnew = wnew * (1.0f / p);
          o = h.p;
          dnew = ex;
          tmin = next_min_t(S, h, ex);
          cont = true;
        }
      }
    }
  }
  const int q = queue_append(cont, out.count);
  if (cont) queue_push(out, q, o, dnew, tmin, wnew, path | diffuse_path);
}

// Exclusive scan of per-path counts, 1024 per block, then block offsets.
constexpr int kScanBlock = 1024;

template <typename T>
__global__ void k_scan_blocks(const T *__restrict__ cnt, int n, int stride_mul, int *__restrict__ excl,
                              int *__restrict__ block_sums) {
  __shared__ int s[kScanBlock];
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  const int v = i < n ? (int)cnt[i] * stride_mul : 0;
  s[threadIdx.x] = v;
  __syncthreads();
  for (int off = 1; off < kScanBlock; off <<= 1) {
    const int t = threadIdx.x >= off ? s[threadIdx.x - off] : 0;
    __syncthreads();
    s[threadIdx.x] += t;
    __syncthreads();
  }
  if (i < n) excl[i] = s[threadIdx.x] - v;
  if (threadIdx.x == kScanBlock - 1) block_sums[blockIdx.x] = s[threadIdx.x];
}

// Exclusive scan of the block sums in place (one block, any count); the
// total goes to *total.
__global__ void k_scan_sums(int *__restrict__ sums, int nb, int *__restrict__ total) {
  __shared__ int s[kScanBlock];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nb; base += kScanBlock) {
    const int i = base + threadIdx.x;
    const int v = i < nb ? sums[i] : 0;
    s[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < kScanBlock; off <<= 1) {
      const int t = threadIdx.x >= off ? s[threadIdx.x - off] : 0;
      __syncthreads();
      s[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < nb) sums[i] = carry + s[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == kScanBlock - 1) carry += s[threadIdx.x];
    __syncthreads();
  }
  if (threadIdx.x == 0) *total = carry;
}

// Copies path i's deposits (count per path from has/cnt) to their place.
__global__ void k_gather_photons(const PhotonRec *__restrict__ staging, int per_path, const uint8_t *__restrict__ has,
                                 const int *__restrict__ cnt, int n, const int *__restrict__ excl,
                                 const int *__restrict__ block_off, PhotonRec *__restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int c = has ? (int)has[i] : cnt[i];
  const int o = excl[i] + block_off[i / kScanBlock];
  for (int j = 0; j < c; ++j) out[o + j] = staging[(int64_t)i * per_path + j];
}

// _LookupPhotonIrradiance (PhotonLTEIntegrator.cpp:127-169) for one map:
// the weights of the found photons (k-NN output, the reference's heap
// order) summed in double by the side of the query normal they arrive from,
// over pi * paths * r^2 with the reference's radius rule; the result (float)
// is added to the running irradiance of the query, so that the maps combine
// as (caustic + direct) + indirect in float.
__global__ void k_irradiance_sum(const float4 *__restrict__ nodes, const float *__restrict__ weight,
                                 const uint16_t *__restrict__ dirid, const double *__restrict__ dirs,
                                 const double *__restrict__ q, const double *__restrict__ qn,
                                 const int32_t *__restrict__ idx, const int32_t *__restrict__ count, int nq, int k,
                                 double paths, double max_lookup_dist, bool first, float *__restrict__ ext,
                                 float *__restrict__ intr) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nq) return;
  const int found = count[i];
  float e[3] = {0, 0, 0}, in[3] = {0, 0, 0};
  if (found > 0) {
    double se[3] = {0, 0, 0}, si[3] = {0, 0, 0}, md2 = 0.0;
    const double px = q[3 * i], py = q[3 * i + 1], pz = q[3 * i + 2];
    const double nx = qn[3 * i], ny = qn[3 * i + 1], nz = qn[3 * i + 2];
    for (int j = 0; j < found; ++j) {
      const int t = idx[(int64_t)i * k + j];
      const float4 p = nodes[t];
      const double dx = __dsub_rn((double)p.x, px), dy = __dsub_rn((double)p.y, py), dz = __dsub_rn((double)p.z, pz);
      const double d2 = __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
      if (d2 > md2) md2 = d2;
      const int did = dirid[t];
      const double c = __dadd_rn(__dadd_rn(__dmul_rn(dirs[3 * did], nx), __dmul_rn(dirs[3 * did + 1], ny)),
                                 __dmul_rn(dirs[3 * did + 2], nz));
      double *acc = c > 0.0 ? se : si;
      acc[0] = __dadd_rn(acc[0], (double)weight[3 * (int64_t)t]);
      acc[1] = __dadd_rn(acc[1], (double)weight[3 * (int64_t)t + 1]);
      acc[2] = __dadd_rn(acc[2], (double)weight[3 * (int64_t)t + 2]);
    }
    if (found < k || md2 == 0.0)
      md2 = __dmul_rn(max_lookup_dist, max_lookup_dist);
    else
      md2 = __dmul_rn(md2, __ddiv_rn((double)found, __dsub_rn((double)found, 0.5)));
    const double inv = __ddiv_rn(1.0, __dmul_rn(__dmul_rn(3.14159265358979323846, paths), md2));
    for (int c = 0; c < 3; ++c) {
      e[c] = (float)__dmul_rn(se[c], inv);
      in[c] = (float)__dmul_rn(si[c], inv);
    }
  }
  for (int c = 0; c < 3; ++c) {
    if (first) {
      ext[3 * i + c] = e[c];
      intr[3 * i + c] = in[c];
    } else {
      ext[3 * i + c] = __fadd_rn(ext[3 * i + c], e[c]);
      intr[3 * i + c] = __fadd_rn(intr[3 * i + c], in[c]);
    }
  }
}

}  // namespace

size_t photon_chunk_bytes(int64_t n_paths, int slots) {
  const int64_t B1 = slots > 1 ? slots : 1;
  auto al = [](int64_t x) { return (size_t)((x + 255) & ~(int64_t)255); };
  const int64_t nb = (n_paths + kScanBlock - 1) / kScanBlock;
  return 2 * (al(n_paths * 32) + al(n_paths * 12) + al(n_paths * 4)) + al(n_paths * 16) + 256 +
         al(n_paths * 28) + al(n_paths) + al(n_paths * B1 * 28) + al(n_paths * 4) + 3 * al(n_paths * 4) +
         3 * al(nb * 4) + 256 + al(n_paths * 28) + al(n_paths);
}

cudaError_t photon_shoot_chunk(const SceneDev &S, const PhotonShootArgs &A, const TraceFn &trace, int64_t path0,
                               int n_paths, void *ws, PhotonRec *out_direct, PhotonRec *out_indirect,
                               PhotonRec *out_caustic, int *d_totals, cudaStream_t st) {
  const int64_t B1 = A.slots > 1 ? A.slots : 1;
  auto al = [](int64_t x) { return (size_t)((x + 255) & ~(int64_t)255); };
  char *p = (char *)ws;
  auto take = [&](size_t b) {
    char *r = p;
    p += b;
    return r;
  };
  Queue Q[2];
  for (int k = 0; k < 2; ++k) {
    Q[k].rays = (float4 *)take(al((int64_t)n_paths * 32));
    Q[k].w = (float *)take(al((int64_t)n_paths * 12));
    Q[k].path = (int *)take(al((int64_t)n_paths * 4));
  }
  int4 *hits = (int4 *)take(al((int64_t)n_paths * 16));
  int *counts = (int *)take(256);
  Q[0].count = counts;
  Q[1].count = counts + 1;
  PhotonRec *st_direct = (PhotonRec *)take(al((int64_t)n_paths * 28));
  uint8_t *has_direct = (uint8_t *)take(al(n_paths));
  PhotonRec *st_indirect = (PhotonRec *)take(al((int64_t)n_paths * B1 * 28));
  int *n_indirect = (int *)take(al((int64_t)n_paths * 4));
  int *excl[3] = {(int *)take(al((int64_t)n_paths * 4)), (int *)take(al((int64_t)n_paths * 4)),
                  (int *)take(al((int64_t)n_paths * 4))};
  const int nb = (n_paths + kScanBlock - 1) / kScanBlock;
  int *bsum[3] = {(int *)take(al((int64_t)nb * 4)), (int *)take(al((int64_t)nb * 4)), (int *)take(al((int64_t)nb * 4))};
  PhotonRec *st_caustic = (PhotonRec *)take(al((int64_t)n_paths * 28));
  uint8_t *has_caustic = (uint8_t *)take(al(n_paths));
  cudaError_t e;
  if ((e = cudaMemsetAsync(counts, 0, 2 * sizeof(int), st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(has_direct, 0, (size_t)n_paths, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(has_caustic, 0, (size_t)n_paths, st)) != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(n_indirect, 0, (size_t)n_paths * 4, st)) != cudaSuccess) return e;
  const unsigned grid = (unsigned)((n_paths + 127) / 128);
  k_photon_emit<<<grid, 128, 0, st>>>(S, A, path0, n_paths, Q[0]);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  for (int b = 0; b < A.max_bounces; ++b) {
    Queue &in = Q[b & 1], &out = Q[(b + 1) & 1];
    if ((e = trace(in.rays, n_paths, in.count, hits, st, counts + 8)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(out.count, 0, sizeof(int), st)) != cudaSuccess) return e;
    k_photon_bounce<<<grid, 128, 0, st>>>(S, A, path0, b, n_paths, in, hits, out, st_direct, has_direct,
                                          st_indirect, n_indirect, st_caustic, has_caustic);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (A.max_bounces > 16 && (b & 7) == 7 && b + 1 < A.max_bounces) {
      // long caps: stop launching once every path of the chunk has ended
      int left = 0;
      if ((e = cudaMemcpyAsync(&left, out.count, sizeof(int), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
          (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return e;
      if (left == 0) break;
    }
  }
  // direct: one per path; indirect: n_indirect[path] per path
  k_scan_blocks<uint8_t><<<nb, kScanBlock, 0, st>>>(has_direct, n_paths, 1, excl[0], bsum[0]);
  k_scan_sums<<<1, kScanBlock, 0, st>>>(bsum[0], nb, d_totals);
  k_gather_photons<<<grid, 128, 0, st>>>(st_direct, 1, has_direct, nullptr, n_paths, excl[0], bsum[0], out_direct);
  k_scan_blocks<int><<<nb, kScanBlock, 0, st>>>(n_indirect, n_paths, 1, excl[1], bsum[1]);
  k_scan_sums<<<1, kScanBlock, 0, st>>>(bsum[1], nb, d_totals + 1);
  k_gather_photons<<<grid, 128, 0, st>>>(st_indirect, (int)B1, nullptr, n_indirect, n_paths, excl[1], bsum[1],
                                         out_indirect);
  // caustic: at most one per path
  k_scan_blocks<uint8_t><<<nb, kScanBlock, 0, st>>>(has_caustic, n_paths, 1, excl[2], bsum[2]);
  k_scan_sums<<<1, kScanBlock, 0, st>>>(bsum[2], nb, d_totals + 2);
  k_gather_photons<<<grid, 128, 0, st>>>(st_caustic, 1, has_caustic, nullptr, n_paths, excl[2], bsum[2], out_caustic);
  return cudaGetLastError();
}

cudaError_t launch_irradiance_sum(const void *nodes, const float *weight, const uint16_t *dirid, const double *dirs,
                                  const double *q, const double *qn, const int32_t *idx, const int32_t *count,
                                  int64_t nq, int k, double paths, double max_lookup_dist, bool first, float *ext,
                                  float *intr, cudaStream_t st) {
  if (nq <= 0) return cudaSuccess;
  k_irradiance_sum<<<(unsigned)((nq + 127) / 128), 128, 0, st>>>((const float4 *)nodes, weight, dirid, dirs, q, qn,
                                                                  idx, count, (int)nq, k, paths, max_lookup_dist, first,
                                                                  ext, intr);
  return cudaGetLastError();
}

// ------------------------------------------------------------ final gather --
// PhotonLTEIntegrator::_FinalGather (PhotonLTEIntegrator.cpp:387-577) as
// stages over the camera hits of a render pass:
//   k_gather_sources  camera hits with a surface -> query points of the
//                     32-photon lookup in the indirect map
//   k_gather_rays     gather_samples BSDF-sampled and gather_samples
//                     photon-guided directions (uniform cone of 10 degrees
//                     around a found photon's incident direction), each
//                     weighted with the power heuristic of the two densities
//   k_trace           closest hit of the gather rays
//   k_gather_hits     at each gather hit: BSDF::TotalScattering over the
//                     reflection components (a 5x5 grid of samples) and the
//                     query of the nearest irradiance photon
//   k_gather_resolve  TotalScattering * irradiance / pi * weight / gather_samples
namespace {

constexpr double kCosGather = 0.9848;  // 10 degrees (PhotonLTEIntegrator.cpp:397)
constexpr int kGatherLookup = 32;      // :446-456

// The gather stages' random numbers: a stream of their own per sample.
__device__ __forceinline__ float rnd_g(uint64_t seed, uint64_t gid, uint32_t d) {
  return rnd(seed ^ 0x5851F42D4C957F2Dull, gid * 8ull + (d >> 6), d & 63u);
}

struct GatherArgs {
  int n;               // shading points: the pass's samples, or a chunk of a specular level
  int64_t px_begin;
  int spp;
  int slots;
  int base_slot;       // first gather slot of a sample
  int gs;              // gather samples (a square, as the sampler rounds it)
  const ViewDev *views;
  int n_views;
  SpecSource sp;       // in_sample null: camera hits
};

// Camera sample, random-stream seed, weight and first target slot of
// shading point i (a camera hit, or a specular-level entry).
struct PointRef {
  int sample;
  uint64_t gid, seed;
  V3 w;
  int64_t slot0;
};
__device__ __forceinline__ PointRef point_ref(const GatherArgs &G, int i) {
  PointRef r;
  unsigned node = 1;
  r.sample = i;
  r.w = v3(1.0f, 1.0f, 1.0f);
  if (G.sp.in_sample) {
    r.sample = G.sp.in_sample[i];
    node = (unsigned)G.sp.in_node[i];
    r.w = load3(G.sp.in_w + 3 * (int64_t)i);
  }
  const int64_t P = G.px_begin + r.sample / G.spp;
  int lo = 0, hi = G.n_views - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (G.views[mid].px_begin <= P) lo = mid; else hi = mid - 1;
  }
  r.gid = (uint64_t)((P - G.views[lo].px_begin) * G.spp + r.sample % G.spp);
  r.seed = G.views[lo].seed;
  if (G.sp.in_sample) r.seed ^= 0xA0761D6478BD642Full * (uint64_t)node;  // as k_shade's specular levels
  r.slot0 = G.sp.in_sample ? (int64_t)r.sample * G.slots + G.sp.slot : (int64_t)r.sample * G.slots + G.base_slot;
  return r;
}

__global__ void k_gather_sources(SceneDev S, GatherArgs G, const float4 *__restrict__ rays,
                                 const int4 *__restrict__ hits, int *__restrict__ src, double *__restrict__ q,
                                 double *__restrict__ qn, int *__restrict__ count) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool ok = false;
  Hit h{};
  if (i < G.n) {
    const int4 hit = hits[i];
    // only surfaces with a non-specular component (PhotonLTEIntegrator.cpp:337-343)
    if (hit.y >= 0) {
      const float4 ra = rays[2 * i], rb = rays[2 * i + 1];
      h = make_hit(S, v3(ra.x, ra.y, ra.z), v3(ra.w, rb.x, rb.y), __int_as_float(hit.x), hit.y, hit.z);
      ok = bsdf_ncomp(make_bsdf(S, h, hit.y)) > 0;
    }
  }
  const int j = queue_append(ok, count);
  if (ok) {
    src[j] = i;
    q[3 * j] = h.p.x;
    q[3 * j + 1] = h.p.y;
    q[3 * j + 2] = h.p.z;
    qn[3 * j] = h.ng.x;
    qn[3 * j + 1] = h.ng.y;
    qn[3 * j + 2] = h.ng.z;
  }
}

__device__ __forceinline__ float photon_pdf_of(const V3 *pd, int found, V3 w) {
  // uniform cones around the found photons' directions (:473-481, 515-523)
  const float cone_pdf = (float)(1.0 / (2.0 * 3.14159265358979323846 * (1.0 - kCosGather)));
  int c = 0;
  for (int j = 0; j < found; ++j) c += dot(pd[j], w) > (float)kCosGather ? 1 : 0;
  return found > 0 ? c * cone_pdf / found : 0.0f;
}

__global__ void __launch_bounds__(128) k_gather_rays(SceneDev S, GatherArgs G, GatherMaps M,
                                                     const float4 *__restrict__ rays, const int4 *__restrict__ hits,
                                                     const int *__restrict__ src, const int *__restrict__ src_count,
                                                     const int32_t *__restrict__ kidx,
                                                     const int32_t *__restrict__ kcount, float4 *__restrict__ grays,
                                                     int *__restrict__ gtarget, float *__restrict__ gweight,
                                                     int *__restrict__ gcount) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = j < *src_count;
  Hit h{};
  Bsdf b{};
  V3 wo = v3(0, 0, 0);
  uint64_t gid = 0, seed = 0;
  int64_t slot0 = 0;
  int found = 0;
  V3 ew = v3(1.0f, 1.0f, 1.0f);  // specular-level weight of the shading point
  const bool acc = G.sp.in_sample != nullptr;
  V3 pd[kGatherLookup];
  if (valid) {
    const int i = src[j];
    const int4 hit = hits[i];
    const float4 ra = rays[2 * i], rb = rays[2 * i + 1];
    const V3 d = v3(ra.w, rb.x, rb.y);
    h = make_hit(S, v3(ra.x, ra.y, ra.z), d, __int_as_float(hit.x), hit.y, hit.z);
    b = make_bsdf(S, h, hit.y);
    wo = d * -1.0f;
    const PointRef pr = point_ref(G, i);
    gid = pr.gid;
    seed = pr.seed;
    slot0 = pr.slot0;
    ew = pr.w;
    found = kcount[j];
    for (int k = 0; k < found; ++k) {
      const int did = M.ind_dirid[kidx[(int64_t)j * kGatherLookup + k]];
      pd[k] = v3((float)M.dirs[3 * did], (float)M.dirs[3 * did + 1], (float)M.dirs[3 * did + 2]);
    }
  }
  const V3 ns = b.n;
  const int gs = G.gs;
  // BSDF samples (:468-497)
  for (int k = 0; k < gs; ++k) {
    bool want = false;
    V3 ex = v3(0, 0, 0), wt = v3(0, 0, 0);
    float tmin = 0.0f;
    if (valid) {
      const float uc = rnd_g(seed, gid, 3 * k), u0 = rnd_g(seed, gid, 3 * k + 1), u1 = rnd_g(seed, gid, 3 * k + 2);
      float pdf = 0.0f;
      const V3 f = bsdf_sample(b, wo, uc, u0, u1, ex, pdf);
      if (pdf > 0.0f && !black(f)) {
        const float ppdf = photon_pdf_of(pd, found, ex);
        const float w = power_heuristic(gs, pdf, gs, ppdf);
        wt = f * (w * fabsf(dot(ex, ns)) / pdf);
        tmin = next_min_t(S, h, ex);
        want = true;
      }
    }
    const int q = queue_append(want, gcount);
    if (want) {
      store_ray(grays, q, h.p, ex, tmin, __int_as_float(0x7f800000));
      gtarget[q] = (int)(acc ? slot0 : slot0 + k);
      store_rgb(gweight, q, mul(wt, ew));
    }
  }
  // Photon-guided samples (:499-533)
  for (int k = 0; k < gs; ++k) {
    bool want = false;
    V3 ex = v3(0, 0, 0), wt = v3(0, 0, 0);
    float tmin = 0.0f;
    if (valid && found > 0) {
      const float u = rnd_g(seed, gid, 3 * gs + 3 * k), c0 = rnd_g(seed, gid, 3 * gs + 3 * k + 1),
                  c1 = rnd_g(seed, gid, 3 * gs + 3 * k + 2);
      const int si = min((int)(u * found), found - 1);
      const V3 n = pd[si];
      // MathRoutines::CoordinateSystem (Math/MathRoutines.h:298-312)
      V3 e2;
      if (fabsf(n.x) > fabsf(n.y)) {
        const float il = 1.0f / sqrtf(n.x * n.x + n.z * n.z);
        e2 = v3(-n.z * il, 0.0f, n.x * il);
      } else {
        const float il = 1.0f / sqrtf(n.y * n.y + n.z * n.z);
        e2 = v3(0.0f, n.z * il, -n.y * il);
      }
      const V3 e3 = cross(n, e2);
      // UniformConeSampling (SamplingRoutines.h:300-310)
      const float ct = (1.0f - c0) + c0 * (float)kCosGather, st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct));
      const float phi = c1 * 2.0f * kPi;
      ex = normalized(e2 * (st * cosf(phi)) + e3 * (st * sinf(phi)) + n * ct);
      const V3 f = bsdf_eval(b, wo, ex);
      if (!black(f)) {
        const float bpdf = bsdf_pdf(b, wo, ex);
        const float ppdf = photon_pdf_of(pd, found, ex);
        if (ppdf > 0.0f) {
          const float w = power_heuristic(gs, ppdf, gs, bpdf);
          wt = f * (w * fabsf(dot(ex, ns)) / ppdf);
          tmin = next_min_t(S, h, ex);
          want = true;
        }
      }
    }
    const int q = queue_append(want, gcount);
    if (want) {
      store_ray(grays, q, h.p, ex, tmin, __int_as_float(0x7f800000));
      gtarget[q] = (int)(acc ? slot0 : slot0 + gs + k);
      store_rgb(gweight, q, mul(wt, ew));
    }
  }
}

// BxDF::TotalScattering (Core/BxDF.cpp:43-69) of one non-Lambertian BxDF
// with the 5x5 grid of BSDF::TotalScattering's caller.  The reference hands
// the BxDF the WORLD incident direction (BSDF.cpp:213-219 passes i_incident,
// not its local form), which the BxDF then treats as local; this keeps that.
// what: 0 Oren-Nayar, 1 the Blinn microfacet, 2 FresnelBlend.
__device__ V3 total_scattering_bxdf(const Layer &b, int what, V3 wi) {
  V3 ret = v3(0, 0, 0);
  for (int y = 0; y < 5; ++y)
    for (int x = 0; x < 5; ++x) {
      const float u0 = (x + 0.5f) * 0.2f, u1 = (y + 0.5f) * 0.2f;
      V3 wo;
      float pdf;
      V3 f;
      if (what == 1) {
        // Microfacet::Sample (BxDFs/Microfacet.h:112-129) with BlinnDistribution::Sample
        if (!blinn_sample(b.exponent, wi, u0, u1, wo)) continue;
        pdf = microfacet_pdf(b, wi, wo);
        f = microfacet_eval(b, wi, wo);
      } else if (what == 2) {
        // FresnelBlend::Sample: the lobe mixture, Evaluate at the sampled direction
        if (!fb_sample(b, wi, u0, u1, wo)) continue;
        pdf = fb_pdf(b, wi, wo);
        f = fb_eval(b, wi, wo);
      } else {
        wo = cosine_hemisphere(u0, u1);
        if (wi.z < 0.0f) wo.z = -wo.z;
        pdf = diffuse_pdf(wi, wo);
        f = diffuse_eval(b, wi, wo);
      }
      if (pdf > 0.0f) ret = ret + f * (fabsf(wo.z) / pdf);
    }
  ret = ret * (1.0f / 25.0f);
  return v3(fminf(1.0f, fmaxf(0.0f, ret.x)), fminf(1.0f, fmaxf(0.0f, ret.y)), fminf(1.0f, fmaxf(0.0f, ret.z)));
}

// BxDF::TotalScattering of the measured BRDF: MERLMeasured::Sample over the
// same grid, again with the world incident direction taken as local.
__device__ V3 total_scattering_measured(const Layer &b, V3 wi) {
  V3 ret = v3(0, 0, 0);
  for (int y = 0; y < 5; ++y)
    for (int x = 0; x < 5; ++x) {
      V3 wo;
      float pdf = 0.0f;
      const V3 f = merl_sample(b.merl, wi, (x + 0.5f) * 0.2f, (y + 0.5f) * 0.2f, wo, pdf);
      if (pdf > 0.0f) ret = ret + f * (fabsf(wo.z) / pdf);
    }
  ret = ret * (1.0f / 25.0f);
  return v3(fminf(1.0f, fmaxf(0.0f, ret.x)), fminf(1.0f, fmaxf(0.0f, ret.y)), fminf(1.0f, fmaxf(0.0f, ret.z)));
}

__device__ __forceinline__ V3 clamp01(V3 r) {
  return v3(fminf(1.0f, fmaxf(0.0f, r.x)), fminf(1.0f, fmaxf(0.0f, r.y)), fminf(1.0f, fmaxf(0.0f, r.z)));
}

// BSDF::TotalScattering (BSDF.cpp:209-224) over the reflection components
// (refl: the non-specular ones and a specular reflection) and over the
// transmission components (trans: a specular transmission), each sum
// clamped; every layer's components scaled by the layer's scale
// (ScaledBxDF::TotalScattering).  SpecularReflection / SpecularTransmission::
// TotalScattering (BxDFs/SpecularReflection.h, SpecularTransmission.cpp:
// 75-92) receive the WORLD incident direction as if it were local too, so
// the Fresnel term and the total-internal-reflection test read its world z.
__device__ void total_scattering(const Bsdf &bs, V3 wi, V3 &refl, V3 &trans) {
  refl = trans = v3(0, 0, 0);
  for (int i = 0; i < bs.nl; ++i) {
    const Layer b = i == 0 ? bs.L0 : layer1(bs);
    V3 r = v3(0, 0, 0), t = v3(0, 0, 0);
    switch (b.kind) {
      case kMeasured: r = total_scattering_measured(b, wi); break;
      case kLambert: r = b.kd; break;  // Lambertian::TotalScattering returns kd
      case kOrenNayar: r = total_scattering_bxdf(b, 0, wi); break;
      case kPlastic: r = b.kd + total_scattering_bxdf(b, 1, wi); break;
      case kMetal: r = total_scattering_bxdf(b, 1, wi); break;
      case kSubstrate: r = total_scattering_bxdf(b, 2, wi); break;
      case kUber:
        if (!black(b.kd)) r = b.kd;
        if (!black(b.ks)) r = r + total_scattering_bxdf(b, 1, wi);
        break;
      default: break;
    }
    const V3 sr = layer_spec_r(b), st = layer_spec_t(b);
    if (!black(sr) || !black(st)) {
      const float F = fresnel_dielectric_ior(wi.z, b.ior);
      if (!black(sr)) r = r + clamp01(sr * F);
      const float eta = wi.z >= 0.0f ? 1.0f / b.ior : b.ior;
      const bool tir = eta * eta * (1.0f - wi.z * wi.z) >= 1.0f;
      if (!black(st) && !tir) t = clamp01(st * (1.0f - F));
    }
    refl = refl + mul(b.scale, r);
    trans = trans + mul(b.scale, t);
  }
  refl = clamp01(refl);
  trans = clamp01(trans);
}

// ts: TotalScattering over the reflection components (times the irradiance
// on the side the gather ray comes from), tt: over the transmission
// components (times the irradiance on the other side; only a transparent
// BSDF has one) -- PhotonLTEIntegrator.cpp:556-567.
__global__ void k_gather_hits(SceneDev S, const float4 *__restrict__ grays, const int4 *__restrict__ ghits,
                              const int *__restrict__ gcount, int *__restrict__ hsrc, double *__restrict__ q,
                              double *__restrict__ qn, float *__restrict__ ts, float *__restrict__ tt,
                              uint8_t *__restrict__ side, int *__restrict__ hcount) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  bool ok = false;
  Hit h{};
  V3 t = v3(0, 0, 0), tr = v3(0, 0, 0);
  bool outside = false;
  if (i < *gcount) {
    const int4 hit = ghits[i];
    if (hit.y >= 0) {
      const float4 ra = grays[2 * i], rb = grays[2 * i + 1];
      const V3 d = v3(ra.w, rb.x, rb.y);
      h = make_hit(S, v3(ra.x, ra.y, ra.z), d, __int_as_float(hit.x), hit.y, hit.z);
      const Bsdf b = make_bsdf(S, h, hit.y);
      const V3 gdir = d * -1.0f;
      outside = dot(gdir, h.ng) > 0.0f;
      total_scattering(b, gdir, t, tr);
      ok = true;
    }
  }
  const int j = queue_append(ok, hcount);
  if (ok) {
    hsrc[j] = i;
    q[3 * j] = h.p.x;
    q[3 * j + 1] = h.p.y;
    q[3 * j + 2] = h.p.z;
    qn[3 * j] = h.ng.x;
    qn[3 * j + 1] = h.ng.y;
    qn[3 * j + 2] = h.ng.z;
    ts[3 * j] = t.x;
    ts[3 * j + 1] = t.y;
    ts[3 * j + 2] = t.z;
    tt[3 * j] = tr.x;
    tt[3 * j + 1] = tr.y;
    tt[3 * j + 2] = tr.z;
    side[j] = outside ? 1 : 0;
  }
}

__global__ void k_gather_resolve(GatherMaps M, int gs, const int *__restrict__ hcount, const int *__restrict__ hsrc,
                                 const int32_t *__restrict__ nearest, const float *__restrict__ ts,
                                 const float *__restrict__ tt, const uint8_t *__restrict__ side,
                                 const int *__restrict__ gtarget, const float *__restrict__ gweight,
                                 float *__restrict__ contrib, bool accumulate) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= *hcount) return;
  const int t = nearest[j];
  if (t < 0) return;
  // the side the gather ray arrives from selects external or internal
  // irradiance for the reflection part, the other side for transmission
  const float *E = (side[j] ? M.irr_ext : M.irr_int) + 3 * (int64_t)t;
  const float *Eo = (side[j] ? M.irr_int : M.irr_ext) + 3 * (int64_t)t;
  const int g = hsrc[j];
  const int64_t slot = gtarget[g];
  const float s = kInvPi / gs;
  for (int c = 0; c < 3; ++c) {
    float te = ts[3 * j + c] * E[c];
    if (tt[3 * j + c] != 0.0f) te += tt[3 * j + c] * Eo[c];
    const float v = te * gweight[3 * g + c] * s;
    if (accumulate) {
      if (v != 0.0f) atomicAdd(contrib + 3 * slot + c, v);
    } else {
      contrib[3 * slot + c] = v;
    }
  }
}

// _LookupCausticRadiance (PhotonLTEIntegrator.cpp:579-627) at camera hit j
// of the pass, from the k-NN output in the reference's heap order: each
// found photon adds BSDF(photon direction, viewer) * weight * Simpson's
// kernel 3/pi (1 - d2 / m)^2 (_PhotonKernel, :629-636), where m is the
// largest squared distance among the photons visited so far -- the
// reference's running maximum, not the final radius (so the first photon
// always gets kernel 0).  The sum is divided by the caustic paths times the
// area term: the lookup radius squared when fewer than k were found (or
// m == 0), else m * n / (n - 0.5).  Sums in double, as the reference's
// Spectrum_d; the BSDF in float as everywhere in this renderer.
__global__ void __launch_bounds__(128) k_caustic_resolve(SceneDev S, GatherArgs G, CausticMap C,
                                                         const float4 *__restrict__ rays,
                                                         const int4 *__restrict__ hits, const int *__restrict__ src,
                                                         const int *__restrict__ src_count,
                                                         const int32_t *__restrict__ kidx,
                                                         const double *__restrict__ kd2,
                                                         const int32_t *__restrict__ kcount, int slot,
                                                         float *__restrict__ contrib) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= *src_count) return;
  const int found = kcount[j];
  if (found <= 0) return;
  const int i = src[j];
  const int4 hit = hits[i];
  const float4 ra = rays[2 * i], rb = rays[2 * i + 1];
  const V3 dir = v3(ra.w, rb.x, rb.y);
  const Hit h = make_hit(S, v3(ra.x, ra.y, ra.z), dir, __int_as_float(hit.x), hit.y, hit.z);
  const Bsdf b = make_bsdf(S, h, hit.y);
  const V3 wo = v3(-dir.x, -dir.y, -dir.z);
  double m = 0.0, r0 = 0.0, r1 = 0.0, r2 = 0.0;
  for (int f = 0; f < found; ++f) {
    const int64_t e = (int64_t)j * C.k + f;
    const int t = kidx[e];
    const double d2 = kd2[e];
    if (d2 > m) m = d2;
    const double u = 1.0 - d2 / m;
    const double kern = 3.0 * 0.31830988618379067154 * u * u;
    const uint16_t id = C.dirid[t];
    const V3 wi = v3((float)C.dirs[3 * id], (float)C.dirs[3 * id + 1], (float)C.dirs[3 * id + 2]);
    const V3 f3 = bsdf_eval(b, wi, wo);
    r0 += (double)f3.x * (double)C.weight[3 * t] * kern;
    r1 += (double)f3.y * (double)C.weight[3 * t + 1] * kern;
    r2 += (double)f3.z * (double)C.weight[3 * t + 2] * kern;
  }
  if (found < C.k || m == 0.0)
    m = C.max_dist * C.max_dist;
  else
    m *= (double)found / ((double)found - 0.5);
  const double sc = 1.0 / (C.paths * m);
  if (G.sp.in_sample) {  // a specular-level entry: weighted, added into its sample's slot
    const PointRef pr = point_ref(G, i);
    float *o = contrib + 3 * pr.slot0;
    const float v[3] = {(float)(r0 * sc) * pr.w.x, (float)(r1 * sc) * pr.w.y, (float)(r2 * sc) * pr.w.z};
    for (int c = 0; c < 3; ++c)
      if (v[c] != 0.0f) atomicAdd(o + c, v[c]);
    return;
  }
  float *o = contrib + 3 * ((int64_t)i * G.slots + slot);
  o[0] = (float)(r0 * sc);
  o[1] = (float)(r1 * sc);
  o[2] = (float)(r2 * sc);
}

}  // namespace

size_t caustic_bytes(int64_t n, int k) {
  auto al = [](int64_t x) { return (size_t)((x + 255) & ~(int64_t)255); };
  return 256 + al(n * 4) + 2 * al(n * 24) + al(n * (int64_t)k * 4) + al(n * (int64_t)k * 8) + al(n * 4) +
         al((int64_t)knn_scratch_bytes(n, k)) + 256;
}

cudaError_t launch_caustic(const SceneDev &S, const CausticMap &C, const ViewDev *views, int n_views, int n,
                           int64_t px_begin, int spp, int slots, int slot, const void *rays, const void *hits,
                           void *cws, float *contrib, unsigned *status, cudaStream_t st, const SpecSource *sp) {
  if (n <= 0 || C.n <= 0 || C.k <= 0) return cudaSuccess;
  auto al = [](int64_t x) { return (size_t)((x + 255) & ~(int64_t)255); };
  char *p = (char *)cws;
  auto take = [&](size_t b) {
    char *r = p;
    p += b;
    return r;
  };
  int *counts = (int *)take(256);
  int *src = (int *)take(al((int64_t)n * 4));
  double *q = (double *)take(al((int64_t)n * 24)), *qn = (double *)take(al((int64_t)n * 24));
  int32_t *kidx = (int32_t *)take(al((int64_t)n * C.k * 4));
  double *kd2 = (double *)take(al((int64_t)n * C.k * 8));
  int32_t *kcnt = (int32_t *)take(al((int64_t)n * 4));
  void *scratch = take(al((int64_t)knn_scratch_bytes(n, C.k)));
  // GatherArgs: only n, px_begin, spp, slots and the views are used here
  GatherArgs G{n, px_begin, spp, slots, slot, 0, views, n_views, sp ? *sp : SpecSource{}};
  cudaError_t e;
  if ((e = cudaMemsetAsync(counts, 0, sizeof(int), st)) != cudaSuccess) return e;
  k_gather_sources<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(S, G, (const float4 *)rays, (const int4 *)hits, src, q,
                                                                 qn, counts);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  // PhotonFilter at the hit's geometric normal, MAX_NORMAL_DEVIATION_COS = 0.87 (:27, :593-594)
  if ((e = launch_knn(C.nodes, C.nids, C.dirs, C.n, q, qn, n, C.k, C.max_dist, 0.87, kidx, kd2, kcnt, nullptr,
                      scratch, status, st, counts)) != cudaSuccess)
    return e;
  k_caustic_resolve<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(S, G, C, (const float4 *)rays, (const int4 *)hits,
                                                                  src, counts, kidx, kd2, kcnt, slot, contrib);
  return cudaGetLastError();
}

cudaError_t launch_gather(const SceneDev &S, const GatherMaps &M, const ViewDev *views, int n_views, int n,
                          int64_t px_begin, int spp, int slots, int base_slot, int gs, const void *rays,
                          const void *hits, void *gws, float *contrib, const TraceFn &trace, unsigned *status,
                          cudaStream_t st, const SpecSource *sp) {
  if (n <= 0 || gs <= 0 || M.n_irr <= 0) return cudaSuccess;
  auto al = [](int64_t x) { return (size_t)((x + 255) & ~(int64_t)255); };
  const int64_t ng = (int64_t)n * 2 * gs;
  char *p = (char *)gws;
  auto take = [&](size_t b) {
    char *r = p;
    p += b;
    return r;
  };
  int *counts = (int *)take(256);  // [0] sources, [1] gather rays, [2] gather hits
  int *src = (int *)take(al((int64_t)n * 4));
  double *q = (double *)take(al((int64_t)n * 24)), *qn = (double *)take(al((int64_t)n * 24));
  int32_t *kidx = (int32_t *)take(al((int64_t)n * kGatherLookup * 4));
  double *kd2 = (double *)take(al((int64_t)n * kGatherLookup * 8));
  int32_t *kcnt = (int32_t *)take(al((int64_t)n * 4));
  float4 *grays = (float4 *)take(al(ng * 32));
  int4 *ghits = (int4 *)take(al(ng * 16));
  int *gtarget = (int *)take(al(ng * 4));
  float *gweight = (float *)take(al(ng * 12));
  int *hsrc = (int *)take(al(ng * 4));
  double *hq = (double *)take(al(ng * 24)), *hqn = (double *)take(al(ng * 24));
  float *ts = (float *)take(al(ng * 12));
  float *tt = (float *)take(al(ng * 12));
  uint8_t *side = (uint8_t *)take(al(ng));
  int32_t *nearest = (int32_t *)take(al(ng * 4));
  uint32_t *bkey = (uint32_t *)take(al(ng * 4));
  int32_t *border = (int32_t *)take(al(ng * 4));
  int *bins = (int *)take(al((int64_t)bin_order_bins() * 4));
  GatherArgs G{n, px_begin, spp, slots, base_slot, gs, views, n_views, sp ? *sp : SpecSource{}};
  cudaError_t e;
  if ((e = cudaMemsetAsync(counts, 0, 3 * sizeof(int), st)) != cudaSuccess) return e;
  k_gather_sources<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(S, G, (const float4 *)rays, (const int4 *)hits, src, q,
                                                                 qn, counts);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if (M.n_ind > 0 &&
      (e = launch_knn(M.ind_nodes, M.ind_nids, M.dirs, M.n_ind, q, qn, n, kGatherLookup, M.ind_lookup_dist, 0.87,
                      kidx, kd2, kcnt, nullptr, nullptr, status, st, counts)) != cudaSuccess)
    return e;
  if (M.n_ind == 0 && (e = cudaMemsetAsync(kcnt, 0, (size_t)n * 4, st)) != cudaSuccess) return e;
  k_gather_rays<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(S, G, M, (const float4 *)rays, (const int4 *)hits, src,
                                                              counts, kidx, kcnt, grays, gtarget, gweight, counts + 1);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = trace(grays, ng, counts + 1, ghits, st, counts + 8)) != cudaSuccess) return e;
  k_gather_hits<<<(unsigned)((ng + 127) / 128), 128, 0, st>>>(S, grays, ghits, counts + 1, hsrc, hq, hqn, ts, tt,
                                                               side, counts + 2);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  // the gather hits' nearest-photon queries in spatial-bin order
  if ((e = launch_bin_order(hq, ng, counts + 2, M.lo, M.hi, bkey, bins, border, st)) != cudaSuccess) return e;
  if ((e = launch_nearest(M.irr_nodes, M.irr_nids, M.dirs, M.n_irr, hq, hqn, ng, M.max_irr_dist, 0.87, nearest,
                          status, st, counts + 2, border)) != cudaSuccess)
    return e;
  k_gather_resolve<<<(unsigned)((ng + 255) / 256), 256, 0, st>>>(M, gs, counts + 2, hsrc, nearest, ts, tt, side,
                                                                  gtarget, gweight, contrib, sp != nullptr);
  return cudaGetLastError();
}

size_t gather_bytes(int64_t n, int gs) {
  auto al = [](int64_t x) { return (size_t)((x + 255) & ~(int64_t)255); };
  const int64_t ng = n * 2 * gs;
  return 256 + al(n * 4) + 2 * al(n * 24) + al(n * kGatherLookup * 4) + al(n * kGatherLookup * 8) + al(n * 4) +
         al(ng * 32) + al(ng * 16) + al(ng * 4) + al(ng * 12) + al(ng * 4) + 2 * al(ng * 24) + 2 * al(ng * 12) +
         al(ng) + al(ng * 4) + 2 * al(ng * 4) + al((int64_t)bin_order_bins() * 4) + 256;
}

}  // namespace skw
