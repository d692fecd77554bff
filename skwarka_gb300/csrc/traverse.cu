// Closest-hit and any-hit traversal of the ternary bbox kd-tree on sm_103a.
//
// Semantics follow TriangleAccelerator::_NodeIntersect / _NodeIntersectTest
// (Raytracer/Core/TriangleAccelerator.cpp:154-293, 354-462):
//   * a stack of nodes; each popped node's AABB is tested against the ray's
//     [tmin, current tmax] with the reference's twelve slab comparisons;
//   * an internal node pushes its present children so that the child on the
//     ray's near side of the split axis is popped first;
//   * a leaf tests its triangles in order with Moller-Trumbore; a hit with
//     tmin <= t <= current tmax replaces the current one (so among exactly
//     equal t the last tested triangle wins) and becomes the new tmax.
//
// The reference does all of this in double precision over float data.  Here
// the node tests run in float: a plane distance is fma(coordinate, 1/d,
// -o/d -+ w) with the per-ray absolute widening w = 6u (B + |o|) |1/d|
// (u = 2^-24, B = the scene's largest absolute coordinate; see SlabRay),
// which bounds the float error for every node, so a node is culled only if
// the reference culls it too.  The triangle test runs in float with a
// forward error bound on every quantity; only when a decision
// (inside/outside an edge, t inside [tmin, tmax], which of two hits is
// nearer) falls inside that bound is the triangle re-tested with the
// reference's exact double-precision arithmetic (round-to-nearest
// intrinsics, no fused multiply-add).  Such hits are flagged
// SKW_HIT_FP64_DECIDED.
//
// Layout: nodes are 32-byte DevNode records read as two 16-byte loads; each
// triangle slot is 3 x float4 (v0|prim, v1|tri, v2|slot); rays are 2 x float4.
// The traversal stack holds 12-byte entries (node words 6-7 and the widened
// entry distance): the first SKW_TRAV_SCAP (8) of each thread in shared
// memory, deeper ones in local memory.  Its capacity CAP is chosen on the
// host as >= 2 * tree depth + 1, which bounds its use (at most two entries
// are pushed per level).
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <mutex>
#include <unordered_map>

#include "accel_build.h"
#include "kernels.h"

namespace skw {
namespace {

constexpr float kWiden = 8.0f * 5.9604645e-8f;  // 8 * 2^-24: slab interval widening
// Forward error bound of the float triangle test: with u = 2^-24, the edge
// and offset vectors carry <= u relative error, the cross products <= 4u of
// their magnitude sums, and det, n1, n2, nt <= 8u of the matching
// magnitude dot products (first order); 10u leaves room for the second-order
// terms and for the bounds being evaluated in float.
constexpr float kTriErr = 10.0f * 5.9604645e-8f;
constexpr double kDblEps = 2.220446049250313e-16;

// Launch shape: threads per block and the minimum resident blocks per SM
// that bounds the register budget (set by measurement; overridable at
// build time for sweeps).
#ifndef SKW_TRAV_BLOCK
#define SKW_TRAV_BLOCK 128
#endif
#ifndef SKW_TRAV_MINB
#define SKW_TRAV_MINB 10
#endif

enum : int { kMiss = 0, kHit = 1, kAmbiguous = 2 };

struct RayF {
  float ox, oy, oz, dx, dy, dz, tmin, tmax;
};

// Rays and results stream through once: with SKW_TRAV_STREAMING they are
// loaded and stored with the evict-first policy so that they do not push the
// tree out of L2.
// Measured slower (shared-memory latency on every triangle test outweighs
// the registers it frees): off by default.
#ifndef SKW_TRAV_RAYSMEM
#define SKW_TRAV_RAYSMEM 0
#endif
// Preferred shared-memory carveout in percent (cudaFuncAttribute
// PreferredSharedMemoryCarveout); negative leaves the driver's choice.
#ifndef SKW_TRAV_CARVEOUT
#define SKW_TRAV_CARVEOUT -1
#endif
#ifndef SKW_TRAV_STREAMING
#define SKW_TRAV_STREAMING 1
#endif
#if SKW_TRAV_STREAMING
#define SKW_LD_STREAM(p) __ldcs(p)
#define SKW_ST_STREAM(p, v) __stcs(p, v)
#else
#define SKW_LD_STREAM(p) __ldg(p)
#define SKW_ST_STREAM(p, v) (*(p) = (v))
#endif

__device__ __forceinline__ RayF load_ray(const float4 *__restrict__ rays, int64_t i) {
  const float4 a = SKW_LD_STREAM(rays + 2 * i);
  const float4 b = SKW_LD_STREAM(rays + 2 * i + 1);
  return RayF{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
}

// Float triangle test with a forward error bound.  Returns kMiss when the
// reference's double test certainly rejects (barycentrics or t < tmin),
// kHit when its barycentric tests and t >= tmin certainly pass (t and a bound
// et on |t - t_exact| are returned), else kAmbiguous.
__device__ __forceinline__ int tri_test32(const RayF &r, float3 v0, float3 v1, float3 v2, float &t, float &et) {
  t = __int_as_float(0x7fffffff);  // NaN until computed
  et = 0.0f;
  const float e1x = v1.x - v0.x, e1y = v1.y - v0.y, e1z = v1.z - v0.z;
  const float e2x = v2.x - v0.x, e2y = v2.y - v0.y, e2z = v2.z - v0.z;
  const float s1x = r.dy * e2z - r.dz * e2y;
  const float s1y = r.dz * e2x - r.dx * e2z;
  const float s1z = r.dx * e2y - r.dy * e2x;
  const float det = s1x * e1x + s1y * e1y + s1z * e1z;
  const float ddx = r.ox - v0.x, ddy = r.oy - v0.y, ddz = r.oz - v0.z;
  const float n1 = ddx * s1x + ddy * s1y + ddz * s1z;
  const float s2x = ddy * e1z - ddz * e1y;
  const float s2y = ddz * e1x - ddx * e1z;
  const float s2z = ddx * e1y - ddy * e1x;
  const float n2 = r.dx * s2x + r.dy * s2y + r.dz * s2z;
  const float nt = e2x * s2x + e2y * s2y + e2z * s2z;
  // Componentwise magnitude bounds of the cross products.
  const float adx = fabsf(r.dx), ady = fabsf(r.dy), adz = fabsf(r.dz);
  const float a2x = fabsf(e2x), a2y = fabsf(e2y), a2z = fabsf(e2z);
  const float a1x = fabsf(e1x), a1y = fabsf(e1y), a1z = fabsf(e1z);
  const float aox = fabsf(ddx), aoy = fabsf(ddy), aoz = fabsf(ddz);
  const float A1x = ady * a2z + adz * a2y, A1y = adz * a2x + adx * a2z, A1z = adx * a2y + ady * a2x;
  const float A2x = aoy * a1z + aoz * a1y, A2y = aoz * a1x + aox * a1z, A2z = aox * a1y + aoy * a1x;
  const float D = fabsf(det);
  const float edet = kTriErr * (a1x * A1x + a1y * A1y + a1z * A1z) + 1e-15f * D;
  const float en1 = kTriErr * (aox * A1x + aoy * A1y + aoz * A1z) + 1e-15f * D;
  const float en2 = kTriErr * (adx * A2x + ady * A2y + adz * A2z) + 1e-15f * D;
  const float ent = kTriErr * (a2x * A2x + a2y * A2y + a2z * A2z);
  if (!(D > 2.0f * edet)) return kAmbiguous;  // nearly parallel (or degenerate)
  const float sgn = det < 0.0f ? -1.0f : 1.0f;
  const float N1 = sgn * n1, N2 = sgn * n2, NT = sgn * nt;
  if (N1 + en1 < 0.0f || N2 + en2 < 0.0f) return kMiss;
  if (N1 - en1 > D + edet) return kMiss;
  if ((N1 + N2) - (en1 + en2) > D + edet) return kMiss;
  const float inv = 1.0f / D;
  t = NT * inv;
  et = (ent + fabsf(t) * edet) * inv * 1.0001f + fabsf(t) * 2.4e-7f + 1e-30f;
  if (t + et < r.tmin) return kMiss;
  if (N1 - en1 > 0.0f && N2 - en2 > 0.0f && (N1 + N2) + (en1 + en2) < D - edet && t - et >= r.tmin) return kHit;
  return kAmbiguous;
}

// A ray given in double (skw_ray_d): origin, direction, tmin, tmax.
struct RayD {
  double ox, oy, oz, dx, dy, dz, tmin, tmax;
};

__device__ __forceinline__ RayD load_ray_d(const float4 *__restrict__ rays, int64_t i) {
  const double2 *p = reinterpret_cast<const double2 *>(rays) + 4 * i;
  const double2 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2), d = __ldg(p + 3);
  return RayD{a.x, a.y, b.x, b.y, c.x, c.y, d.x, d.y};
}

// The reference's double-precision Moller-Trumbore test, operation by
// operation (TriangleAccelerator.cpp:240-273).  Intrinsics keep every
// product and sum separately rounded, as in the x86-64 SSE2 build.
__device__ __forceinline__ bool tri_test64v(double ox, double oy, double oz, double dx, double dy, double dz,
                                            float3 v0f, float3 v1f, float3 v2f, double tmin, double tmax,
                                            double &t_out) {
  const double v0x = v0f.x, v0y = v0f.y, v0z = v0f.z;
  const double e1x = __dsub_rn((double)v1f.x, v0x), e1y = __dsub_rn((double)v1f.y, v0y),
               e1z = __dsub_rn((double)v1f.z, v0z);
  const double e2x = __dsub_rn((double)v2f.x, v0x), e2y = __dsub_rn((double)v2f.y, v0y),
               e2z = __dsub_rn((double)v2f.z, v0z);
  const double s1x = __dsub_rn(__dmul_rn(dy, e2z), __dmul_rn(dz, e2y));
  const double s1y = __dsub_rn(__dmul_rn(dz, e2x), __dmul_rn(dx, e2z));
  const double s1z = __dsub_rn(__dmul_rn(dx, e2y), __dmul_rn(dy, e2x));
  const double divisor = __dadd_rn(__dadd_rn(__dmul_rn(s1x, e1x), __dmul_rn(s1y, e1y)), __dmul_rn(s1z, e1z));
  const double inv = __ddiv_rn(1.0, divisor);
  const double ddx = __dsub_rn(ox, v0x), ddy = __dsub_rn(oy, v0y), ddz = __dsub_rn(oz, v0z);
  const double b1 =
      __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(ddx, s1x), __dmul_rn(ddy, s1y)), __dmul_rn(ddz, s1z)), inv);
  if (b1 > -kDblEps && b1 < (1.0 + kDblEps)) {
    const double s2x = __dsub_rn(__dmul_rn(ddy, e1z), __dmul_rn(ddz, e1y));
    const double s2y = __dsub_rn(__dmul_rn(ddz, e1x), __dmul_rn(ddx, e1z));
    const double s2z = __dsub_rn(__dmul_rn(ddx, e1y), __dmul_rn(ddy, e1x));
    const double b2 =
        __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(dx, s2x), __dmul_rn(dy, s2y)), __dmul_rn(dz, s2z)), inv);
    if (b2 > -kDblEps && __dadd_rn(b1, b2) < (1.0 + kDblEps)) {
      const double t =
          __dmul_rn(__dadd_rn(__dadd_rn(__dmul_rn(e2x, s2x), __dmul_rn(e2y, s2y)), __dmul_rn(e2z, s2z)), inv);
      if (t >= tmin && t <= tmax) {
        t_out = t;
        return true;
      }
    }
  }
  return false;
}

// The same test for a float ray widened exactly to double.
__device__ __forceinline__ bool tri_test64(const RayF &r, float3 v0f, float3 v1f, float3 v2f, double tmin, double tmax,
                                        double &t_out) {
  return tri_test64v(r.ox, r.oy, r.oz, r.dx, r.dy, r.dz, v0f, v1f, v2f, tmin, tmax, t_out);
}

__device__ __forceinline__ void load_tri(const float4 *__restrict__ tris, uint32_t slot, float3 &v0, float3 &v1,
                                         float3 &v2, int &prim, int &tri) {
  const float4 a = __ldg(tris + 3 * slot);
  const float4 b = __ldg(tris + 3 * slot + 1);
  const float4 c = __ldg(tris + 3 * slot + 2);
  v0 = make_float3(a.x, a.y, a.z);
  v1 = make_float3(b.x, b.y, b.z);
  v2 = make_float3(c.x, c.y, c.z);
  prim = __float_as_int(a.w);
  tri = __float_as_int(b.w);
}

// Per-ray data for the slab test.  A plane distance is computed as
// fma(coordinate, 1/d, offset) with the offset -o/d -+ w folded in, where the
// per-axis widening w = 6u (B + |o|) |1/d| (u = 2^-24, B = largest absolute
// coordinate in the scene) bounds the float result's distance from the exact
// value for every node of the scene; the reference's double result is within
// a far smaller distance of the exact one.  The near plane of each axis is
// selected by the sign of 1/d, which is the reference's "swap if
// tNear > tFar" for every non-NaN slab.  Together with tmin, tmax and the
// near-child side of each axis this is all the node walk needs, so the
// ray's origin and direction can stay out of registers while it runs.
struct SlabRay {
  float ix, iy, iz;  // 1/d
  float nx, ny, nz;  // near-plane offsets: -o/d - w
  float fx, fy, fz;  // far-plane offsets:  -o/d + w
  float tmin, tmax;
  // bits 0-2: !(d[axis] > 0), the reference pops the right child first;
  // bits 3-5: 1/d[axis] < 0, the near plane is the box maximum
  uint32_t bits;
};

// widen_u: the widening in units of u -- 6 for a float ray; 9 for a double
// ray rounded to float, whose rounding moves a plane distance by at most
// u |o| |1/d| (origin) + u |b - o| |1/d| (direction) more.
__device__ __forceinline__ SlabRay make_slab_ray(const RayF &r, float scene_abs, float widen_u = 6.0f) {
  SlabRay s;
  s.ix = 1.0f / r.dx;
  s.iy = 1.0f / r.dy;
  s.iz = 1.0f / r.dz;
  const float c = widen_u * 5.9604645e-8f;
  const float wx = c * (scene_abs + fabsf(r.ox)) * fabsf(s.ix);
  const float wy = c * (scene_abs + fabsf(r.oy)) * fabsf(s.iy);
  const float wz = c * (scene_abs + fabsf(r.oz)) * fabsf(s.iz);
  const float ox = -r.ox * s.ix, oy = -r.oy * s.iy, oz = -r.oz * s.iz;
  s.nx = ox - wx;
  s.ny = oy - wy;
  s.nz = oz - wz;
  s.fx = ox + wx;
  s.fy = oy + wy;
  s.fz = oz + wz;
  s.tmin = r.tmin;
  s.tmax = r.tmax;
  s.bits = (r.dx > 0.0f ? 0u : 1u) | (r.dy > 0.0f ? 0u : 2u) | (r.dz > 0.0f ? 0u : 4u) |
           (signbit(s.ix) ? 8u : 0u) | (signbit(s.iy) ? 16u : 0u) | (signbit(s.iz) ? 32u : 0u);
  return s;
}

// The reference's slab test (TriangleAccelerator.cpp:176-192) on the widened
// interval: true when the node must be visited.  `lo` receives the widened
// entry distance max(tnear_x, tnear_y, tnear_z, tmin), all that a later
// re-test against a smaller tmax needs.  fmaxf/fminf drop NaN operands
// (0 * inf slabs), as the reference's comparisons are all false on NaN.
#ifndef SKW_TRAV_MAX3
#define SKW_TRAV_MAX3 0
#endif
#if SKW_TRAV_MAX3
// Three-input max / min (sm_100+): a NaN operand is dropped, as by fmaxf /
// fminf.
__device__ __forceinline__ float max3f(float a, float b, float c) {
  float d;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
  float d;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}
#endif

__device__ __forceinline__ bool node_visit(const float4 na, const float4 nb, const SlabRay &s, float tcull,
                                           float &lo) {
  const bool sx = s.bits & 8u, sy = s.bits & 16u, sz = s.bits & 32u;
  const float tn0 = fmaf(sx ? na.w : na.x, s.ix, s.nx), tf0 = fmaf(sx ? na.x : na.w, s.ix, s.fx);
  const float tn1 = fmaf(sy ? nb.x : na.y, s.iy, s.ny), tf1 = fmaf(sy ? na.y : nb.x, s.iy, s.fy);
  const float tn2 = fmaf(sz ? nb.y : na.z, s.iz, s.nz), tf2 = fmaf(sz ? na.z : nb.y, s.iz, s.fz);
#if SKW_TRAV_MAX3
  lo = max3f(tn0, tn1, fmaxf(tn2, s.tmin));
  const float hi = min3f(tf0, tf1, fminf(tf2, tcull));
#else
  lo = fmaxf(fmaxf(tn0, tn1), fmaxf(tn2, s.tmin));
  const float hi = fminf(fminf(tf0, tf1), fminf(tf2, tcull));
#endif
  return !(lo > hi);
}

#ifndef SKW_TRAV_SCAP
#define SKW_TRAV_SCAP 8
#endif
#ifndef SKW_TRAV_REFILL
#define SKW_TRAV_REFILL 8
#endif
// A walk round ends once at most SKW_TRAV_LAG walking lanes still have no
// leaf; those keep their place and go on walking in the next round.
#ifndef SKW_TRAV_LAG
#define SKW_TRAV_LAG 12
#endif
// Postponed leaves (speculative node steps), see k_trace.
#ifndef SKW_TRAV_POSTPONE
#define SKW_TRAV_POSTPONE 1
#endif

// Traversal stack: the first SCAP entries of each thread live in shared
// memory as three word arrays indexed [entry][thread] (so lanes never
// conflict on a bank), deeper entries in local memory.  An entry holds a
// node's words 6-7 and its widened entry distance.
#ifndef SKW_TRAV_STACK8
#define SKW_TRAV_STACK8 0
#endif
// Any-hit walks recompute the slab data (12 words) from the ray at the
// start of every walk round instead of holding it through the triangle
// tests (measured: 1,439 -> 1,488 Mrays/s on uniform rays over 1.1M
// triangles); closest-hit walks keep it (there the recomputation measured
// 2 % slower).  SKW_TRAV_SLAB_ROUND: 0 never, 1 any-hit only, 2 both.
#ifndef SKW_TRAV_SLAB_ROUND
#define SKW_TRAV_SLAB_ROUND 1
#endif

template <int CAP>
struct Stack {
  static constexpr int SCAP = CAP < SKW_TRAV_SCAP ? CAP : SKW_TRAV_SCAP;
#if SKW_TRAV_STACK8
  // Entries are (node index, widened entry distance); a popped node's words
  // are read back from the tree (a recent, L1-resident line).
  uint32_t (*sa)[SKW_TRAV_BLOCK];
  float (*slo)[SKW_TRAV_BLOCK];
  uint2 ovf[CAP - SCAP > 0 ? CAP - SCAP : 1];
  const float4 *nodes;
  int sp;

  __device__ __forceinline__ void push(uint32_t, uint32_t, float lo, uint32_t slot) {
    if (sp < SCAP) {
      sa[sp][threadIdx.x] = slot;
      slo[sp][threadIdx.x] = lo;
    } else {
      ovf[sp - SCAP] = make_uint2(slot, __float_as_uint(lo));
    }
    ++sp;
  }
  __device__ __forceinline__ bool pop(float tcull, uint32_t &a, uint32_t &b) {
    float lo;
    return pop(tcull, a, b, lo);
  }
  __device__ __forceinline__ bool pop(float tcull, uint32_t &a, uint32_t &b, float &lo) {
    while (sp > 0) {
      --sp;
      uint32_t slot;
      if (sp < SCAP) {
        lo = slo[sp][threadIdx.x];
        slot = sa[sp][threadIdx.x];
      } else {
        const uint2 e = ovf[sp - SCAP];
        slot = e.x;
        lo = __uint_as_float(e.y);
      }
      if (!(lo > tcull)) {
        const float4 nb = __ldg(nodes + 2 * slot + 1);
        a = __float_as_uint(nb.z);
        b = __float_as_uint(nb.w);
        return true;
      }
    }
    return false;
  }
#else
  uint32_t (*sa)[SKW_TRAV_BLOCK];
  uint32_t (*sb)[SKW_TRAV_BLOCK];
  float (*slo)[SKW_TRAV_BLOCK];
  uint4 ovf[CAP - SCAP > 0 ? CAP - SCAP : 1];
  int sp;

  __device__ __forceinline__ void push(uint32_t a, uint32_t b, float lo, uint32_t) {
    if (sp < SCAP) {
      sa[sp][threadIdx.x] = a;
      sb[sp][threadIdx.x] = b;
      slo[sp][threadIdx.x] = lo;
    } else {
      ovf[sp - SCAP] = make_uint4(a, b, __float_as_uint(lo), 0u);
    }
    ++sp;
  }
  // Pops until an entry survives the re-cull against tcull (the reference
  // culls the others when it pops them).
  __device__ __forceinline__ bool pop(float tcull, uint32_t &a, uint32_t &b) {
    float lo;
    return pop(tcull, a, b, lo);
  }
  __device__ __forceinline__ bool pop(float tcull, uint32_t &a, uint32_t &b, float &lo) {
    while (sp > 0) {
      --sp;
      if (sp < SCAP) {
        lo = slo[sp][threadIdx.x];
        a = sa[sp][threadIdx.x];
        b = sb[sp][threadIdx.x];
      } else {
        const uint4 e = ovf[sp - SCAP];
        a = e.x;
        b = e.y;
        lo = __uint_as_float(e.z);
      }
      if (!(lo > tcull)) return true;
    }
    return false;
  }
#endif
};

// Expands internal nodes until (cur_a, cur_b) is a leaf; false when the
// stack runs out.
//
// Visit order equals the reference's (TriangleAccelerator.cpp:170-211): the
// reference pushes an internal node's children and pops the near-side one
// first, testing each node's box when it is popped.  Here an internal node's
// present children (contiguous, so their loads go out together) are
// box-tested right away; the first passing one in the reference's pop order
// becomes the current node and the rest are pushed so that they pop in that
// order.  A pushed entry keeps its widened entry distance and is re-culled on
// pop against the tmax of that moment -- the only part of the reference's
// pop-time test that can change after the push, since tmax only shrinks.
template <int CAP>
__device__ __forceinline__ bool descend(const float4 *__restrict__ nodes, const SlabRay &s,
                                        float tcull, Stack<CAP> &st, uint32_t &cur_a, uint32_t &cur_b,
                                        unsigned *status) {
  while ((cur_b & 3u) != 0u) {
    const uint32_t type = cur_b & 3u, mask = (cur_b >> 2) & 7u;
    const uint32_t sL = cur_a, sM = cur_a + (mask & 1u), sR = sM + ((mask >> 1) & 1u);
    const bool near_right = (s.bits >> (type - 1u)) & 1u;  // the reference pops left first when d[axis] > 0
    uint32_t slot[3], present[3];
    slot[0] = near_right ? sR : sL;
    present[0] = near_right ? (mask & 4u) : (mask & 1u);
    slot[1] = sM;
    present[1] = mask & 2u;
    slot[2] = near_right ? sL : sR;
    present[2] = near_right ? (mask & 1u) : (mask & 4u);
    bool pass[3];
    float lo[3];
    uint32_t wa[3], wb[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      pass[k] = false;
      wa[k] = wb[k] = 0u;
      lo[k] = 0.0f;
      if (present[k]) {
        const float4 ca = __ldg(nodes + 2 * slot[k]);
        const float4 cb = __ldg(nodes + 2 * slot[k] + 1);
        pass[k] = node_visit(ca, cb, s, tcull, lo[k]);
        wa[k] = __float_as_uint(cb.z);
        wb[k] = __float_as_uint(cb.w);
      }
    }
    const int first = pass[0] ? 0 : (pass[1] ? 1 : (pass[2] ? 2 : -1));
    if (st.sp + 2 > CAP) {
      atomicOr(status, 1u);
      return false;
    }
    if (pass[2] && first != 2) st.push(wa[2], wb[2], lo[2], slot[2]);
    if (pass[1] && first != 1) st.push(wa[1], wb[1], lo[1], slot[1]);
    if (first < 0) {
      if (!st.pop(tcull, cur_a, cur_b)) return false;
      continue;
    }
    cur_a = first == 0 ? wa[0] : (first == 1 ? wa[1] : wa[2]);
    cur_b = first == 0 ? wb[0] : (first == 1 ? wb[1] : wb[2]);
  }
  return true;
}

// One internal-node step of descend(): box-tests the present children of
// (cur_a, cur_b), makes the first passing one (in the reference's pop order)
// current and pushes the others; pops when none passes.  cur_lo tracks the
// current node's widened entry distance.  False when the stack runs out.
template <int CAP>
__device__ __forceinline__ bool step_internal(const float4 *__restrict__ nodes, const SlabRay &s,
                                              float tcull, Stack<CAP> &st, uint32_t &cur_a, uint32_t &cur_b,
                                              float &cur_lo, unsigned *status) {
  const uint32_t type = cur_b & 3u, mask = (cur_b >> 2) & 7u;
  const uint32_t sL = cur_a, sM = cur_a + (mask & 1u), sR = sM + ((mask >> 1) & 1u);
  const bool near_right = (s.bits >> (type - 1u)) & 1u;
  uint32_t slot[3], present[3];
  slot[0] = near_right ? sR : sL;
  present[0] = near_right ? (mask & 4u) : (mask & 1u);
  slot[1] = sM;
  present[1] = mask & 2u;
  slot[2] = near_right ? sL : sR;
  present[2] = near_right ? (mask & 1u) : (mask & 4u);
  bool pass[3];
  float lo[3];
  uint32_t wa[3], wb[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    pass[k] = false;
    wa[k] = wb[k] = 0u;
    lo[k] = 0.0f;
    if (present[k]) {
      const float4 ca = __ldg(nodes + 2 * slot[k]);
      const float4 cb = __ldg(nodes + 2 * slot[k] + 1);
      pass[k] = node_visit(ca, cb, s, tcull, lo[k]);
      wa[k] = __float_as_uint(cb.z);
      wb[k] = __float_as_uint(cb.w);
    }
  }
  const int first = pass[0] ? 0 : (pass[1] ? 1 : (pass[2] ? 2 : -1));
  if (st.sp + 2 > CAP) {
    atomicOr(status, 1u);
    return false;
  }
  if (pass[2] && first != 2) st.push(wa[2], wb[2], lo[2], slot[2]);
  if (pass[1] && first != 1) st.push(wa[1], wb[1], lo[1], slot[1]);
  if (first < 0) return st.pop(tcull, cur_a, cur_b, cur_lo);
  cur_a = first == 0 ? wa[0] : (first == 1 ? wa[1] : wa[2]);
  cur_b = first == 0 ? wb[0] : (first == 1 ? wb[1] : wb[2]);
  cur_lo = first == 0 ? lo[0] : (first == 1 ? lo[1] : lo[2]);
  return true;
}

// Exact double-precision t of the hit on slot `slot` (its barycentric tests
// are known to pass).
__device__ __forceinline__ double exact_t(const float4 *__restrict__ tris, const RayF &r, int slot, float fallback) {
  const float4 a = __ldg(tris + 3 * slot), b = __ldg(tris + 3 * slot + 1), c = __ldg(tris + 3 * slot + 2);
  double t;
  return tri_test64(r, make_float3(a.x, a.y, a.z), make_float3(b.x, b.y, b.z), make_float3(c.x, c.y, c.z),
                    (double)r.tmin, 1.0e308, t)
             ? t
             : (double)fallback;
}

template <bool CLOSEST>
__device__ __forceinline__ void store_result(void *__restrict__ out, const int32_t *__restrict__ out_index, int ray_i,
                                             int4 h, bool hit) {
  const int o = out_index ? SKW_LD_STREAM(out_index + ray_i) : ray_i;
  if (CLOSEST) {
    SKW_ST_STREAM((int4 *)out + o, h);
  } else {
    ((uint8_t *)out)[o] = hit ? 1 : 0;
  }
}

// Persistent traversal.  The rays form groups of 32 consecutive rays; a warp
// takes the launch's next group from the launch's counter (`work`, one
// atomicAdd per group) when its current group is used up, or, without a
// counter, warp w of W owns groups w, w + W, w + 2W, ...  A lane whose ray
// is finished takes the next ray of the warp's group when at least
// SKW_TRAV_REFILL lanes are idle (or all are), so lanes rarely idle while
// long rays finish.  No cross-warp waits.
//
// Closest-hit state is kept small: the slot of the current best hit and a
// float interval [lo_t, hi_t] that contains the reference's current tmax
// (the best hit's double t).  Where a decision needs that tmax exactly, it is
// recomputed from the slot with the exact test.
//
// surf: the rays leave surfaces with tmin from next_min_t (the renders'
// shadow, BSDF, specular and gather rays, photon bounces).
//
// DRAY: the rays are skw_ray_d (double).  The walk runs on the ray rounded
// to float (origin and direction to nearest, tmin down, tmax up) with the
// slab widening of make_slab_ray for rounded rays, so a node is still
// culled only if the reference culls it; every triangle of a reached leaf
// is tested with the reference's double arithmetic on the double ray
// (reloaded from memory for the leaf), and the current tmax is kept as the
// exact double t of the best hit.  Closest-hit results are skw_hit_d
// (double t, prim, tri).
template <int CAP, bool CLOSEST, bool DRAY>
__global__ void __launch_bounds__(SKW_TRAV_BLOCK, SKW_TRAV_MINB)
    k_trace(const float4 *__restrict__ nodes, const float4 *__restrict__ tris, const float4 *__restrict__ rays,
            int n, const int *__restrict__ n_dev, float scene_abs, const int32_t *__restrict__ out_index,
            void *__restrict__ out, unsigned *__restrict__ status, int *__restrict__ work, int surf,
            unsigned long long *__restrict__ traced) {
  static_assert(!DRAY || SKW_TRAV_POSTPONE, "double rays use the postponed-leaf walk");
  if (n_dev) n = min(n, *n_dev);  // a queue whose length lives on the device
  if (traced && blockIdx.x == 0 && threadIdx.x == 0 && n > 0) atomicAdd(traced, (unsigned long long)n);
  constexpr int SCAP = Stack<CAP>::SCAP;
  __shared__ uint32_t s_a[SCAP][SKW_TRAV_BLOCK];
  __shared__ float s_lo[SCAP][SKW_TRAV_BLOCK];
  Stack<CAP> st;
  st.sa = s_a;
  st.slo = s_lo;
#if SKW_TRAV_STACK8
  st.nodes = nodes;
#else
  __shared__ uint32_t s_b[SCAP][SKW_TRAV_BLOCK];
  st.sb = s_b;
#endif
  st.sp = 0;

  const unsigned lane = threadIdx.x & 31u;
  const int warp = (int)((blockIdx.x * (unsigned)SKW_TRAV_BLOCK + threadIdx.x) >> 5);
  const int n_warps = (int)(gridDim.x * (unsigned)(SKW_TRAV_BLOCK / 32));
  const int groups = (n + 31) >> 5;
  // Rays come in groups of 32.  Static (work == null): warp w takes groups
  // w, w + W, ...; next / end are positions in that sequence.  Dynamic: a
  // warp whose group is used up takes the launch's next group from the
  // counter *work (zero at launch), so warps that drew cheap rays take more
  // and the launch's tail is one group long; next / end are positions in
  // the current group [gbase, gbase + 32), end = -1 once the rays are gone.
  int next = 0;
  int end = work ? 0 : (warp < groups ? ((groups - warp + n_warps - 1) / n_warps) << 5 : 0);
  int gbase = 0;

  int ray_i = -1;
  // The ray itself is read only by the triangle tests: with
  // SKW_TRAV_RAYSMEM it waits in shared memory (one word array per field,
  // [field][thread], conflict-free) instead of holding eight registers
  // through the node walk.
#if SKW_TRAV_RAYSMEM
  __shared__ float s_ray[8][SKW_TRAV_BLOCK];
#define SKW_RAY()                                                                                          \
  RayF {                                                                                                   \
    s_ray[0][threadIdx.x], s_ray[1][threadIdx.x], s_ray[2][threadIdx.x], s_ray[3][threadIdx.x],            \
        s_ray[4][threadIdx.x], s_ray[5][threadIdx.x], s_ray[6][threadIdx.x], s_ray[7][threadIdx.x]        \
  }
#else
  RayF r_reg{};
#define SKW_RAY() r_reg
#endif
  constexpr bool kSlabRound = SKW_TRAV_SLAB_ROUND == 2 || (SKW_TRAV_SLAB_ROUND == 1 && !CLOSEST);
  SlabRay s_keep{};  // the walk's slab data when it is kept across rounds
  uint32_t cur_a = 0, cur_b = 0;
  int best_slot = -1;
  double best_t = 0.0;             // DRAY: the exact t of the best hit
  float lo_t = 0.0f, hi_t = 0.0f;  // bracket of the reference's current tmax
  uint32_t flags = 0;              // SKW_HIT_* bits; bit 3: [lo_t, hi_t] brackets an exact double
#if SKW_TRAV_POSTPONE
  bool trav = false, has_post = false;  // traversal not finished; a leaf is postponed
  uint32_t post_a = 0, post_cnt = 0;
  float cur_lo = 0.0f;
#endif

  while (true) {
    const unsigned idle = __ballot_sync(0xffffffffu, ray_i < 0);
    if (idle != 0u && (__popc(idle) >= SKW_TRAV_REFILL || idle == 0xffffffffu) && work && end >= 0 && next >= end) {
      int base = 0;
      if (lane == 0) base = atomicAdd(work, 32);
      base = __shfl_sync(0xffffffffu, base, 0);
      gbase = base;
      next = 0;
      end = base < n ? min(32, n - base) : -1;
    }
    if (idle != 0u && next < end && (__popc(idle) >= SKW_TRAV_REFILL || idle == 0xffffffffu)) {
      const int mine = next + __popc(idle & ((1u << lane) - 1u));
      next += __popc(idle);
      const int idx = work ? gbase + mine : ((warp + (mine >> 5) * n_warps) << 5) + (mine & 31);
      if (ray_i < 0 && mine < end && idx < n) {
        ray_i = idx;
        RayF rl;
        if (DRAY) {
          const RayD rd = load_ray_d(rays, ray_i);
          rl = RayF{(float)rd.ox, (float)rd.oy, (float)rd.oz, (float)rd.dx, (float)rd.dy, (float)rd.dz,
                    __double2float_rd(rd.tmin), __double2float_ru(rd.tmax)};
        } else {
          rl = load_ray(rays, ray_i);
        }
#if SKW_TRAV_RAYSMEM
        s_ray[0][threadIdx.x] = rl.ox;
        s_ray[1][threadIdx.x] = rl.oy;
        s_ray[2][threadIdx.x] = rl.oz;
        s_ray[3][threadIdx.x] = rl.dx;
        s_ray[4][threadIdx.x] = rl.dy;
        s_ray[5][threadIdx.x] = rl.dz;
        s_ray[6][threadIdx.x] = rl.tmin;
        s_ray[7][threadIdx.x] = rl.tmax;
#else
        r_reg = rl;
#endif
        const SlabRay s = make_slab_ray(rl, scene_abs, DRAY ? 9.0f : 6.0f);
        if (!kSlabRound) s_keep = s;
        best_slot = -1;
        lo_t = hi_t = rl.tmax;
        flags = 8u;
        st.sp = 0;
        const float4 na = __ldg(nodes), nb = __ldg(nodes + 1);
        float lo;
        cur_a = __float_as_uint(nb.z);
        cur_b = __float_as_uint(nb.w);
        if (!node_visit(na, nb, s, rl.tmax, lo)) {  // root culled: a miss
          if (DRAY && CLOSEST) {
            ((int4 *)out)[out_index ? out_index[ray_i] : ray_i] = make_int4(0, 0x7ff00000, -1, -1);
          } else {
            store_result<CLOSEST>(out, out_index, ray_i, make_int4(0x7f800000, -1, -1, 0), false);
          }
          ray_i = -1;
        }
#if SKW_TRAV_POSTPONE
        trav = true;
        has_post = false;
        cur_lo = lo;
#endif
      }
    }
    const unsigned busy = __ballot_sync(0xffffffffu, ray_i >= 0);
    if (busy == 0u) {
      if (next >= end && (!work || end < 0)) break;
      continue;
    }
    if (ray_i < 0) continue;
    // Independent thread scheduling does not promise that the busy lanes run
    // the rest of the iteration as one group; without an explicit sync they
    // were measured to split into 2-3 groups that each walked on their own.
    __syncwarp(busy);
    const SlabRay s = kSlabRound ? make_slab_ray(SKW_RAY(), scene_abs, DRAY ? 9.0f : 6.0f) : s_keep;

#if SKW_TRAV_POSTPONE
    // Node steps continue past a lane's first leaf (postponed) until all but
    // SKW_TRAV_LAG walking lanes hold one, or the lane reaches a second leaf;
    // the leaves are then tested in the order they were reached, which is
    // the reference's order.  (Waiting for the last few lanes to find a leaf
    // left most of the warp idle: with 32 lanes the round length is the
    // slowest lane's.)  Nodes stepped through before the postponed leaf
    // is tested see a larger tmax than the reference's -- a superset of its
    // visits, whose extra triangles all lie beyond the final tmax.
    //
    // Every busy lane is walking when the round starts (a busy lane whose
    // walk had ended would have finished its ray).  All of them stay in the
    // loop -- a lane that is done idles -- and vote on every step over the
    // busy mask, so they stay one group (a vote over __activemask() would
    // only cover whatever fragment happens to be running together) and one
    // vote per step suffices.
    const float tcull = CLOSEST ? hi_t : s.tmax;
    bool walking = trav;
    while (true) {
      if (walking) {
        bool stop = false;
        if ((cur_b & 3u) == 0u) {  // a leaf
          if (has_post) {
            stop = true;  // a second leaf: it waits for the next round
          } else {
            if (!(cur_lo > tcull)) {
              post_a = cur_a;
              post_cnt = cur_b >> 8;
              has_post = true;
            }
            trav = st.pop(tcull, cur_a, cur_b, cur_lo);
          }
        } else {
          trav = step_internal(nodes, s, tcull, st, cur_a, cur_b, cur_lo, status);
        }
        walking = trav && !stop;
      }
      if (__popc(__ballot_sync(busy, walking && !has_post)) <= SKW_TRAV_LAG) break;
    }
    __syncwarp(busy);
    bool hit = false;
    if (DRAY && has_post) {
      // every triangle of the leaf in the reference's double arithmetic
      has_post = false;
      const RayD rd = load_ray_d(rays, ray_i);
      for (uint32_t k = 0; k < post_cnt; ++k) {
        const int slot = (int)(post_a + k);
        float3 v0, v1, v2;
        int prim, tri;
        load_tri(tris, (uint32_t)slot, v0, v1, v2, prim, tri);
        double t64;
        if (tri_test64v(rd.ox, rd.oy, rd.oz, rd.dx, rd.dy, rd.dz, v0, v1, v2, rd.tmin,
                        CLOSEST && best_slot >= 0 ? best_t : rd.tmax, t64)) {
          if (!CLOSEST) {
            hit = true;
            break;
          }
          if (best_slot >= 0 && fabs(t64 - best_t) <= 1e-12 * fabs(t64)) flags |= 2u;
          best_slot = slot;
          best_t = t64;
          lo_t = __double2float_rd(t64);
          hi_t = __double2float_ru(t64);
        }
      }
    }
    if (!DRAY && has_post) {
      has_post = false;
      const RayF r = SKW_RAY();
      const uint32_t a = post_a, cnt = post_cnt;
      for (uint32_t k = 0; k < cnt; ++k) {
        const int slot = (int)(a + k);
        float3 v0, v1, v2;
        int prim, tri;
        load_tri(tris, (uint32_t)slot, v0, v1, v2, prim, tri);
        float t, et;
        int res = tri_test32(r, v0, v1, v2, t, et);
        if (res == kMiss) continue;
        // A ray leaving a surface (surf) starts at an upper bound of the
        // reference's GetNextMinT: a triangle whose t cannot be told apart
        // from that tmin in float lies on the ray's own plane crossing --
        // the triangle it leaves, or geometry touching it there -- and is
        // skipped, as the reference's tmin skips the triangle it leaves.
        if (surf && res == kAmbiguous && t - et < r.tmin) continue;
        if (CLOSEST) {
          if (res == kHit) {
            if (__fsub_rd(t, et) > hi_t) continue;  // certainly beyond the current tmax
            if (__fadd_ru(t, et) < lo_t) {          // certainly nearer: accept in float
              best_slot = slot;
              lo_t = __fsub_rd(t, et);
              hi_t = __fadd_ru(t, et);
              flags &= ~8u;
              continue;
            }
          }
          // Exact re-test against the reference's exact current tmax.
          const double cur_max = best_slot < 0 ? (double)r.tmax : exact_t(tris, r, best_slot, hi_t);
          double t64;
          if (tri_test64(r, v0, v1, v2, (double)r.tmin, cur_max, t64)) {
            if (best_slot >= 0 && fabs(t64 - cur_max) <= 1e-12 * fabs(t64)) flags |= 2u;
            best_slot = slot;
            lo_t = __double2float_rd(t64);
            hi_t = __double2float_ru(t64);
            flags |= 1u | 8u;
          }
        } else {
          if (res == kHit) {
            if (t + et < r.tmax) {
              hit = true;
              break;
            }
            if (t - et > r.tmax) continue;
          }
          double t64;
          if (tri_test64(r, v0, v1, v2, (double)r.tmin, (double)r.tmax, t64)) {
            hit = true;
            break;
          }
        }
      }
    }
    bool done = hit || (!trav && !has_post);
#else
    const float tcull = CLOSEST ? hi_t : s.tmax;
    bool done = !descend(nodes, s, tcull, st, cur_a, cur_b, status);
    bool hit = false;
    if (!done) {
      const RayF r = SKW_RAY();
      // cur is a leaf: test its triangles in order.
      const uint32_t a = cur_a, cnt = cur_b >> 8;
      for (uint32_t k = 0; k < cnt; ++k) {
        const int slot = (int)(a + k);
        float3 v0, v1, v2;
        int prim, tri;
        load_tri(tris, (uint32_t)slot, v0, v1, v2, prim, tri);
        float t, et;
        int res = tri_test32(r, v0, v1, v2, t, et);
        if (res == kMiss) continue;
        // A ray leaving a surface (surf) starts at an upper bound of the
        // reference's GetNextMinT: a triangle whose t cannot be told apart
        // from that tmin in float lies on the ray's own plane crossing --
        // the triangle it leaves, or geometry touching it there -- and is
        // skipped, as the reference's tmin skips the triangle it leaves.
        if (surf && res == kAmbiguous && t - et < r.tmin) continue;
        if (CLOSEST) {
          if (res == kHit) {
            if (__fsub_rd(t, et) > hi_t) continue;  // certainly beyond the current tmax
            if (__fadd_ru(t, et) < lo_t) {          // certainly nearer: accept in float
              best_slot = slot;
              lo_t = __fsub_rd(t, et);
              hi_t = __fadd_ru(t, et);
              flags &= ~8u;
              continue;
            }
          }
          // Exact re-test against the reference's exact current tmax.
          const double cur_max = best_slot < 0 ? (double)r.tmax : exact_t(tris, r, best_slot, hi_t);
          double t64;
          if (tri_test64(r, v0, v1, v2, (double)r.tmin, cur_max, t64)) {
            if (best_slot >= 0 && fabs(t64 - cur_max) <= 1e-12 * fabs(t64)) flags |= 2u;
            best_slot = slot;
            lo_t = __double2float_rd(t64);
            hi_t = __double2float_ru(t64);
            flags |= 1u | 8u;
          }
        } else {
          if (res == kHit) {
            if (t + et < r.tmax) {
              hit = true;
              break;
            }
            if (t - et > r.tmax) continue;
          }
          double t64;
          if (tri_test64(r, v0, v1, v2, (double)r.tmin, (double)r.tmax, t64)) {
            hit = true;
            break;
          }
        }
      }
      done = hit || !st.pop(CLOSEST ? hi_t : s.tmax, cur_a, cur_b);
    }
#endif
    if (DRAY && done) {
      if (CLOSEST) {
        int4 h = make_int4(0, 0x7ff00000, -1, -1);  // t = +inf, a miss
        if (best_slot >= 0) {
          const float4 ta = __ldg(tris + 3 * best_slot), tb = __ldg(tris + 3 * best_slot + 1);
          const long long tb64 = __double_as_longlong(best_t);
          h = make_int4((int)(tb64 & 0xffffffffll), (int)(tb64 >> 32), __float_as_int(ta.w), __float_as_int(tb.w));
        }
        ((int4 *)out)[out_index ? out_index[ray_i] : ray_i] = h;
      } else {
        store_result<CLOSEST>(out, out_index, ray_i, int4{}, hit);
      }
      ray_i = -1;
    } else if (done) {
      int4 h = make_int4(0x7f800000, -1, -1, (int)(flags & 7u));
      if (CLOSEST && best_slot >= 0) {
        const float4 ta = __ldg(tris + 3 * best_slot), tb = __ldg(tris + 3 * best_slot + 1);
        float tout = 0.5f * lo_t + 0.5f * hi_t;
        // A float-decided hit whose bracket is wider than the 1e-5 reporting
        // tolerance (grazing incidence) takes t from the exact test.
        if (!(flags & 8u) && hi_t - lo_t > 1.0e-5f * fabsf(tout)) {
          tout = (float)exact_t(tris, SKW_RAY(), best_slot, tout);
          flags |= 4u;
        }
        h = make_int4(__float_as_int(tout), __float_as_int(ta.w), __float_as_int(tb.w), (int)(flags & 7u));
      }
      store_result<CLOSEST>(out, out_index, ray_i, h, hit);
      ray_i = -1;
    }
  }
}

// --------------------------------------------------------------------------
// Accelerators with instances (meshes shared by several primitives) are
// traversed by k_trace_inst: one ray per thread, the reference's
// _NodeIntersect / _NodeIntersectTest restated in double throughout
// (TriangleAccelerator.cpp:154-293, 354-462) -- the slab test of every
// node, the children pushed in the reference's order, at a leaf first its
// instances (the ray taken to mesh space by the instance's world-to-mesh
// Transform, TriangleAccelerator.cpp:213-233, and the instance's subtree
// traversed with it) and then its triangles, all with the reference's
// double Moller-Trumbore.  Exact but slow: instanced scenes are rare and
// the float walk of k_trace does not apply to rays in mesh space.

struct InstDev {
  double m[16];  // world to mesh, row-major
  uint32_t root;
  int32_t prim;
  uint32_t pad[2];
};

// Transform::operator() on a point (with the w division) and a vector
// (Math/Transform.h:239-269), every sum and product rounded separately.
__device__ __forceinline__ void xf_point(const double *m, double x, double y, double z, double *o) {
  const double xp = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(m[0], x), __dmul_rn(m[1], y)), __dmul_rn(m[2], z)), m[3]);
  const double yp = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(m[4], x), __dmul_rn(m[5], y)), __dmul_rn(m[6], z)), m[7]);
  const double zp = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(m[8], x), __dmul_rn(m[9], y)), __dmul_rn(m[10], z)), m[11]);
  const double w = __dadd_rn(__dadd_rn(__dadd_rn(__dmul_rn(m[12], x), __dmul_rn(m[13], y)), __dmul_rn(m[14], z)), m[15]);
  o[0] = xp;
  o[1] = yp;
  o[2] = zp;
  if (w != 1.0) {
    const double inv = __ddiv_rn(1.0, w);
    o[0] = __dmul_rn(xp, inv);
    o[1] = __dmul_rn(yp, inv);
    o[2] = __dmul_rn(zp, inv);
  }
}
__device__ __forceinline__ void xf_vector(const double *m, double x, double y, double z, double *o) {
  o[0] = __dadd_rn(__dadd_rn(__dmul_rn(m[0], x), __dmul_rn(m[1], y)), __dmul_rn(m[2], z));
  o[1] = __dadd_rn(__dadd_rn(__dmul_rn(m[4], x), __dmul_rn(m[5], y)), __dmul_rn(m[6], z));
  o[2] = __dadd_rn(__dadd_rn(__dmul_rn(m[8], x), __dmul_rn(m[9], y)), __dmul_rn(m[10], z));
}

// The reference's slab test (TriangleAccelerator.cpp:176-192): true when
// the node is culled.
__device__ __forceinline__ bool slab_culled(float4 na, float4 nb, const double *o, const double *inv, double tmin,
                                            double tmax) {
  const double lo[3] = {na.x, na.y, na.z}, hi[3] = {na.w, nb.x, nb.y};
  double tn[3], tf[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    tn[k] = __dmul_rn(__dsub_rn(lo[k], o[k]), inv[k]);
    tf[k] = __dmul_rn(__dsub_rn(hi[k], o[k]), inv[k]);
    if (tn[k] > tf[k]) {
      const double t = tn[k];
      tn[k] = tf[k];
      tf[k] = t;
    }
  }
  return tmin > tf[0] || tn[0] > tf[1] || tn[1] > tf[0] || tn[2] > tf[0] || tmin > tf[1] || tn[0] > tf[2] ||
         tn[1] > tf[2] || tn[2] > tf[1] || tmin > tf[2] || tn[0] > tmax || tn[1] > tmax || tn[2] > tmax;
}

// One (sub)tree walk from `root` for the ray (o, d, tmin, tmax): closest hit
// updates tmax and the hit's slot (best_slot; the instance's primitive in
// best_prim when inside an instance), any hit returns on the first.  Leaves
// of the top tree may hold instances (INNER = false); a subtree's do not.
// Returns false on stack overflow.
template <int CAP, bool CLOSEST, bool INNER>
__device__ bool walk_exact(const float4 *__restrict__ nodes, const float4 *__restrict__ tris,
                           const InstDev *__restrict__ inst, const uint4 *__restrict__ ext, uint32_t root,
                           const double *o, const double *d, double tmin, double &tmax, int &best_slot,
                           int &best_prim, bool &hit, uint32_t *stk) {
  const double inv[3] = {__ddiv_rn(1.0, d[0]), __ddiv_rn(1.0, d[1]), __ddiv_rn(1.0, d[2])};
  int sp = 0;
  stk[sp++] = root;
  while (sp > 0) {
    const uint32_t ni = stk[--sp];
    const float4 na = __ldg(nodes + 2 * ni), nb = __ldg(nodes + 2 * ni + 1);
    if (slab_culled(na, nb, o, inv, tmin, tmax)) continue;
    const uint32_t a = __float_as_uint(nb.z), b = __float_as_uint(nb.w);
    if (b & 3u) {
      const uint32_t axis = (b & 3u) - 1u, mask = (b >> 2) & 7u;
      const uint32_t sL = a, sM = a + (mask & 1u), sR = sM + ((mask >> 1) & 1u);
      if (sp + 3 > CAP) return false;
      if (d[axis] > 0.0) {  // children pushed in reverse so that the left one pops first
        if (mask & 4u) stk[sp++] = sR;
        if (mask & 2u) stk[sp++] = sM;
        if (mask & 1u) stk[sp++] = sL;
      } else {
        if (mask & 1u) stk[sp++] = sL;
        if (mask & 2u) stk[sp++] = sM;
        if (mask & 4u) stk[sp++] = sR;
      }
      continue;
    }
    uint32_t tf = a, tc = b >> 8, i0 = 0, ic = 0;
    if (!INNER && (b & kLeafExt)) {
      const uint4 e = __ldg(ext + a);
      tf = e.x;
      tc = e.y;
      i0 = e.z;
      ic = e.w;
    }
    for (uint32_t k = 0; k < ic && !INNER; ++k) {
      const InstDev *I = inst + i0 + k;
      double mo[3], md[3];
      xf_point(I->m, o[0], o[1], o[2], mo);
      xf_vector(I->m, d[0], d[1], d[2], md);
      int slot = -1, pr = -1;
      bool h2 = false;
      if (!walk_exact<CAP, CLOSEST, true>(nodes, tris, inst, ext, I->root, mo, md, tmin, tmax, slot, pr, h2,
                                          stk + sp))
        return false;
      if (h2) {
        hit = true;
        if (!CLOSEST) return true;
        best_slot = slot;
        best_prim = I->prim;
      }
    }
    for (uint32_t k = 0; k < tc; ++k) {
      const int slot = (int)(tf + k);
      float3 v0, v1, v2;
      int prim, tri;
      load_tri(tris, (uint32_t)slot, v0, v1, v2, prim, tri);
      double t64;
      if (tri_test64v(o[0], o[1], o[2], d[0], d[1], d[2], v0, v1, v2, tmin, tmax, t64)) {
        hit = true;
        if (!CLOSEST) return true;
        tmax = t64;
        best_slot = slot;
        best_prim = prim;
      }
    }
  }
  return true;
}

template <int CAP, bool CLOSEST, bool DRAY>
__global__ void __launch_bounds__(128)
    k_trace_inst(const float4 *__restrict__ nodes, const float4 *__restrict__ tris, const InstDev *__restrict__ inst,
                 const uint4 *__restrict__ ext, const float4 *__restrict__ rays, int n, const int *__restrict__ n_dev,
                 const int32_t *__restrict__ out_index, void *__restrict__ out, unsigned *__restrict__ status,
                 unsigned long long *__restrict__ traced) {
  if (n_dev) n = min(n, *n_dev);
  if (traced && blockIdx.x == 0 && threadIdx.x == 0 && n > 0) atomicAdd(traced, (unsigned long long)n);
  uint32_t stk[2 * CAP];
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double o[3], d[3], tmin, tmax;
    if (DRAY) {
      const RayD r = load_ray_d(rays, i);
      o[0] = r.ox, o[1] = r.oy, o[2] = r.oz, d[0] = r.dx, d[1] = r.dy, d[2] = r.dz, tmin = r.tmin, tmax = r.tmax;
    } else {
      const RayF r = load_ray(rays, i);
      o[0] = r.ox, o[1] = r.oy, o[2] = r.oz, d[0] = r.dx, d[1] = r.dy, d[2] = r.dz, tmin = r.tmin, tmax = r.tmax;
    }
    int slot = -1, prim = -1;
    bool hit = false;
    if (!walk_exact<CAP, CLOSEST, false>(nodes, tris, inst, ext, 0u, o, d, tmin, tmax, slot, prim, hit, stk))
      atomicOr(status, 1u);
    const int oi = out_index ? out_index[i] : i;
    if (!CLOSEST) {
      ((uint8_t *)out)[oi] = hit ? 1 : 0;
    } else if (DRAY) {
      int4 h = make_int4(0, 0x7ff00000, -1, -1);
      if (hit) {
        const long long tb = __double_as_longlong(tmax);
        h = make_int4((int)(tb & 0xffffffffll), (int)(tb >> 32), prim, __float_as_int(__ldg(tris + 3 * slot + 1).w));
      }
      ((int4 *)out)[oi] = h;
    } else {
      int4 h = make_int4(0x7f800000, -1, -1, 0);
      if (hit) h = make_int4(__float_as_int((float)tmax), prim, __float_as_int(__ldg(tris + 3 * slot + 1).w), 1);
      ((int4 *)out)[oi] = h;
    }
  }
}

// Per-device launch facts, computed once per device on first use and read
// without a lock afterwards (launches may come from several host threads).
constexpr int kMaxDevices = 64;

std::mutex &prepare_mutex() {
  static std::mutex m;
  return m;
}

cudaError_t current_device(int &dev) {
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  return dev < 0 || dev >= kMaxDevices ? cudaErrorInvalidDevice : cudaSuccess;
}

// The kernel of a variant: bit 0 closest hit, bit 1 double rays.
template <int CAP>
const void *trace_kernel(int variant) {
  switch (variant) {
    case 0: return (const void *)k_trace<CAP, false, false>;
    case 1: return (const void *)k_trace<CAP, true, false>;
    case 2: return (const void *)k_trace<CAP, false, true>;
    default: return (const void *)k_trace<CAP, true, true>;
  }
}

// Resident CTAs per SM of each variant on each device (0 = not yet known).
template <int CAP>
std::atomic<int> &cap_occupancy(int dev, int variant) {
  static std::atomic<int> blocks_per_sm[kMaxDevices][4];
  return blocks_per_sm[dev][variant];
}

template <int CAP>
cudaError_t cap_prepare(int dev) {
  bool known = true;
  for (int v = 0; v < 4; ++v) known = known && cap_occupancy<CAP>(dev, v).load(std::memory_order_acquire) != 0;
  if (known) return cudaSuccess;
  std::lock_guard<std::mutex> lock(prepare_mutex());
  for (int v = 0; v < 4; ++v) {
    std::atomic<int> &slot = cap_occupancy<CAP>(dev, v);
    if (slot.load(std::memory_order_relaxed) != 0) continue;
    cudaError_t e;
    if (SKW_TRAV_CARVEOUT >= 0) {
      e = cudaFuncSetAttribute(trace_kernel<CAP>(v), cudaFuncAttributePreferredSharedMemoryCarveout,
                               SKW_TRAV_CARVEOUT);
      if (e != cudaSuccess) return e;
    }
    int occ = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, trace_kernel<CAP>(v), SKW_TRAV_BLOCK, 0);
    if (e != cudaSuccess) return e;
    slot.store(occ < 1 ? 1 : occ, std::memory_order_release);
  }
  return cudaSuccess;
}

// SM count of each device (0 = not yet known).
cudaError_t device_sms(int dev, int &sms) {
  static std::atomic<int> cache[kMaxDevices];
  sms = cache[dev].load(std::memory_order_acquire);
  if (sms != 0) return cudaSuccess;
  cudaError_t e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return e;
  cache[dev].store(sms, std::memory_order_release);
  return cudaSuccess;
}

// Device tables of the accelerators that have instances, by their node
// array (the traversal launches receive the node pointer).
// Per-accelerator launch tables, keyed by the device node array: the
// instance tables (null: no instances) and the accelerator's traced-ray
// counter (null: none).
struct InstTables {
  const void *inst = nullptr;
  const void *ext = nullptr;
  unsigned long long *traced = nullptr;
};
std::mutex &inst_mutex() {
  static std::mutex m;
  return m;
}
std::unordered_map<const void *, InstTables> &inst_registry() {
  static std::unordered_map<const void *, InstTables> r;
  return r;
}
bool find_instances(const void *nodes, InstTables &t) {
  std::lock_guard<std::mutex> lock(inst_mutex());
  auto &r = inst_registry();
  if (r.empty()) return false;
  auto it = r.find(nodes);
  if (it == r.end()) return false;
  t = it->second;
  return true;
}

template <int CAP>
cudaError_t launch_inst(int variant, const void *nodes, const void *tris, const InstTables &T, const void *rays,
                        int64_t n, const int *n_dev, const int32_t *out_index, void *out, unsigned *status,
                        cudaStream_t stream, int sms) {
  const int64_t want = (n + 127) / 128, cap = (int64_t)sms * 16;
  const dim3 grid((unsigned)(want < cap ? want : cap)), block(128);
  const float4 *nd = (const float4 *)nodes, *tr = (const float4 *)tris, *ry = (const float4 *)rays;
  const InstDev *in = (const InstDev *)T.inst;
  const uint4 *ex = (const uint4 *)T.ext;
  switch (variant) {
    case 0:
      k_trace_inst<CAP, false, false><<<grid, block, 0, stream>>>(nd, tr, in, ex, ry, (int)n, n_dev, out_index, out, status, T.traced);
      break;
    case 1:
      k_trace_inst<CAP, true, false><<<grid, block, 0, stream>>>(nd, tr, in, ex, ry, (int)n, n_dev, out_index, out, status, T.traced);
      break;
    case 2:
      k_trace_inst<CAP, false, true><<<grid, block, 0, stream>>>(nd, tr, in, ex, ry, (int)n, n_dev, out_index, out, status, T.traced);
      break;
    default:
      k_trace_inst<CAP, true, true><<<grid, block, 0, stream>>>(nd, tr, in, ex, ry, (int)n, n_dev, out_index, out, status, T.traced);
  }
  return cudaGetLastError();
}

template <int CAP>
cudaError_t launch_cap(int variant, const void *nodes, const void *tris, const void *rays, int64_t n,
                       const int *n_dev, float scene_abs, const int32_t *out_index, void *out, unsigned *status,
                       cudaStream_t stream, int ctas_per_sm, int *work, int surf) {
  int dev = 0, sms = 0;
  cudaError_t e = current_device(dev);
  if (e != cudaSuccess || (e = cap_prepare<CAP>(dev)) != cudaSuccess || (e = device_sms(dev, sms)) != cudaSuccess)
    return e;
  InstTables T;
  if (find_instances(nodes, T) && T.inst)
    return launch_inst<CAP>(variant, nodes, tris, T, rays, n, n_dev, out_index, out, status, stream, sms);
  int per_sm = cap_occupancy<CAP>(dev, variant).load(std::memory_order_acquire);
  if (ctas_per_sm > 0 && ctas_per_sm < per_sm) per_sm = ctas_per_sm;
  const int64_t warps_per_block = SKW_TRAV_BLOCK / 32;
  int64_t blocks = (int64_t)per_sm * sms;
  const int64_t needed = (n + 32 * warps_per_block - 1) / (32 * warps_per_block);
  if (blocks > needed) blocks = needed;
  // every warp draws at most one group past the end: keep the counter in int range
  if (n > (int64_t)INT32_MAX - 32 * warps_per_block * blocks) work = nullptr;
  if (work && (e = cudaMemsetAsync(work, 0, sizeof(int), stream)) != cudaSuccess) return e;
  const float4 *nd = (const float4 *)nodes, *tr = (const float4 *)tris, *ry = (const float4 *)rays;
  const dim3 grid((unsigned)blocks), block(SKW_TRAV_BLOCK);
  switch (variant) {
    case 0:
      k_trace<CAP, false, false><<<grid, block, 0, stream>>>(nd, tr, ry, (int)n, n_dev, scene_abs, out_index, out,
                                                             status, work, surf, T.traced);
      break;
    case 1:
      k_trace<CAP, true, false><<<grid, block, 0, stream>>>(nd, tr, ry, (int)n, n_dev, scene_abs, out_index, out,
                                                            status, work, surf, T.traced);
      break;
    case 2:
      k_trace<CAP, false, true><<<grid, block, 0, stream>>>(nd, tr, ry, (int)n, n_dev, scene_abs, out_index, out,
                                                            status, work, surf, T.traced);
      break;
    default:
      k_trace<CAP, true, true><<<grid, block, 0, stream>>>(nd, tr, ry, (int)n, n_dev, scene_abs, out_index, out,
                                                           status, work, surf, T.traced);
  }
  return cudaGetLastError();
}

cudaError_t launch_variant(int variant, int stack_cap, const void *nodes, const void *tris, const void *rays,
                           int64_t n, const int *n_dev, float scene_abs, const int32_t *out_index, void *out,
                           unsigned *status, cudaStream_t stream, int ctas_per_sm, int *work, int surf) {
  if (n <= 0) return cudaSuccess;
  switch (stack_cap) {
    case 48:
      return launch_cap<48>(variant, nodes, tris, rays, n, n_dev, scene_abs, out_index, out, status, stream,
                            ctas_per_sm, work, surf);
    case 96:
      return launch_cap<96>(variant, nodes, tris, rays, n, n_dev, scene_abs, out_index, out, status, stream,
                            ctas_per_sm, work, surf);
    case 192:
      return launch_cap<192>(variant, nodes, tris, rays, n, n_dev, scene_abs, out_index, out, status, stream,
                             ctas_per_sm, work, surf);
    default:
      return launch_cap<416>(variant, nodes, tris, rays, n, n_dev, scene_abs, out_index, out, status, stream,
                             ctas_per_sm, work, surf);
  }
}

}  // namespace

cudaError_t prepare_traversal(int stack_cap) {
  int dev = 0, sms = 0;
  cudaError_t e = current_device(dev);
  if (e != cudaSuccess || (e = device_sms(dev, sms)) != cudaSuccess) return e;
  switch (stack_cap) {
    case 48: return cap_prepare<48>(dev);
    case 96: return cap_prepare<96>(dev);
    case 192: return cap_prepare<192>(dev);
    default: return cap_prepare<416>(dev);
  }
}

int traversal_max_ctas_per_sm(int stack_cap) {
  int dev = 0;
  if (current_device(dev) != cudaSuccess || prepare_traversal(stack_cap) != cudaSuccess) return 1;
  switch (stack_cap) {
    case 48: return cap_occupancy<48>(dev, 1).load();
    case 96: return cap_occupancy<96>(dev, 1).load();
    case 192: return cap_occupancy<192>(dev, 1).load();
    default: return cap_occupancy<416>(dev, 1).load();
  }
}

int traversal_stack_capacity(int max_depth) {
  const int need = 2 * max_depth + 1;
  if (need <= 48) return 48;
  if (need <= 96) return 96;
  if (need <= 192) return 192;
  return 416;  // the reference's depth limit 200 needs 401 entries
}

cudaError_t launch_traversal(bool closest, int stack_cap, const void *nodes, const void *tris, const void *rays,
                             int64_t n, const int *n_dev, float scene_abs, const int32_t *out_index, void *out,
                             unsigned *status, cudaStream_t stream, int ctas_per_sm, int *work, bool surface) {
  return launch_variant(closest ? 1 : 0, stack_cap, nodes, tris, rays, n, n_dev, scene_abs, out_index, out, status,
                        stream, ctas_per_sm, work, surface ? 1 : 0);
}

void register_instances(const void *nodes, const void *inst, const void *ext) {
  std::lock_guard<std::mutex> lock(inst_mutex());
  InstTables &t = inst_registry()[nodes];
  t.inst = inst;
  t.ext = ext;
}

void register_ray_counter(const void *nodes, unsigned long long *traced) {
  std::lock_guard<std::mutex> lock(inst_mutex());
  inst_registry()[nodes].traced = traced;
}

void unregister_instances(const void *nodes) {
  std::lock_guard<std::mutex> lock(inst_mutex());
  inst_registry().erase(nodes);
}

cudaError_t launch_traversal_d(bool closest, int stack_cap, const void *nodes, const void *tris, const void *rays,
                               int64_t n, float scene_abs, void *out, unsigned *status, cudaStream_t stream,
                               int *work) {
  return launch_variant(closest ? 3 : 2, stack_cap, nodes, tris, rays, n, nullptr, scene_abs, nullptr, out, status,
                        stream, 0, work, 0);
}

}  // namespace skw
