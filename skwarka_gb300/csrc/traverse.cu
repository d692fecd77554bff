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
// the node tests run in float with the slab interval widened by 8 ulp, so a
// node is culled only if the reference culls it too.  The triangle test runs
// in float with a forward error bound on every quantity; only when a decision
// (inside/outside an edge, t inside [tmin, tmax], which of two hits is
// nearer) falls inside that bound is the triangle re-tested with the
// reference's exact double-precision arithmetic (round-to-nearest intrinsics,
// no fused multiply-add).  Such hits are flagged SKW_HIT_FP64_DECIDED.
//
// Layout: nodes are 32-byte DevNode records read as two 16-byte loads; each
// triangle slot is 3 x float4 (v0|prim, v1|tri, v2|slot); rays are 2 x float4.
// The per-thread stack (16-byte entries) lives in local memory (L1-resident);
// its capacity CAP is chosen on the host as >= 2 * tree depth + 1, which
// bounds its use (at most two entries are pushed per level).
#include <cuda_runtime.h>
#include <cstdint>

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
#define SKW_TRAV_MINB 4
#endif

enum : int { kMiss = 0, kHit = 1, kAmbiguous = 2 };

struct RayF {
  float ox, oy, oz, dx, dy, dz, tmin, tmax;
};

__device__ __forceinline__ RayF load_ray(const float4 *__restrict__ rays, int64_t i) {
  const float4 a = __ldg(rays + 2 * i);
  const float4 b = __ldg(rays + 2 * i + 1);
  return RayF{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
}

// Float triangle test with a forward error bound.  Returns kMiss when the
// reference's double test certainly rejects (barycentrics or t < tmin),
// kHit when its barycentric tests and t >= tmin certainly pass (t and a bound
// et on |t - t_exact| are returned), else kAmbiguous.
__device__ __forceinline__ int tri_test32(const RayF &r, float3 v0, float3 v1, float3 v2, float &t, float &et) {
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

// The reference's double-precision Moller-Trumbore test, operation by
// operation (TriangleAccelerator.cpp:240-273).  Intrinsics keep every
// product and sum separately rounded, as in the x86-64 SSE2 build.
__device__ __noinline__ bool tri_test64(const RayF &r, float3 v0f, float3 v1f, float3 v2f, double tmin, double tmax,
                                        double &t_out) {
  const double ox = r.ox, oy = r.oy, oz = r.oz, dx = r.dx, dy = r.dy, dz = r.dz;
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

// Reference slab test (TriangleAccelerator.cpp:176-192) on a widened float
// interval.  Returns true when the node must be visited; `lo` receives the
// widened entry distance max(tnear_x, tnear_y, tnear_z, tmin), which is all
// a later re-test against a smaller tmax needs.
__device__ __forceinline__ bool node_visit(const float4 na, const float4 nb, const RayF &r, float ix, float iy,
                                           float iz, float tcull, float &lo) {
  float tn0 = (na.x - r.ox) * ix, tf0 = (na.w - r.ox) * ix;
  float tn1 = (na.y - r.oy) * iy, tf1 = (nb.x - r.oy) * iy;
  float tn2 = (na.z - r.oz) * iz, tf2 = (nb.y - r.oz) * iz;
  const float a0 = fminf(tn0, tf0), b0 = fmaxf(tn0, tf0);
  const float a1 = fminf(tn1, tf1), b1 = fmaxf(tn1, tf1);
  const float a2 = fminf(tn2, tf2), b2 = fmaxf(tn2, tf2);
  // NaN (0 * inf) slabs: fminf/fmaxf return the other operand, and the
  // widened bounds below drop NaN, matching the reference's comparisons,
  // which are all false on NaN.
  const float l0 = fmaf(-kWiden, fabsf(a0), a0), h0 = fmaf(kWiden, fabsf(b0), b0);
  const float l1 = fmaf(-kWiden, fabsf(a1), a1), h1 = fmaf(kWiden, fabsf(b1), b1);
  const float l2 = fmaf(-kWiden, fabsf(a2), a2), h2 = fmaf(kWiden, fabsf(b2), b2);
  lo = fmaxf(fmaxf(l0, l1), fmaxf(l2, r.tmin));
  const float hi = fminf(fminf(h0, h1), fminf(h2, tcull));
  return !(lo > hi);
}

// Per-thread traversal state shared by the closest-hit and any-hit kernels.
//
// Visit order equals the reference's (TriangleAccelerator.cpp:170-211): the
// reference pushes an internal node's children and pops the near-side one
// first, testing each node's box when it is popped.  Here an internal node's
// present children (contiguous, so their loads go out together) are box-tested
// right away; the first passing one in the reference's pop order becomes the
// current node and the rest are pushed so that they pop in that order.  A
// pushed entry keeps its widened entry distance, and popping re-culls it
// against the tmax of that moment -- the only part of the reference's
// pop-time box test that can change after the push, since tmax only shrinks.
struct StackEntry {
  uint32_t a, b;  // the node's words 6 and 7
  float lo;       // widened entry distance
  uint32_t pad;
};

template <int CAP>
struct Traversal {
  uint4 stack[CAP];
  int sp;
  uint32_t cur_a, cur_b;  // current node (passed its box test)

  __device__ __forceinline__ bool pop(float tcull) {
    while (sp > 0) {
      const uint4 e = stack[--sp];
      if (__uint_as_float(e.z) > tcull) continue;  // the reference culls it at pop
      cur_a = e.x;
      cur_b = e.y;
      return true;
    }
    return false;
  }

  // Expands internal nodes until the current node is a leaf; false when the
  // stack runs out.  status bit 0 records an (impossible by construction)
  // stack overflow.
  __device__ __forceinline__ bool descend(const float4 *__restrict__ nodes, const RayF &r, float ix, float iy,
                                          float iz, float tcull, unsigned *status) {
    while ((cur_b & 3u) != 0u) {
      const uint32_t type = cur_b & 3u, mask = (cur_b >> 2) & 7u;
      const uint32_t sL = cur_a, sM = cur_a + (mask & 1u), sR = sM + ((mask >> 1) & 1u);
      const float dax = type == 1u ? r.dx : (type == 2u ? r.dy : r.dz);
      const bool near_left = !(dax > 0.0f);  // reference pops left first when d[axis] > 0
      // Children in the reference's pop order.
      uint32_t slot[3];
      uint32_t present[3];
      slot[0] = near_left ? sR : sL;
      present[0] = near_left ? (mask & 4u) : (mask & 1u);
      slot[1] = sM;
      present[1] = mask & 2u;
      slot[2] = near_left ? sL : sR;
      present[2] = near_left ? (mask & 1u) : (mask & 4u);
      bool pass[3];
      float lo[3];
      uint32_t wa[3], wb[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        pass[k] = false;
        if (present[k]) {
          const float4 ca = __ldg(nodes + 2 * slot[k]);
          const float4 cb = __ldg(nodes + 2 * slot[k] + 1);
          pass[k] = node_visit(ca, cb, r, ix, iy, iz, tcull, lo[k]);
          wa[k] = __float_as_uint(cb.z);
          wb[k] = __float_as_uint(cb.w);
        }
      }
      // Push the passing children after the first, last-visited first.
      int first = pass[0] ? 0 : (pass[1] ? 1 : (pass[2] ? 2 : -1));
      if (sp + 2 > CAP) {
        atomicOr(status, 1u);
        return false;
      }
#pragma unroll
      for (int k = 2; k >= 1; --k) {
        if (pass[k] && k != first) stack[sp++] = make_uint4(wa[k], wb[k], __float_as_uint(lo[k]), 0u);
      }
      if (first < 0) {
        if (!pop(tcull)) return false;
        continue;
      }
      cur_a = first == 0 ? wa[0] : (first == 1 ? wa[1] : wa[2]);
      cur_b = first == 0 ? wb[0] : (first == 1 ? wb[1] : wb[2]);
    }
    return true;
  }
};

template <int CAP>
__global__ void __launch_bounds__(SKW_TRAV_BLOCK, SKW_TRAV_MINB) k_closest_hit(const float4 *__restrict__ nodes, const float4 *__restrict__ tris,
                                                     const float4 *__restrict__ rays, int64_t n,
                                                     int4 *__restrict__ hits, unsigned *__restrict__ status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const RayF r = load_ray(rays, i);
  const float ix = 1.0f / r.dx, iy = 1.0f / r.dy, iz = 1.0f / r.dz;

  int best_slot = -1, best_prim = -1, best_tri = -1;
  float best_t = r.tmax, best_et = 0.0f;  // best_t +- best_et holds the reference's current tmax
  double best_t64 = (double)r.tmax;
  bool have64 = true;  // best_t64 is the reference's exact current tmax
  float tcull = r.tmax;
  uint32_t flags = 0;

  Traversal<CAP> tr;
  tr.sp = 0;
  bool alive;
  {
    const float4 na = __ldg(nodes), nb = __ldg(nodes + 1);
    float lo;
    alive = node_visit(na, nb, r, ix, iy, iz, tcull, lo);
    tr.cur_a = __float_as_uint(nb.z);
    tr.cur_b = __float_as_uint(nb.w);
  }
  while (alive) {
    if (!tr.descend(nodes, r, ix, iy, iz, tcull, status)) break;
    // Current node is a leaf: test its triangles in order.
    const uint32_t a = tr.cur_a, cnt = tr.cur_b >> 8;
    for (uint32_t k = 0; k < cnt; ++k) {
      const uint32_t slot = a + k;
      float3 v0, v1, v2;
      int prim, tri;
      load_tri(tris, slot, v0, v1, v2, prim, tri);
      float t, et;
      int res = tri_test32(r, v0, v1, v2, t, et);
      if (res == kMiss) continue;
      if (res == kHit) {
        if (t - et > best_t + best_et) continue;  // certainly beyond the current tmax
        if (t + et < best_t - best_et) {          // certainly nearer: accept in float
          best_slot = (int)slot;
          best_prim = prim;
          best_tri = tri;
          best_t = t;
          best_et = et;
          have64 = false;
          tcull = t + et;
          continue;
        }
      }
      // Exact re-test against the reference's exact current tmax.
      if (!have64) {
        float3 b0, b1, b2;
        int bp, bt;
        load_tri(tris, (uint32_t)best_slot, b0, b1, b2, bp, bt);
        double tb;
        best_t64 = tri_test64(r, b0, b1, b2, (double)r.tmin, 1.0e308, tb) ? tb : (double)best_t;
        have64 = true;
      }
      double t64;
      if (tri_test64(r, v0, v1, v2, (double)r.tmin, best_t64, t64)) {
        if (best_slot >= 0 && fabs(t64 - best_t64) <= 1e-12 * fabs(t64)) flags |= 2u;
        best_slot = (int)slot;
        best_prim = prim;
        best_tri = tri;
        best_t64 = t64;
        best_t = (float)t64;
        best_et = fabsf(best_t) * 1.2e-7f;
        tcull = __double2float_ru(t64);
        flags |= 1u;
      }
    }
    alive = tr.pop(tcull);
  }
  // A float-decided hit whose t bound exceeds half the 1e-5 reporting
  // tolerance (grazing incidence) gets its t from the exact test, once,
  // after the traversal loop where the warp has reconverged.
  if (best_slot >= 0 && !have64 && best_et > 5.0e-6f * fabsf(best_t)) {
    float3 b0, b1, b2;
    int bp, bt;
    load_tri(tris, (uint32_t)best_slot, b0, b1, b2, bp, bt);
    double tb;
    if (tri_test64(r, b0, b1, b2, (double)r.tmin, 1.0e308, tb)) {
      best_t64 = tb;
      have64 = true;
      flags |= 4u;
    }
  }
  int4 h;
  if (best_slot >= 0) {
    h = make_int4(__float_as_int(have64 ? (float)best_t64 : best_t), best_prim, best_tri, (int)flags);
  } else {
    h = make_int4(__float_as_int(__int_as_float(0x7f800000)), -1, -1, (int)flags);
  }
  hits[i] = h;
}

template <int CAP>
__global__ void __launch_bounds__(SKW_TRAV_BLOCK, SKW_TRAV_MINB) k_any_hit(const float4 *__restrict__ nodes, const float4 *__restrict__ tris,
                                                 const float4 *__restrict__ rays, int64_t n,
                                                 uint8_t *__restrict__ occluded, unsigned *__restrict__ status) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const RayF r = load_ray(rays, i);
  const float ix = 1.0f / r.dx, iy = 1.0f / r.dy, iz = 1.0f / r.dz;
  Traversal<CAP> tr;
  tr.sp = 0;
  bool alive, hit = false;
  {
    const float4 na = __ldg(nodes), nb = __ldg(nodes + 1);
    float lo;
    alive = node_visit(na, nb, r, ix, iy, iz, r.tmax, lo);
    tr.cur_a = __float_as_uint(nb.z);
    tr.cur_b = __float_as_uint(nb.w);
  }
  while (alive && !hit) {
    if (!tr.descend(nodes, r, ix, iy, iz, r.tmax, status)) break;
    const uint32_t a = tr.cur_a, cnt = tr.cur_b >> 8;
    for (uint32_t k = 0; k < cnt; ++k) {
      float3 v0, v1, v2;
      int prim, tri;
      load_tri(tris, a + k, v0, v1, v2, prim, tri);
      float t, et;
      int res = tri_test32(r, v0, v1, v2, t, et);
      if (res == kMiss) continue;
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
    if (!hit) alive = tr.pop(r.tmax);
  }
  occluded[i] = hit ? 1 : 0;
}

template <int CAP>
cudaError_t launch_pair(bool closest, const void *nodes, const void *tris, const void *rays, int64_t n, void *out,
                        unsigned *status, cudaStream_t stream) {
  const int block = SKW_TRAV_BLOCK;
  const int64_t grid = (n + block - 1) / block;
  if (closest) {
    k_closest_hit<CAP><<<(unsigned)grid, block, 0, stream>>>((const float4 *)nodes, (const float4 *)tris,
                                                            (const float4 *)rays, n, (int4 *)out, status);
  } else {
    k_any_hit<CAP><<<(unsigned)grid, block, 0, stream>>>((const float4 *)nodes, (const float4 *)tris,
                                                        (const float4 *)rays, n, (uint8_t *)out, status);
  }
  return cudaGetLastError();
}

}  // namespace

int traversal_stack_capacity(int max_depth) {
  const int need = 2 * max_depth + 1;
  if (need <= 48) return 48;
  if (need <= 96) return 96;
  if (need <= 192) return 192;
  return 416;  // the reference's depth limit 200 needs 401 entries
}

cudaError_t launch_traversal(bool closest, int stack_cap, const void *nodes, const void *tris, const void *rays,
                             int64_t n, void *out, unsigned *status, cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  switch (stack_cap) {
    case 48:
      return launch_pair<48>(closest, nodes, tris, rays, n, out, status, stream);
    case 96:
      return launch_pair<96>(closest, nodes, tris, rays, n, out, status, stream);
    case 192:
      return launch_pair<192>(closest, nodes, tris, rays, n, out, status, stream);
    default:
      return launch_pair<416>(closest, nodes, tris, rays, n, out, status, stream);
  }
}

}  // namespace skw
