// Construction of the ternary bbox kd-tree on the GPU: node for node the
// tree of the host build (accel_build.cpp), which restates the reference's
// TriangleAccelerator build (Raytracer/Core/TriangleAccelerator.cpp:470-729):
// node box, leaf rule, bucketed split search with its float / double
// arithmetic, and the in-place three-way partition's exact element order.
//
// Layout: the triangles' float boxes in slot order (6 floats: lo xyz,
// hi xyz) and each slot's triangle; every slot carries the range [b, e) of
// the node it is in (b = -1 once that node is a leaf), so a level of the
// tree is a fixed sequence of slot-parallel launches and 64-bit scans, and
// a node's own values live at its first slot b.  Per level:
//   * node boxes: a warp-segmented reduction of 64-bit keys (value order,
//     then slot) merged with atomics — the reference's min / max keep the
//     first of equal values (it matters only for the sign of a zero);
//   * leaf rule (<= 4 triangles, all three axes split through the middle,
//     depth 200), candidate count tries = min(200, 2n), per-axis scale;
//   * buckets: per candidate plane the left / middle / right boxes and
//     counts, filled by atomics on order-preserving float keys (box unions
//     and counts do not depend on the order they are formed in);
//   * split search: one thread per (node, axis), suffix unions of the right
//     boxes, then the costs in the reference's double arithmetic in order;
//   * partition: the reference's sequential swap loop (left to the front in
//     order of processing, right to the back, a rotating middle block)
//     computed in parallel.  Elements are processed from the front, except
//     that after each right-class element the loop takes elements from the
//     back until it meets one that is not right-class: with prefix counts
//     over the front stream (right-class elements so far) and the back
//     stream (its runs), each element's processing step follows; left and
//     right destinations are ranks in that order, and a middle element's
//     destination follows the chain "moved to the block's end when the
//     block's front reaches it" by pointer jumping.
// Accelerators whose meshes are shared by several primitives (instancing)
// are built on the host.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <vector>

#include "accel_build.h"
#include "kernels.h"

namespace skw {
namespace {

constexpr int kB = 256;
constexpr int kTries = 200;    // TriangleAccelerator.h:131
constexpr int kLeafMax = 4;    // TriangleAccelerator.h:128
constexpr int kDepthMax = 200; // TriangleAccelerator.h:134

// Order-preserving key of a float (NaN excluded by the callers).
__device__ __forceinline__ uint32_t okey(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float okey_inv(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}
// Bucket keys: min identity 0xFFFFFFFF (decodes to +inf), max identity 0
// (decodes to -inf), as the reference's empty BBox3D.
__device__ __forceinline__ float lo_of(uint32_t k) { return k == 0xFFFFFFFFu ? INFINITY : okey_inv(k); }
__device__ __forceinline__ float hi_of(uint32_t k) { return k == 0u ? -INFINITY : okey_inv(k); }

// (size_t) of a double as the reference's x86-64 build computes it: NaN ->
// 2^63, values >= 2^64 -> 0 (the same rule as the host build's cast_size).
__device__ __forceinline__ uint64_t cast_size(double v) {
  if (isnan(v)) return 1ull << 63;
  if (v >= 18446744073709551616.0) return 0ull;
  if (v >= 9223372036854775808.0) return (uint64_t)__double2ll_rz(v - 9223372036854775808.0) + (1ull << 63);
  return (uint64_t)__double2ll_rz(v);
}

// BBox3D<double>::Area of a box with float corners.
__device__ __forceinline__ double area_d(const float *lo, const float *hi) {
  const double x = fabs(__dsub_rn((double)hi[0], (double)lo[0]));
  const double y = fabs(__dsub_rn((double)hi[1], (double)lo[1]));
  const double z = fabs(__dsub_rn((double)hi[2], (double)lo[2]));
  return __dmul_rn(2.0, __dadd_rn(__dadd_rn(__dmul_rn(x, y), __dmul_rn(x, z)), __dmul_rn(y, z)));
}
// BBox3D<float>::Area.
__device__ __forceinline__ float area_f(const float *lo, const float *hi) {
  const float x = fabsf(__fsub_rn(hi[0], lo[0]));
  const float y = fabsf(__fsub_rn(hi[1], lo[1]));
  const float z = fabsf(__fsub_rn(hi[2], lo[2]));
  return __fmul_rn(2.0f, __fadd_rn(__fadd_rn(__fmul_rn(x, y), __fmul_rn(x, z)), __fmul_rn(y, z)));
}
// std::min(1.0, v)
__device__ __forceinline__ double min1(double v) { return v < 1.0 ? v : 1.0; }

struct Dev {
  int64_t n;
  float *box, *box2;          // 6 floats per slot
  uint32_t *perm, *perm2;     // triangle of each slot
  int2 *seg;                  // node range of each slot ((-1, -1): in a leaf)
  uint8_t *smask, *sord;      // node's middle-split axes; child ordinal in its parent
  int32_t *spar;              // parent node id (-1: the root)
  // per node, at its first slot
  unsigned long long *hkeys;  // 6 box keys
  float *hbox;                // 6 floats
  double *hcoef;              // 3 per node
  double *hsplit;
  // (a node's bucket base is cnt2[b] between the bucket scan and the split search)
  int32_t *hid, *htries, *haxis;
  uint32_t *heads;            // the level's nodes' first slots, by rank
  uint32_t *hnl, *hnr;
  uint8_t *hleaf;
  double *bcost, *bpos;       // 3 per node
  uint32_t *buckets;          // 7 words per bucket: lo keys, hi keys, count
  // per level
  uint8_t *cls;
  uint64_t *cnt, *cnt2, *cnt3, *sums;  // n + 1 each (sums: block totals)
  uint32_t *tarr, *jarr, *ord, *iarr, *f0, *f1, *lmb, *dest;
  int *err;
  int *maxseg;                // the level's largest node (triangles)
  unsigned long long *n_leaves;
  // node records, by node id
  float *rbox;
  uint32_t *rtb, *rte;
  uint8_t *rflags;
  int32_t *rchild;
};

inline unsigned grid_of(int64_t m) { return (unsigned)((m + kB - 1) / kB); }

__global__ void k_init(Dev D, const float *__restrict__ tbox) {
  const int64_t s = (int64_t)blockIdx.x * kB + threadIdx.x;
  if (s >= D.n) return;
  for (int c = 0; c < 6; ++c) D.box[s * 6 + c] = tbox[s * 6 + c];
  D.perm[s] = (uint32_t)s;
  D.seg[s] = make_int2(0, (int)D.n);
  D.smask[s] = 0;
  D.sord[s] = 0;
  D.spar[s] = -1;
}

// Heads of the level's nodes: their rank (a scan) gives the node id.
__global__ void k_heads(Dev D) {
  const int64_t s = (int64_t)blockIdx.x * kB + threadIdx.x;
  if (s > D.n) return;
  uint64_t h = 0;
  if (s < D.n && D.seg[s].x == (int)s) {
    h = 1;
    atomicMax(D.maxseg, D.seg[s].y - (int)s);
    for (int c = 0; c < 3; ++c) {
      D.hkeys[s * 6 + c] = ~0ull;
      D.hkeys[s * 6 + 3 + c] = 0ull;
    }
  }
  D.cnt[s] = h;
}

// Node boxes: keys (value, slot) so that the first of equal values wins,
// as in the reference's min / max over the node's triangles in slot order;
// -0 and +0 compare equal, NaN is skipped.  Runs of lanes in one node are
// reduced with shuffles, then merged with atomics.
__global__ void k_node_box(Dev D) {
  const int64_t s = (int64_t)blockIdx.x * kB + threadIdx.x;
  const int lane = threadIdx.x & 31;
  int b = -1;
  unsigned long long k[6];
  for (int c = 0; c < 3; ++c) {
    k[c] = ~0ull;
    k[3 + c] = 0ull;
  }
  if (s < D.n) {
    b = D.seg[s].x;
    if (b >= 0) {
      for (int c = 0; c < 3; ++c) {
        const float lo = D.box[s * 6 + c], hi = D.box[s * 6 + 3 + c];
        if (!isnan(lo)) k[c] = ((unsigned long long)okey(lo == 0.0f ? 0.0f : lo) << 32) | (uint32_t)s;
        if (!isnan(hi))
          k[3 + c] = ((unsigned long long)okey(hi == 0.0f ? 0.0f : hi) << 32) | (0xFFFFFFFFu - (uint32_t)s);
      }
    }
  }
  for (int o = 1; o < 32; o <<= 1) {
    const int ob = __shfl_up_sync(0xffffffffu, b, o);
    unsigned long long t[6];
    for (int c = 0; c < 6; ++c) t[c] = __shfl_up_sync(0xffffffffu, k[c], o);
    if (lane >= o && ob == b) {
      for (int c = 0; c < 3; ++c) {
        k[c] = t[c] < k[c] ? t[c] : k[c];
        k[3 + c] = t[3 + c] > k[3 + c] ? t[3 + c] : k[3 + c];
      }
    }
  }
  const int nb = __shfl_down_sync(0xffffffffu, b, 1);
  if (b >= 0 && (lane == 31 || nb != b)) {
    for (int c = 0; c < 3; ++c) {
      atomicMin(&D.hkeys[(int64_t)b * 6 + c], k[c]);
      atomicMax(&D.hkeys[(int64_t)b * 6 + 3 + c], k[3 + c]);
    }
  }
}

// A node's record and leaf decision (Node::Node, TriangleAccelerator.cpp:
// 621-636); internal nodes get their candidate count and per-axis scale
// (_DetermineBestSplit, :512-530) and ask for 9 * tries buckets.
__global__ void k_head_setup(Dev D, int64_t level_base, int depth) {
  const int64_t s = (int64_t)blockIdx.x * kB + threadIdx.x;
  if (s > D.n) return;
  uint64_t need = 0;
  if (s < D.n && D.seg[s].x == (int)s) {
    const int2 r = D.seg[s];
    const int64_t id = level_base + (int64_t)D.cnt[s];
    D.hid[s] = (int32_t)id;
    D.heads[D.cnt[s]] = (uint32_t)s;
    float lo[3], hi[3];
    for (int c = 0; c < 3; ++c) {
      const unsigned long long kl = D.hkeys[s * 6 + c], kh = D.hkeys[s * 6 + 3 + c];
      lo[c] = kl == ~0ull ? INFINITY : D.box[(int64_t)(uint32_t)kl * 6 + c];
      hi[c] = kh == 0ull ? -INFINITY : D.box[(int64_t)(0xFFFFFFFFu - (uint32_t)kh) * 6 + 3 + c];
      D.hbox[s * 6 + c] = lo[c];
      D.hbox[s * 6 + 3 + c] = hi[c];
      D.rbox[id * 6 + c] = lo[c];
      D.rbox[id * 6 + 3 + c] = hi[c];
    }
    D.rtb[id] = (uint32_t)r.x;
    D.rte[id] = (uint32_t)r.y;
    for (int c = 0; c < 3; ++c) D.rchild[id * 3 + c] = -1;
    const int32_t par = D.spar[s];
    if (par >= 0) D.rchild[(int64_t)par * 3 + D.sord[s]] = (int32_t)id;
    const int count = r.y - r.x;
    const unsigned mask = D.smask[s];
    if (count <= kLeafMax || mask == 7u || depth >= kDepthMax) {
      D.hleaf[s] = 1;
      D.rflags[id] = 0;
      atomicAdd(D.n_leaves, 1ull);
    } else {
      D.hleaf[s] = 0;
      const int tries = min(kTries, 2 * count);
      D.htries[s] = tries;
      for (int a = 0; a < 3; ++a) {
        // size_t / float converts the count to float: a float division
        D.hcoef[s * 3 + a] = (double)__fdiv_rn((float)tries, __fsub_rn(hi[a], lo[a]));
      }
      need = 9ull * (uint64_t)tries;
    }
  }
  D.cnt2[s] = need;
}

__global__ void k_bucket_init(Dev D) {
  const int64_t total = (int64_t)D.cnt2[D.n];
  for (int64_t i = (int64_t)blockIdx.x * kB + threadIdx.x; i < total; i += (int64_t)gridDim.x * kB) {
    uint32_t *r = D.buckets + i * 7;
    r[0] = r[1] = r[2] = 0xFFFFFFFFu;
    r[3] = r[4] = r[5] = 0u;
    r[6] = 0u;
  }
}

// Adds a box to bucket idx (-1: none) for the lanes that reach this call
// together: lanes adding to the same bucket are merged first, one atomic
// per bucket and key (NaN coordinates take no part, as in the reference's
// min / max).
__device__ __forceinline__ void bucket_add_grouped(uint32_t *buckets, int64_t idx, const float *lo, const float *hi) {
  const unsigned grp = __match_any_sync(__activemask(), idx);
  if (idx < 0) return;
  uint32_t kl[3], kh[3];
  for (int c = 0; c < 3; ++c) {
    kl[c] = __reduce_min_sync(grp, isnan(lo[c]) ? 0xFFFFFFFFu : okey(lo[c]));
    kh[c] = __reduce_max_sync(grp, isnan(hi[c]) ? 0u : okey(hi[c]));
  }
  if ((threadIdx.x & 31) != __ffs(grp) - 1) return;
  uint32_t *r = buckets + idx * 7;
  for (int c = 0; c < 3; ++c) {
    if (kl[c] != 0xFFFFFFFFu) atomicMin(r + c, kl[c]);
    if (kh[c] != 0u) atomicMax(r + 3 + c, kh[c]);
  }
  atomicAdd(r + 6, (uint32_t)__popc(grp));
}

// The buckets of every internal node (_DetermineBestSplit, :531-565): per
// axis not split through the middle on the path, a triangle's box goes to
// the right bucket of its first candidate plane, the left one of its last,
// and the middle ones of the planes it straddles.
__global__ void k_bucket_fill(Dev D) {
  const int64_t s = (int64_t)blockIdx.x * kB + threadIdx.x;
  if (s >= D.n) return;
  const int b = D.seg[s].x;
  if (b < 0 || D.hleaf[b]) return;
  const unsigned mask = D.smask[s];
  const uint64_t tries = (uint64_t)D.htries[b];
  const int64_t base = (int64_t)D.cnt2[b];
  float lo[3], hi[3];
  for (int c = 0; c < 3; ++c) {
    lo[c] = D.box[s * 6 + c];
    hi[c] = D.box[s * 6 + 3 + c];
  }
  for (int a = 0; a < 3; ++a) {
    if (mask & (1u << a)) continue;
    const float nlo = D.hbox[(int64_t)b * 6 + a];
    const double coef = D.hcoef[(int64_t)b * 3 + a];
    const float dmax = __fsub_rn(hi[a], nlo), dmin = __fsub_rn(lo[a], nlo);
    const uint64_t lefts_begin = min(tries, cast_size(__dadd_rn(__dmul_rn((double)dmax, coef), 1.0)));
    const uint64_t rights_end = min(tries, cast_size(__dadd_rn(__dmul_rn((double)dmin, coef), 1.0)));
    const int64_t lb = base + (int64_t)(a * 3) * (int64_t)tries;  // bucket index of L[0]
    bucket_add_grouped(D.buckets, rights_end > 0 ? lb + 2 * (int64_t)tries + (int64_t)(rights_end - 1) : -1, lo, hi);
    bucket_add_grouped(D.buckets, lefts_begin < tries ? lb + (int64_t)lefts_begin : -1, lo, hi);
    // the middle buckets: the lanes of one node walk the union of their
    // ranges together, one merged add per bucket
    uint32_t *M = D.buckets + (lb + (int64_t)tries) * 7;
    const unsigned grp = __match_any_sync(__activemask(), b);
    const bool any = rights_end < lefts_begin;
    const uint32_t jlo = __reduce_min_sync(grp, any ? (uint32_t)rights_end : 0xFFFFFFFFu);
    const uint32_t jhi = __reduce_max_sync(grp, any ? (uint32_t)lefts_begin : 0u);
    uint32_t kl[3], kh[3];
    for (int c = 0; c < 3; ++c) {
      kl[c] = isnan(lo[c]) ? 0xFFFFFFFFu : okey(lo[c]);
      kh[c] = isnan(hi[c]) ? 0u : okey(hi[c]);
    }
    const bool leader = (threadIdx.x & 31) == __ffs(grp) - 1;
    for (uint32_t j = jlo; j < jhi; ++j) {
      const bool in = rights_end <= j && j < lefts_begin;
      const unsigned who = __ballot_sync(grp, in);
      if (who == 0u) continue;
      uint32_t ml[3], mh[3];
      for (int c = 0; c < 3; ++c) {
        ml[c] = __reduce_min_sync(grp, in ? kl[c] : 0xFFFFFFFFu);
        mh[c] = __reduce_max_sync(grp, in ? kh[c] : 0u);
      }
      if (leader) {
        uint32_t *r = M + (int64_t)j * 7;
        for (int c = 0; c < 3; ++c) {
          if (ml[c] != 0xFFFFFFFFu) atomicMin(r + c, ml[c]);
          if (mh[c] != 0u) atomicMax(r + 3 + c, mh[c]);
        }
        atomicAdd(r + 6, (uint32_t)__popc(who));
      }
    }
  }
}

// Union of two bucket boxes with counts (the order of unions does not
// change a union of float boxes).
struct BoxN {
  float lo[3], hi[3];
  uint32_t n;
};
__device__ __forceinline__ BoxN box_empty() {
  BoxN b;
  for (int c = 0; c < 3; ++c) {
    b.lo[c] = INFINITY;
    b.hi[c] = -INFINITY;
  }
  b.n = 0;
  return b;
}
__device__ __forceinline__ void box_unite(BoxN &a, const BoxN &b) {
  for (int c = 0; c < 3; ++c) {
    a.lo[c] = fminf(a.lo[c], b.lo[c]);
    a.hi[c] = fmaxf(a.hi[c], b.hi[c]);
  }
  a.n += b.n;
}
__device__ __forceinline__ BoxN box_keys(const uint32_t *r) {  // a bucket as filled (keys)
  BoxN b;
  for (int c = 0; c < 3; ++c) {
    b.lo[c] = lo_of(r[c]);
    b.hi[c] = hi_of(r[3 + c]);
  }
  b.n = r[6];
  return b;
}
__device__ __forceinline__ BoxN box_shfl_up(const BoxN &a, int o) {
  BoxN b;
  for (int c = 0; c < 3; ++c) {
    b.lo[c] = __shfl_up_sync(0xffffffffu, a.lo[c], o);
    b.hi[c] = __shfl_up_sync(0xffffffffu, a.hi[c], o);
  }
  b.n = __shfl_up_sync(0xffffffffu, a.n, o);
  return b;
}
__device__ __forceinline__ BoxN box_shfl_down(const BoxN &a, int o) {
  BoxN b;
  for (int c = 0; c < 3; ++c) {
    b.lo[c] = __shfl_down_sync(0xffffffffu, a.lo[c], o);
    b.hi[c] = __shfl_down_sync(0xffffffffu, a.hi[c], o);
  }
  b.n = __shfl_down_sync(0xffffffffu, a.n, o);
  return b;
}

// One axis of one node's split search (_DetermineBestSplit, :566-608),
// one warp: lane l takes a contiguous slice of the candidate planes.  The
// right buckets' suffix unions and the left buckets' prefix unions come
// from warp scans of the slices' unions; each lane then walks its slice
// (the right suffixes stored back in place), computing the cost
// sum(n_child * area_child / area_node) in the reference's double
// arithmetic with the 0.8 bonus for an empty side; the first strict
// minimum over all planes is the smallest (cost, plane) pair.
__global__ void k_score(Dev D, int64_t level_nodes) {
  const int64_t w = ((int64_t)blockIdx.x * kB + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= 3 * level_nodes) return;  // whole warps
  const int64_t node = w / 3;
  const int a = (int)(w - 3 * node);
  const int64_t s = D.heads[node];
  if (D.hleaf[s]) return;
  if (D.smask[s] & (1u << a)) {
    if (lane == 0) {
      D.bcost[3 * s + a] = INFINITY;
      D.bpos[3 * s + a] = 0.0;
    }
    return;
  }
  const int tries = D.htries[s];
  uint32_t *L = D.buckets + ((int64_t)D.cnt2[s] + (int64_t)(a * 3) * tries) * 7;
  uint32_t *M = L + (int64_t)tries * 7, *R = M + (int64_t)tries * 7;
  const int per = (tries + 31) / 32, i0 = min(tries, lane * per), i1 = min(tries, i0 + per);
  BoxN ls = box_empty(), rs = box_empty();
  for (int i = i0; i < i1; ++i) {
    box_unite(ls, box_keys(L + (int64_t)i * 7));
    box_unite(rs, box_keys(R + (int64_t)i * 7));
  }
  // inclusive prefix of the left slices, inclusive suffix of the right ones
  for (int o = 1; o < 32; o <<= 1) {
    const BoxN u = box_shfl_up(ls, o), d = box_shfl_down(rs, o);
    if (lane >= o) box_unite(ls, u);
    if (lane + o < 32) box_unite(rs, d);
  }
  BoxN lp = box_shfl_up(ls, 1), rp = box_shfl_down(rs, 1);  // exclusive
  if (lane == 0) lp = box_empty();
  if (lane == 31) rp = box_empty();
  // the right suffixes of the slice, stored back decoded
  for (int i = i1 - 1; i >= i0; --i) {
    uint32_t *r = R + (int64_t)i * 7;
    box_unite(rp, box_keys(r));
    for (int c = 0; c < 3; ++c) {
      r[c] = __float_as_uint(rp.lo[c]);
      r[3 + c] = __float_as_uint(rp.hi[c]);
    }
    r[6] = rp.n;
  }
  const float *nlo = D.hbox + s * 6, *nhi = nlo + 3;
  const double inv_area = __ddiv_rn(1.0, (double)area_f(nlo, nhi));
  double best = INFINITY;
  int bi = 0x7FFFFFFF;
  for (int i = i0; i < i1; ++i) {
    box_unite(lp, box_keys(L + (int64_t)i * 7));
    const BoxN m = box_keys(M + (int64_t)i * 7);
    const uint32_t *r = R + (int64_t)i * 7;
    float sl[3], sh[3];
    for (int c = 0; c < 3; ++c) {
      sl[c] = __uint_as_float(r[c]);
      sh[c] = __uint_as_float(r[3 + c]);
    }
    const uint32_t sn = r[6];
    const double p1 = min1(__dmul_rn(area_d(lp.lo, lp.hi), inv_area));
    const double p2 = min1(__dmul_rn(area_d(m.lo, m.hi), inv_area));
    const double p3 = min1(__dmul_rn(area_d(sl, sh), inv_area));
    double cost = __dadd_rn(__dadd_rn(__dmul_rn((double)lp.n, p1), __dmul_rn((double)m.n, p2)), __dmul_rn((double)sn, p3));
    if (lp.n == 0 || sn == 0) cost = __dmul_rn(cost, 0.8);
    if (cost < best) {
      best = cost;
      bi = i;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const double oc = __shfl_xor_sync(0xffffffffu, best, o);
    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (oc < best || (oc == best && oi < bi)) {
      best = oc;
      bi = oi;
    }
  }
  if (lane == 0) {
    D.bcost[3 * s + a] = best;
    if (bi < tries) {
      // min + i * (max - min) / tries, evaluated in float
      const float ext = __fsub_rn(nhi[a], nlo[a]);
      D.bpos[3 * s + a] = (double)__fadd_rn(nlo[a], __fdiv_rn(__fmul_rn((float)bi, ext), (float)tries));
    } else {
      D.bpos[3 * s + a] = 0.0;
    }
  }
}

// The split axis: the lowest of the axes with the least cost.
__global__ void k_choose(Dev D) {
  const int64_t s = (int64_t)blockIdx.x * kB + threadIdx.x;
  if (s >= D.n || D.seg[s].x != (int)s || D.hleaf[s]) return;
  const double c0 = D.bcost[3 * s], c1 = D.bcost[3 * s + 1], c2 = D.bcost[3 * s + 2];
  int a;
  if (c0 <= c1 && c0 <= c2)
    a = 0;
  else if (c1 <= c0 && c1 <= c2)
    a = 1;
  else
    a = 2;
  D.haxis[s] = a;
  D.hsplit[s] = D.bpos[3 * s + a];
  D.rflags[D.hid[s]] = (uint8_t)(a + 1);
}

// Classes of the partition (Node::Node, :644-673): 0 entirely below the
// split, 2 entirely above, 1 straddling; packed counts of the right class
// (low word) and of the others (high word) for the scan.
__global__ void k_classify(Dev D) {
  const int64_t s = (int64_t)blockIdx.x * kB + threadIdx.x;
  if (s > D.n) return;
  uint64_t v = 0;
  if (s < D.n) {
    const int b = D.seg[s].x;
    if (b >= 0 && !D.hleaf[b]) {
      const int a = D.haxis[b];
      const double split = D.hsplit[b];
      uint8_t c;
      if ((double)D.box[s * 6 + 3 + a] < split)
        c = 0;
      else if ((double)D.box[s * 6 + a] > split)
        c = 2;
      else
        c = 1;
      D.cls[s] = c;
      v = c == 2 ? 1ull : (1ull << 32);
    }
  }
  D.cnt[s] = v;
}

__device__ __forceinline__ uint32_t lo32(uint64_t v) { return (uint32_t)v; }
__device__ __forceinline__ uint32_t hi32(uint64_t v) { return (uint32_t)(v >> 32); }

// The back stream's runs (index u = e - 1 - slot): T[r] = u of its r-th
// element that is not right-class; J[r] = front index of the r-th
// right-class element of the front stream.
__global__ void k_runs(Dev D) {
  const int64_t s = (int64_t)blockIdx.x * kB + threadIdx.x;
  if (s >= D.n) return;
  const int2 g = D.seg[s];
  if (g.x < 0 || D.hleaf[g.x]) return;
  const uint32_t b = (uint32_t)g.x, e = (uint32_t)g.y;
  if (D.cls[s] == 2) {
    const uint32_t r = lo32(D.cnt[s]) - lo32(D.cnt[b]);
    D.jarr[b + r] = (uint32_t)s - b;
  } else {
    const uint32_t r = hi32(D.cnt[e]) - hi32(D.cnt[s + 1]);
    D.tarr[b + r] = e - 1 - (uint32_t)s;
  }
}

// Processing step of every element: the front element j comes after j
// front elements and the runs of the right-class front elements before it;
// a back element comes after its run's trigger and its run's earlier
// elements.  ord[b + step] = slot.
__device__ __forceinline__ uint32_t front_step(const Dev &D, uint32_t b, uint32_t j, uint32_t a, uint32_t cnt_n,
                                               uint32_t nn) {
  if (a == 0) return j;
  if (a - 1 < cnt_n) return j + D.tarr[b + a - 1] + 1;
  return nn + 1;  // more triggers than runs: never reached
}
__global__ void k_steps(Dev D) {
  const int64_t s = (int64_t)blockIdx.x * kB + threadIdx.x;
  if (s >= D.n) return;
  const int2 g = D.seg[s];
  if (g.x < 0 || D.hleaf[g.x]) return;
  const uint32_t b = (uint32_t)g.x, e = (uint32_t)g.y, nn = e - b, j = (uint32_t)s - b;
  const uint64_t cb = D.cnt[b], ce = D.cnt[e];
  const uint32_t cnt_n = hi32(ce) - hi32(cb), cnt_r = lo32(ce) - lo32(cb);
  uint32_t step = front_step(D, b, j, lo32(D.cnt[s]) - lo32(cb), cnt_n, nn);
  if (step >= nn) {
    const uint32_t u = e - 1 - (uint32_t)s;
    const uint32_t r = hi32(ce) - hi32(D.cnt[s + 1]);
    const uint32_t start = r == 0 ? 0u : D.tarr[b + r - 1] + 1;
    step = 0xFFFFFFFFu;
    if (r < cnt_r) {
      const uint32_t jr = D.jarr[b + r];
      const uint32_t sr = front_step(D, b, jr, r, cnt_n, nn);
      if (sr < nn) step = sr + 1 + (u - start);
    }
  }
  if (step >= nn) {
    atomicOr(D.err, 1);
    return;
  }
  D.ord[b + step] = (uint32_t)s;
}

// Every position of an internal node must have received an element.
__global__ void k_steps_check(Dev D) {
  const int64_t p = (int64_t)blockIdx.x * kB + threadIdx.x;
  if (p >= D.n) return;
  const int b = D.seg[p].x;
  if (b >= 0 && !D.hleaf[b] && D.ord[p] == 0xFFFFFFFFu) atomicOr(D.err, 2);
}

// In processing order: packed counts (left, right) and (left or middle, 0).
__global__ void k_order_flags(Dev D) {
  const int64_t p = (int64_t)blockIdx.x * kB + threadIdx.x;
  if (p > D.n) return;
  uint64_t v = 0, w = 0;
  if (p < D.n) {
    const int b = D.seg[p].x;
    const uint32_t s = b >= 0 && !D.hleaf[b] ? D.ord[p] : 0xFFFFFFFFu;
    if (s < (uint64_t)D.n) {  // (an unfilled position is already an error)
      const uint8_t c = D.cls[s];
      v = c == 0 ? 1ull : (c == 2 ? (1ull << 32) : 0ull);
      w = c != 2 ? 1ull : 0ull;
    }
  }
  D.cnt2[p] = v;
  D.cnt3[p] = w;
}

// Destinations: the r-th left element (in processing order) to b + r, the
// r-th right one to e - 1 - r; I[r] = elements of the left-or-middle
// classes processed before the r-th left one (the block's end when it
// moves the middle block's front); a middle element starts at the block
// position lm = left-or-middle elements before it.
__global__ void k_dest(Dev D) {
  const int64_t p = (int64_t)blockIdx.x * kB + threadIdx.x;
  if (p >= D.n) return;
  const int2 g = D.seg[p];
  if (g.x < 0 || D.hleaf[g.x]) return;
  const uint32_t b = (uint32_t)g.x, e = (uint32_t)g.y;
  const uint64_t cb = D.cnt2[b], cp = D.cnt2[p];
  const uint32_t rl = lo32(cp) - lo32(cb), rr = hi32(cp) - hi32(cb);
  const uint32_t lm = (uint32_t)(D.cnt3[p] - D.cnt3[b]);
  const uint32_t s = D.ord[p];
  if (s >= (uint64_t)D.n) return;
  const uint8_t c = D.cls[s];
  if (c == 0) {
    D.dest[s] = b + rl;
    D.iarr[b + rl] = lm;
  } else if (c == 2) {
    D.dest[s] = e - 1 - rr;
  } else {
    D.lmb[p] = lm;
  }
  if (p == b) {
    const uint64_t ce = D.cnt2[e];
    D.hnl[b] = lo32(ce) - lo32(cb);
    D.hnr[b] = hi32(ce) - hi32(cb);
  }
}

// The middle block's moves as a function on block positions: a position
// below the number of left elements moves to I of it, the others stay.
__global__ void k_jump_init(Dev D) {
  const int64_t p = (int64_t)blockIdx.x * kB + threadIdx.x;
  if (p >= D.n) return;
  const int b = D.seg[p].x;
  if (b < 0 || D.hleaf[b]) return;
  const uint32_t x = (uint32_t)p - (uint32_t)b;
  D.f0[p] = x < D.hnl[b] ? D.iarr[p] : x;
}
__global__ void k_jump(Dev D, const uint32_t *__restrict__ fin, uint32_t *__restrict__ fout) {
  const int64_t p = (int64_t)blockIdx.x * kB + threadIdx.x;
  if (p >= D.n) return;
  const int2 g = D.seg[p];
  if (g.x < 0 || D.hleaf[g.x]) return;
  const uint32_t v = fin[p];
  if (v >= (uint32_t)(g.y - g.x)) {  // only after an inconsistent step map
    atomicOr(D.err, 4);
    fout[p] = v;
    return;
  }
  fout[p] = fin[(uint32_t)g.x + v];
}
__global__ void k_dest_middle(Dev D, const uint32_t *__restrict__ f) {
  const int64_t p = (int64_t)blockIdx.x * kB + threadIdx.x;
  if (p >= D.n) return;
  const int b = D.seg[p].x;
  if (b < 0 || D.hleaf[b]) return;
  const uint32_t s = D.ord[p];
  if (s >= (uint64_t)D.n || D.cls[s] != 1) return;
  const uint32_t x = D.lmb[p], nn = (uint32_t)(D.seg[p].y - b);
  const uint32_t d = x < nn ? f[(uint32_t)b + x] : 0xFFFFFFFFu;
  if (d >= nn) {
    atomicOr(D.err, 4);
    return;
  }
  D.dest[s] = (uint32_t)b + d;
}

__global__ void k_scatter(Dev D) {
  const int64_t s = (int64_t)blockIdx.x * kB + threadIdx.x;
  if (s >= D.n) return;
  const int2 g = D.seg[s];
  const int64_t d = (g.x >= 0 && !D.hleaf[g.x]) ? (int64_t)D.dest[s] : s;
  if (d < g.x || (g.x >= 0 && d >= g.y) || d >= D.n) {  // unset: only after an inconsistent step map
    atomicOr(D.err, 8);
    return;
  }
  for (int c = 0; c < 6; ++c) D.box2[d * 6 + c] = D.box[s * 6 + c];
  D.perm2[d] = D.perm[s];
}

// Next level's node of every position (in the partitioned order): the
// left, middle or right child's range, its middle-split axes and parent.
__global__ void k_children(Dev D) {
  const int64_t p = (int64_t)blockIdx.x * kB + threadIdx.x;
  if (p >= D.n) return;
  const int2 g = D.seg[p];
  if (g.x < 0) return;
  if (D.hleaf[g.x]) {
    D.seg[p] = make_int2(-1, -1);
    return;
  }
  const int b = g.x, e = g.y;
  const int l = b + (int)D.hnl[b], r = e - (int)D.hnr[b];
  D.spar[p] = D.hid[b];
  if ((int)p < l) {
    D.seg[p] = make_int2(b, l);
    D.sord[p] = 0;
  } else if ((int)p < r) {
    D.seg[p] = make_int2(l, r);
    D.sord[p] = 1;
    D.smask[p] = (uint8_t)(D.smask[p] | (1u << D.haxis[b]));
  } else {
    D.seg[p] = make_int2(r, e);
    D.sord[p] = 2;
  }
}

inline size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

cudaError_t build_accel_tree_gpu(const float *tbox, int64_t n, cudaStream_t st, AccelTreeGpu &out) {
  out = AccelTreeGpu();
  if (n <= 0 || n > (int64_t)INT32_MAX / 2) return cudaErrorInvalidValue;
  Dev D{};
  D.n = n;
  const size_t n1 = (size_t)n + 1, nb = (n1 + kB - 1) / kB;
  size_t total = 0;
  std::vector<std::pair<void **, size_t>> plan;
  auto want = [&](void *pp, size_t bytes) {
    plan.push_back({(void **)pp, bytes});
    total += al256(bytes);
  };
  const size_t nn = (size_t)n;
  want(&D.box, nn * 24);
  want(&D.box2, nn * 24);
  want(&D.perm, nn * 4);
  want(&D.perm2, nn * 4);
  want(&D.seg, nn * 8);
  want(&D.smask, nn);
  want(&D.sord, nn);
  want(&D.spar, nn * 4);
  want(&D.hkeys, nn * 48);
  want(&D.hbox, nn * 24);
  want(&D.hcoef, nn * 24);
  want(&D.hsplit, nn * 8);
  want(&D.hid, nn * 4);
  want(&D.heads, nn * 4);
  want(&D.htries, nn * 4);
  want(&D.haxis, nn * 4);
  want(&D.hnl, nn * 4);
  want(&D.hnr, nn * 4);
  want(&D.hleaf, nn);
  want(&D.bcost, nn * 24);
  want(&D.bpos, nn * 24);
  // buckets: sum over internal nodes of 9 min(200, 2 count) <= 18 n
  want(&D.buckets, nn * 18 * 28);
  want(&D.cls, nn);
  want(&D.cnt, n1 * 8);
  want(&D.cnt2, n1 * 8);
  want(&D.cnt3, n1 * 8);
  want(&D.sums, nb * 8);
  want(&D.tarr, nn * 4);
  want(&D.jarr, nn * 4);
  want(&D.ord, nn * 4);
  want(&D.iarr, nn * 4);
  want(&D.f0, nn * 4);
  want(&D.f1, nn * 4);
  want(&D.lmb, nn * 4);
  want(&D.dest, nn * 4);
  want(&D.err, 256);
  want(&D.maxseg, 256);
  want(&D.n_leaves, 256);
  char *arena = nullptr;
  cudaError_t e = cudaMalloc(&arena, total);
  if (e != cudaSuccess) return e;
  {
    char *w = arena;
    for (auto &pr : plan) {
      *pr.first = w;
      w += al256(pr.second);
    }
  }
  // node records, grown as levels add nodes
  int64_t cap = 0, n_nodes = 0;
  auto grow = [&](int64_t need) -> cudaError_t {
    if (need <= cap) return cudaSuccess;
    int64_t nc = std::max<int64_t>(need, cap + cap / 2 + (int64_t)1024);
    float *rbox = nullptr;
    uint32_t *rtb = nullptr, *rte = nullptr;
    uint8_t *rflags = nullptr;
    int32_t *rchild = nullptr;
    cudaError_t g;
    if ((g = cudaMalloc(&rbox, (size_t)nc * 24)) != cudaSuccess || (g = cudaMalloc(&rtb, (size_t)nc * 4)) != cudaSuccess ||
        (g = cudaMalloc(&rte, (size_t)nc * 4)) != cudaSuccess || (g = cudaMalloc(&rflags, (size_t)nc)) != cudaSuccess ||
        (g = cudaMalloc(&rchild, (size_t)nc * 12)) != cudaSuccess) {
      cudaFree(rbox);
      cudaFree(rtb);
      cudaFree(rte);
      cudaFree(rflags);
      cudaFree(rchild);
      return g;
    }
    if (n_nodes > 0) {
      cudaMemcpyAsync(rbox, D.rbox, (size_t)n_nodes * 24, cudaMemcpyDeviceToDevice, st);
      cudaMemcpyAsync(rtb, D.rtb, (size_t)n_nodes * 4, cudaMemcpyDeviceToDevice, st);
      cudaMemcpyAsync(rte, D.rte, (size_t)n_nodes * 4, cudaMemcpyDeviceToDevice, st);
      cudaMemcpyAsync(rflags, D.rflags, (size_t)n_nodes, cudaMemcpyDeviceToDevice, st);
      cudaMemcpyAsync(rchild, D.rchild, (size_t)n_nodes * 12, cudaMemcpyDeviceToDevice, st);
    }
    if ((g = cudaStreamSynchronize(st)) != cudaSuccess) return g;
    cudaFree(D.rbox);
    cudaFree(D.rtb);
    cudaFree(D.rte);
    cudaFree(D.rflags);
    cudaFree(D.rchild);
    D.rbox = rbox;
    D.rtb = rtb;
    D.rte = rte;
    D.rflags = rflags;
    D.rchild = rchild;
    cap = nc;
    return cudaSuccess;
  };
  auto release = [&]() {
    cudaFree(D.rbox);
    cudaFree(D.rtb);
    cudaFree(D.rte);
    cudaFree(D.rflags);
    cudaFree(D.rchild);
    cudaFree(arena);
  };
  float *d_tbox = nullptr;
  uint64_t *h_count = nullptr;
  if ((e = cudaMalloc(&d_tbox, nn * 24)) != cudaSuccess || (e = cudaMallocHost(&h_count, 16)) != cudaSuccess) {
    cudaFree(d_tbox);
    release();
    return e;
  }
  const unsigned gn = grid_of(n), gn1 = grid_of((int64_t)n1);
  e = cudaMemcpyAsync(d_tbox, tbox, nn * 24, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(D.err, 0, 4, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(D.n_leaves, 0, 8, st);
  if (e == cudaSuccess) e = grow(std::max<int64_t>(2 * n, 1024));
  if (e == cudaSuccess) {
    k_init<<<gn, kB, 0, st>>>(D, d_tbox);
    e = cudaGetLastError();
  }
  int depth = 0;
  for (; e == cudaSuccess; ++depth) {
    if ((e = cudaMemsetAsync(D.maxseg, 0, 4, st)) != cudaSuccess) break;
    k_heads<<<gn1, kB, 0, st>>>(D);
    if ((e = scan64(D.cnt, (int64_t)n1, D.sums, st)) != cudaSuccess) break;
    if ((e = cudaMemcpyAsync(h_count, D.cnt + n, 8, cudaMemcpyDeviceToHost, st)) != cudaSuccess) break;
    if ((e = cudaMemcpyAsync(h_count + 1, D.err, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess) break;
    if ((e = cudaMemcpyAsync((char *)(h_count + 1) + 4, D.maxseg, 4, cudaMemcpyDeviceToHost, st)) != cudaSuccess) break;
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) break;
    const int64_t level_nodes = (int64_t)h_count[0];
    if (level_nodes == 0 || (uint32_t)h_count[1] != 0) break;
    // a middle element's chain stays inside its node: 2^rounds >= its size
    const int64_t maxseg = (int64_t)(h_count[1] >> 32);
    int rounds = 1;
    while (((int64_t)1 << rounds) < maxseg) ++rounds;
    if ((e = grow(n_nodes + level_nodes)) != cudaSuccess) break;
    k_node_box<<<gn, kB, 0, st>>>(D);
    k_head_setup<<<gn1, kB, 0, st>>>(D, n_nodes, depth);
    n_nodes += level_nodes;
    if ((e = scan64(D.cnt2, (int64_t)n1, D.sums, st)) != cudaSuccess) break;
    k_bucket_init<<<4096, kB, 0, st>>>(D);
    k_bucket_fill<<<gn, kB, 0, st>>>(D);
    k_score<<<grid_of(3 * 32 * level_nodes), kB, 0, st>>>(D, level_nodes);
    k_choose<<<gn, kB, 0, st>>>(D);
    k_classify<<<gn1, kB, 0, st>>>(D);
    if ((e = scan64(D.cnt, (int64_t)n1, D.sums, st)) != cudaSuccess) break;
    k_runs<<<gn, kB, 0, st>>>(D);
    if ((e = cudaMemsetAsync(D.ord, 0xFF, nn * 4, st)) != cudaSuccess) break;
    if ((e = cudaMemsetAsync(D.dest, 0xFF, nn * 4, st)) != cudaSuccess) break;
    k_steps<<<gn, kB, 0, st>>>(D);
    k_steps_check<<<gn, kB, 0, st>>>(D);
    k_order_flags<<<gn1, kB, 0, st>>>(D);
    if ((e = scan64(D.cnt2, (int64_t)n1, D.sums, st)) != cudaSuccess) break;
    if ((e = scan64(D.cnt3, (int64_t)n1, D.sums, st)) != cudaSuccess) break;
    k_dest<<<gn, kB, 0, st>>>(D);
    k_jump_init<<<gn, kB, 0, st>>>(D);
    uint32_t *fa = D.f0, *fb = D.f1;
    for (int r = 0; r < rounds; ++r) {
      k_jump<<<gn, kB, 0, st>>>(D, fa, fb);
      std::swap(fa, fb);
    }
    k_dest_middle<<<gn, kB, 0, st>>>(D, fa);
    k_scatter<<<gn, kB, 0, st>>>(D);
    std::swap(D.box, D.box2);
    std::swap(D.perm, D.perm2);
    k_children<<<gn, kB, 0, st>>>(D);
    e = cudaGetLastError();
  }
  int err_flag = 0;
  unsigned long long leaves = 0;
  if (e == cudaSuccess) {
    out.box.resize((size_t)n_nodes * 6);
    out.tb.resize((size_t)n_nodes);
    out.te.resize((size_t)n_nodes);
    out.flags.resize((size_t)n_nodes);
    out.child.resize((size_t)n_nodes * 3);
    out.perm.resize(nn);
    if ((e = cudaMemcpyAsync(out.box.data(), D.rbox, (size_t)n_nodes * 24, cudaMemcpyDeviceToHost, st)) == cudaSuccess &&
        (e = cudaMemcpyAsync(out.tb.data(), D.rtb, (size_t)n_nodes * 4, cudaMemcpyDeviceToHost, st)) == cudaSuccess &&
        (e = cudaMemcpyAsync(out.te.data(), D.rte, (size_t)n_nodes * 4, cudaMemcpyDeviceToHost, st)) == cudaSuccess &&
        (e = cudaMemcpyAsync(out.flags.data(), D.rflags, (size_t)n_nodes, cudaMemcpyDeviceToHost, st)) == cudaSuccess &&
        (e = cudaMemcpyAsync(out.child.data(), D.rchild, (size_t)n_nodes * 12, cudaMemcpyDeviceToHost, st)) ==
            cudaSuccess &&
        (e = cudaMemcpyAsync(out.perm.data(), D.perm, nn * 4, cudaMemcpyDeviceToHost, st)) == cudaSuccess &&
        (e = cudaMemcpyAsync(&err_flag, D.err, 4, cudaMemcpyDeviceToHost, st)) == cudaSuccess &&
        (e = cudaMemcpyAsync(&leaves, D.n_leaves, 8, cudaMemcpyDeviceToHost, st)) == cudaSuccess)
      e = cudaStreamSynchronize(st);
  }
  out.n_nodes = n_nodes;
  out.max_depth = depth - 1;
  out.n_leaves = (int64_t)leaves;
  out.inconsistent = err_flag != 0;
  cudaFree(d_tbox);
  cudaFreeHost(h_count);
  release();
  return e;
}

}  // namespace skw
