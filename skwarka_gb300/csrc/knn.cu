// Photon kd-tree lookups on sm_103a: filtered k-nearest neighbours
// (KDTree::GetNearestPoints with PhotonFilter) and the nearest point
// (KDTree::GetNearestPoint), one query per thread.
//
// Restated from Raytracer/Core/KDTree.h:
//   * _Lookup (:537-576): visit a node's own point, then the child on the
//     query's side of the split, then the other child if the squared plane
//     distance is below the current search radius -- tested after the near
//     subtree is done.  The recursion becomes an explicit stack whose entries
//     carry the plane distance, re-tested on pop against the radius of that
//     moment, which is exactly when the reference tests it.
//   * distances in double from float positions and a double query
//     (:547-550), compared with strict "<" against the radius;
//   * NearestPointsProc (:331-387): the filter runs first; the first k
//     accepted points fill an unordered array that becomes a max-heap
//     (ordered by squared distance, ties by array position = the reference's
//     pointer order); afterwards each accepted point replaces the heap top.
//     The heap routines below are the classic binary-heap algorithms in the
//     same form as the C++ library's make/pop/push_heap (sift the hole to the
//     bottom, then sift the value up), so that not only the index sets but
//     the output order match the reference.
//   * PhotonFilter (PhotonInternalTypes.h:113-137): the photon's normal (from
//     the 16-bit direction table) within the cosine threshold of the surface
//     normal, and the photon near the surface's tangent plane.
// Double products and sums use round-to-nearest intrinsics so that no fused
// multiply-add changes a result.
//
// Layout: 16-byte nodes (x, y, z, word) read with one vector load; the
// photon normal ids (uint16) are read only for points inside the radius.
// The walk stack lives in shared memory; for k <= 128 the heap (8-byte
// entries: float key, tree position) lives in local memory, larger k use a
// heap in a caller-provided global scratch buffer of k entries per query.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "kernels.h"

// Scratch of the allocation-free k-NN entry point (skw_knn_noalloc): heaps
// of SKW_KNN_NOALLOC_ENTRIES 16-byte entries (16 MiB), allocated with the
// module on every GPU that loads this library and held until the process
// exits.  Host code must not pass this symbol to a kernel (in host code it
// is only a stand-in for the device address); knn_noalloc_scratch() looks
// the device address up.
#define SKW_KNN_NOALLOC_ENTRIES (1 << 20)
static __device__ __align__(256) unsigned char g_knn_noalloc_scratch[(size_t)SKW_KNN_NOALLOC_ENTRIES * 16];

namespace skw {
namespace {

// One warp per block: a block's slot frees as soon as its warp's slowest
// query ends (queries differ widely in cost), and small blocks let the
// walk stack's shared memory be sized to fit, leaving the rest of the SM's
// storage to L1 (measured on the k = 100 photon lookups, 2,971,920 queries:
// 128 threads 34.3 ms, 32 threads 32.7 ms).
#ifndef SKW_KNN_BLOCK
#define SKW_KNN_BLOCK 32
#endif
constexpr int kKnnBlock = SKW_KNN_BLOCK;  // threads per block of the lookup kernels
// Load the near child's node as soon as the node word is read, so that the
// load overlaps the node's own distance, filter and heap work (off: at one
// warp per block it measured slower, 42.4 against 32.7 ms, at 128 threads
// the same).
#ifndef SKW_KNN_EARLY
#define SKW_KNN_EARLY 0
#endif
constexpr bool kEarlyLoad = SKW_KNN_EARLY != 0;
// minimum resident blocks per SM of k_knn: 32 one-warp blocks bound its
// registers at 64 (with 128-thread blocks, measured on the k = 100 photon
// lookups: 72 registers 57 ms, 64 50.5 ms, 48 58.5 ms)
#ifndef SKW_KNN_MINB
#define SKW_KNN_MINB (1024 / SKW_KNN_BLOCK)
#endif


struct Query {
  double q[3];
  double n[3];
  double cos_t, sin_t;
  bool filter;
  float qf[3];  // q rounded to float
  float eq;     // max |q - qf| over the axes
  bool qle[3];  // q <= qf on the axis (decides q <= split when split == qf)
  float nf[3];  // the normal in float (filter pre-test)
  float cos_f, sin_f;  // cos_t, sin_t in float (filter pre-test)
  float ke0, ke1;      // error bound of a float squared distance k: ke0 + ke1 k (key_err)
};

// Fills the float copy of the query point used by the pre-tests.
__device__ __forceinline__ void query_float(Query &Q) {
  float e = 0.0f;
  for (int k = 0; k < 3; ++k) {
    Q.qf[k] = (float)Q.q[k];
    Q.qle[k] = Q.q[k] <= (double)Q.qf[k];
    e = fmaxf(e, (float)fabs(Q.q[k] - (double)Q.qf[k]));
    Q.nf[k] = (float)Q.n[k];
  }
  Q.eq = e * 1.0001f;
  Q.ke0 = 1.001f * (Q.eq + 9.0f * Q.eq * Q.eq) + 1e-37f;
  Q.ke1 = 3.003f * Q.eq + 6.0e-7f;
  Q.cos_f = (float)Q.cos_t;
  Q.sin_f = (float)Q.sin_t;
}

// Coordinates of the query by a run-time axis, selected without indexing so
// that the query stays in registers.
__device__ __forceinline__ float qf_at(const Query &Q, uint32_t a) {
  return a == 0 ? Q.qf[0] : (a == 1 ? Q.qf[1] : Q.qf[2]);
}
__device__ __forceinline__ double q_at(const Query &Q, uint32_t a) {
  return a == 0 ? Q.q[0] : (a == 1 ? Q.q[1] : Q.q[2]);
}

// q[axis] <= split for a float split, exactly, without double arithmetic:
// qf is the float nearest to q, so qf < split implies q < split and
// qf > split implies q > split.
__device__ __forceinline__ bool q_le_split(const Query &Q, uint32_t axis, float split) {
  const float qf = qf_at(Q, axis);
  return qf < split || (qf == split && (axis == 0 ? Q.qle[0] : (axis == 1 ? Q.qle[1] : Q.qle[2])));
}

// PhotonFilter::operator() (PhotonInternalTypes.h:127-133), with float
// pre-tests: the normal's cosine and the in-plane test are decided in float
// when they clear their thresholds by more than the float error (unit
// vectors: a few 1e-7), else in double as the reference computes them.
__device__ __forceinline__ bool photon_filter_exact(const Query &Q, const float4 p, uint16_t nid,
                                                    const double *__restrict__ dirs);
__device__ __forceinline__ bool photon_filter(const Query &Q, const float4 p, uint16_t nid,
                                              const double *__restrict__ dirs) {
  const float *dirs_f = reinterpret_cast<const float *>(dirs + (3 << 16));  // the table rounded to float
  const float nx = __ldg(dirs_f + 3 * nid), ny = __ldg(dirs_f + 3 * nid + 1), nz = __ldg(dirs_f + 3 * nid + 2);
  const float cf = nx * Q.nf[0] + ny * Q.nf[1] + nz * Q.nf[2];
  const float ct = Q.cos_f;
  if (cf < ct - 2e-6f) return false;
  if (cf > ct + 2e-6f) {
    // |to . n| < sin_t |to|, compared as squares when both sides clearly differ
    const float tx = p.x - Q.qf[0], ty = p.y - Q.qf[1], tz = p.z - Q.qf[2];
    const float dn = tx * Q.nf[0] + ty * Q.nf[1] + tz * Q.nf[2];
    const float l2 = tx * tx + ty * ty + tz * tz;
    const float st = Q.sin_f;
    const float lhs = dn * dn, rhs = st * st * l2;
    // error: the float query rounding eq on each component plus relative rounding
    const float a = fabsf(tx) + fabsf(ty) + fabsf(tz);
    // |d(dn)| <= 3 eq + 5e-7 a and |d(l2)| <= 2 a (eq + 6e-8 a) (a = |tx| + |ty| + |tz|), so
    // the squares move by at most 2 a |d(dn)| + |d(dn)|^2 and st^2 |d(l2)|
    const float err = 12.0f * Q.eq * (a + Q.eq) + 4e-6f * a * a + 2e-6f * (lhs + rhs) + 1e-37f;
    if (lhs + err < rhs) return true;
    if (lhs - err > rhs) return false;
  }
  return photon_filter_exact(Q, p, nid, dirs);
}

__device__ __forceinline__ bool photon_filter_exact(const Query &Q, const float4 p, uint16_t nid,
                                                    const double *__restrict__ dirs) {
  const double nx = __ldg(dirs + 3 * nid), ny = __ldg(dirs + 3 * nid + 1), nz = __ldg(dirs + 3 * nid + 2);
  const double cosn = __dadd_rn(__dadd_rn(__dmul_rn(nx, Q.n[0]), __dmul_rn(ny, Q.n[1])), __dmul_rn(nz, Q.n[2]));
  if (!(cosn > Q.cos_t)) return false;
  const double tx = __dsub_rn((double)p.x, Q.q[0]), ty = __dsub_rn((double)p.y, Q.q[1]),
               tz = __dsub_rn((double)p.z, Q.q[2]);
  const double dotn = __dadd_rn(__dadd_rn(__dmul_rn(tx, Q.n[0]), __dmul_rn(ty, Q.n[1])), __dmul_rn(tz, Q.n[2]));
  const double len = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(tx, tx), __dmul_rn(ty, ty)), __dmul_rn(tz, tz)));
  return fabs(dotn) < __dmul_rn(Q.sin_t, len);
}

__device__ __forceinline__ double point_d2(const float4 p, const Query &Q) {
  const double dx = __dsub_rn((double)p.x, Q.q[0]), dy = __dsub_rn((double)p.y, Q.q[1]),
               dz = __dsub_rn((double)p.z, Q.q[2]);
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// Float pre-tests.  A point's squared distance and a splitting plane's
// squared distance are first computed in float and compared with two
// thresholds derived from the current radius and a bound on the float
// value's distance from the reference's double value; only a value between
// the thresholds is decided in double.
// The float squared distance of a point from the float query, and a bound
// E(F) on its distance from the reference's double value, as a function of
// the float value F: with u = 2^-24, each float difference d within u|d| +
// eq of the exact one, its square, the fused sum's three roundings and the
// double result's own rounding give
//   |F - d2| <= 5u D + 2 eq sum|d| + 3 eq^2 (+ 2^-52 D),  D = sum d^2 <= F (1 + 3u),
// and sum|d| <= sqrt(3 D):  E(F) = 3.0e-7 F + 3.47 eq sqrt(F) + 3.01 eq^2,
// plus 1e-37 for roundings in the subnormal range.  A plane's squared
// distance (one axis, one rounding fewer) is within the same bound.
__device__ __forceinline__ float dist2f(const float4 p, const Query &Q) {
  const float dx = p.x - Q.qf[0], dy = p.y - Q.qf[1], dz = p.z - Q.qf[2];
  return fmaf(dz, dz, fmaf(dy, dy, dx * dx));
}
__device__ __forceinline__ float d2_err(const Query &Q, float x) {
  // 1.0001: the roundings of this float evaluation (about 6u)
  return (3.0e-7f * x + 3.47f * Q.eq * __fsqrt_ru(x) + 3.01f * Q.eq * Q.eq + 1e-37f) * 1.0001f;
}
// Thresholds on a float squared distance F against a radius known to lie
// in [rlo, rhi]: F < tin => inside, F >= tout => outside (else decide in
// double).  tin = rlo - E(rlo): for F < tin, F + E(F) < rlo because E grows
// with F.  tout = rhi + E(2 rhi): for F in [tout, 2 rhi], F - E(F) >= rhi;
// above 2 rhi, E(F) <= F / 2 <= F - rhi once sqrt(rhi) >= 8 eq; below that
// (or for an infinite radius) nothing is decided outside in float.
__device__ __forceinline__ void radius_thresholds(const Query &Q, float rlo, float rhi, float &tin, float &tout) {
  tin = isinf(rlo) ? rlo : (rlo > 0.0f ? __fsub_rd(rlo, d2_err(Q, rlo)) : -1.0f);
  const float two = 2.0f * rhi;
  tout = (!isinf(two) && rhi >= fmaxf(64.0f * Q.eq * Q.eq, 1e-36f)) ? __fadd_ru(rhi, d2_err(Q, two)) : INFINITY;
}

// A node's children in the reference's visit order: near = the child on the
// query's side of the split (visited next), far = the other (postponed and
// visited only if its plane is within the radius when it is popped); -1
// where a child is absent or the node is a leaf.
__device__ __forceinline__ void node_children(const float4 p, int cur, int n, const Query &Q, int &near, int &far,
                                              uint32_t &axis, float &split) {
  const uint32_t w = __float_as_uint(p.w);
  near = far = -1;
  axis = w & 3u;
  split = 0.0f;
  if (axis == 3u) return;
  split = axis == 0 ? p.x : (axis == 1 ? p.y : p.z);
  const uint32_t right = w >> 3;
  const bool has_left = (w & 4u) != 0u, has_right = right < (uint32_t)n;
  const bool le = q_le_split(Q, axis, split);
  const int l = has_left ? cur + 1 : -1, r = has_right ? (int)right : -1;
  near = le ? l : r;
  far = le ? r : l;
}

// Walks the tree in the reference's order, calling visit(ni, p, d2, maxd2)
// for every point with d2 < maxd2; visit returns true when it changed
// maxd2.  A point whose float distance is certainly inside the radius is
// visited with d2 = -1 (not computed): the exact double distance is only
// needed for the heap order, and the caller computes it later, many at a
// time (the exact distance is a chain of dependent double operations, slow
// on this GPU's FP64 pipe when done one point after another).  Returns
// nodes visited (for statistics) or -1 on stack overflow.
//
// The stack lives in shared memory ([entry][thread], so lanes never share a
// bank) and holds only the parent of each postponed far child: on pop the
// parent is read again (a recently visited node, usually still in L1) and
// its split gives both the far child and the plane distance to re-test.
// Shared memory and L1 share the SM's storage, and the walk's node and heap
// reads want the L1, so the stack is sized by the tree's depth: the
// median-split tree of n points is floor(log2 n) + 1 levels deep and the
// walk holds at most one entry per level, so S = 20 serves n < 2^20 and
// S = 32 any n < 2^31.
template <int S, class Visit>
__device__ __forceinline__ int walk(const float4 *__restrict__ nodes, int n, const Query &Q, double &maxd2,
                                    uint32_t (*stk)[kKnnBlock], Visit &&visit) {
  if (n <= 0) return 0;
  int sp = 0, visited = 0;
  int cur = 0;
  // maxd2 in float, rounded down / up (a float below the lower one is below
  // maxd2, one at or above the upper one is not)
  auto lo_f = [](double m) { return __double2float_rd(m); };
  auto hi_f = [](double m) { return __double2float_ru(m); };
  float tin, tout;
  radius_thresholds(Q, lo_f(maxd2), hi_f(maxd2), tin, tout);
  float4 p = __ldg(nodes);
  for (;;) {
    ++visited;
    int near, far;
    uint32_t axis;
    float split;
    node_children(p, cur, n, Q, near, far, axis, split);
    float4 pn = p;
    if (kEarlyLoad && near >= 0) pn = __ldg(nodes + near);  // overlaps this node's work
    {
      const float d2f = dist2f(p, Q);
      if (d2f < tin) {  // certainly inside
        if (visit(cur, p, -1.0, maxd2)) radius_thresholds(Q, lo_f(maxd2), hi_f(maxd2), tin, tout);
      } else if (!(d2f >= tout)) {  // not certainly outside: decide exactly
        const double d2 = point_d2(p, Q);
        if (d2 < maxd2 && visit(cur, p, d2, maxd2)) radius_thresholds(Q, lo_f(maxd2), hi_f(maxd2), tin, tout);
      }
    }
    if (far >= 0) {  // the far child waits on the stack
      if (sp >= S) return -1;
      stk[sp][threadIdx.x] = (uint32_t)cur;
      ++sp;
    }
    if (near >= 0) {
      cur = near;
      p = kEarlyLoad ? pn : __ldg(nodes + near);
      continue;
    }
    int next = -1;
    while (sp > 0) {
      --sp;
      // the reference's pop test: (qa - split)^2 < maxd2, in double
      const uint32_t par = stk[sp][threadIdx.x];
      int pnear, pfar;
      uint32_t ax;
      float ps;
      const float4 pp = __ldg(nodes + par);
      node_children(pp, (int)par, n, Q, pnear, pfar, ax, ps);
      const float sd = qf_at(Q, ax) - ps, s2 = sd * sd;
      bool take;
      if (s2 < tin) {
        take = true;
      } else if (s2 >= tout) {
        take = false;
      } else {
        const double pd = __dsub_rn(q_at(Q, ax), (double)ps);
        take = __dmul_rn(pd, pd) < maxd2;
      }
      if (take) {
        next = pfar;
        break;
      }
    }
    if (next < 0) return visited;
    cur = next;
    p = __ldg(nodes + cur);
  }
}

// ------------------------------------------------------------ k_knn --
// The heap holds float squared distances: an entry's key is the float
// distance of its point, within key_err of the reference's double value.
// Heap comparisons are decided on the keys and their bounds, and only when
// two keys' intervals overlap are the exact doubles of both points computed
// (GB300 runs a double operation at ~1/64 of the float rate, and divergent
// double work in the former exact-keyed heap kept its FP64 pipe half busy);
// ties of exact distances go to the lower tree position, as the reference's
// NearestPoint comparison (KDTree.h:331-387) decides them.  So the heap
// takes the same branches as the reference's and its order is the
// reference's.  The search radius is max_dist^2 until the heap is full and
// then the top's exact distance, represented by a float bracket [rlo, rhi]
// and computed exactly on demand.  The exact distances of the output are
// computed at the end, four independent chains at a time.

// A heap entry: float squared distance and tree position.
struct FCand {
  float key;
  int32_t idx;
};

// Entries per query of a global heap: k + 1 rounded up to even.
__host__ __device__ __forceinline__ int64_t knn_heap_stride(int k) { return ((int64_t)k + 2) & ~(int64_t)1; }

// Bound on |key - d2| for a point whose float squared distance is key
// (dist2f): ke0 + ke1 key (Query::ke0, ke1) bounds the error derived
// above, 5u D + 2 sqrt(3) eq sqrt(D) + 3 eq^2, the square-root term by
// 2 sqrt(3) eq sqrt(key) <= 2 sqrt(1.001 eq * 3.003 eq key) <= 1.001 eq + 3.003 eq key.
__device__ __forceinline__ float key_err(const Query &Q, float key) { return fmaf(Q.ke1, key, Q.ke0); }

// (d2, idx) lexicographic on the exact distances, decided on the keys when
// their bounds do not overlap.
__device__ __forceinline__ bool fcand_less(const float4 *__restrict__ nodes, const Query &Q, const FCand &a,
                                           const FCand &b) {
  // decided when |a - b| exceeds both bounds (with a margin for this float arithmetic)
  const float d = a.key - b.key, tol = 1.0001f * fmaf(Q.ke1, a.key + b.key, 2.0f * Q.ke0);
  if (d < -tol) return true;
  if (d > tol) return false;
  const double da = point_d2(__ldg(nodes + a.idx), Q), db = point_d2(__ldg(nodes + b.idx), Q);
  return da == db ? a.idx < b.idx : da < db;
}

__device__ __forceinline__ void fheap_push_up(const float4 *__restrict__ nodes, const Query &Q, FCand *h, int hole, int top, FCand value) {
  int parent = (hole - 1) / 2;
  while (hole > top && fcand_less(nodes, Q, h[parent], value)) {
    h[hole] = h[parent];
    hole = parent;
    parent = (hole - 1) / 2;
  }
  h[hole] = value;
}

// PAIR: h[1] is 16-byte aligned, so that the children 2j+1, 2j+2 of every
// entry j share one 16-byte load.
template <bool PAIR = false>
__device__ __forceinline__ void fheap_adjust(const float4 *__restrict__ nodes, const Query &Q, FCand *h, int hole, int len, FCand value) {
  const int top = hole;
  int second = hole;
  while (second < (len - 1) / 2) {
    second = 2 * (second + 1);
    if (PAIR) {
      const uint4 two = *reinterpret_cast<const uint4 *>(h + second - 1);
      const FCand a{__uint_as_float(two.x), (int32_t)two.y}, b{__uint_as_float(two.z), (int32_t)two.w};
      const bool left = fcand_less(nodes, Q, b, a);
      second -= left ? 1 : 0;
      h[hole] = left ? a : b;
    } else {
      if (fcand_less(nodes, Q, h[second], h[second - 1])) second--;
      h[hole] = h[second];
    }
    hole = second;
  }
  if ((len & 1) == 0 && second == (len - 2) / 2) {
    second = 2 * (second + 1);
    h[hole] = h[second - 1];
    hole = second - 1;
  }
  fheap_push_up(nodes, Q, h, hole, top, value);
}

__device__ __forceinline__ void fheap_make(const float4 *__restrict__ nodes, const Query &Q, FCand *h, int len) {
  if (len < 2) return;
  for (int parent = (len - 2) / 2;; --parent) {
    fheap_adjust(nodes, Q, h, parent, len, h[parent]);
    if (parent == 0) return;
  }
}

// KMAX > 0: heap of KMAX entries in local memory.  KMAX == 0: the heap of
// query i is scratch[i * k ...].  Until the heap is full its entries are
// the accepted points in visit order (the reference's array holds them
// unordered); at k entries it becomes a heap.
template <int KMAX, int S>
__global__ void __launch_bounds__(kKnnBlock, SKW_KNN_MINB) k_knn(const float4 *__restrict__ nodes, const uint16_t *__restrict__ nids,
                                             const double *__restrict__ dirs, int n, const double *__restrict__ q,
                                             const double *__restrict__ qn, int64_t nq, int k, double max_dist,
                                             double cos_t, int32_t *__restrict__ out_idx,
                                             double *__restrict__ out_d2, int32_t *__restrict__ out_count,
                                             int32_t *__restrict__ out_visited, FCand *__restrict__ scratch,
                                             unsigned *__restrict__ status, const int *__restrict__ nq_dev,
                                             const int32_t *__restrict__ order) {
  __shared__ uint32_t stk[S][kKnnBlock];
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (nq_dev && *nq_dev < nq) nq = *nq_dev;
  if (i >= nq) return;
  if (order) i = order[i];
  Query Q;
  Q.q[0] = q[3 * i];
  Q.q[1] = q[3 * i + 1];
  Q.q[2] = q[3 * i + 2];
  Q.filter = cos_t >= 0.0;
  if (Q.filter) {
    Q.n[0] = qn[3 * i];
    Q.n[1] = qn[3 * i + 1];
    Q.n[2] = qn[3 * i + 2];
    Q.cos_t = cos_t;
    Q.sin_t = __dsqrt_rn(__dsub_rn(1.0, __dmul_rn(cos_t, cos_t)));
  } else {
    Q.n[0] = Q.n[1] = Q.n[2] = 0.0;
    Q.cos_t = Q.sin_t = 0.0;
  }
  query_float(Q);
  FCand local_heap[KMAX > 0 ? KMAX : 1];
  // global heaps: query i's entries from scratch[i * stride + 1], stride even
  // (16-byte aligned sibling pairs, fheap_adjust<true>)
  FCand *heap = KMAX > 0 ? local_heap : scratch + i * (int64_t)knn_heap_stride(k) + 1;
  int size = 0, visited = 0;
  if (k > 0 && n > 0) {
    // the search radius: max_dist^2 (KDTree::Lookup, KDTree.h:475-482)
    // until the heap is full, then the top's exact squared distance
    double rex = __dmul_rn(max_dist, max_dist);
    bool rex_ok = true;
    float rlo = __double2float_rd(rex), rhi = __double2float_ru(rex), tin, tout;
    radius_thresholds(Q, rlo, rhi, tin, tout);
    auto radius = [&]() -> double {
      if (!rex_ok) {
        rex = point_d2(__ldg(nodes + heap[0].idx), Q);
        rex_ok = true;
      }
      return rex;
    };
    auto new_top = [&]() {
      const float t = heap[0].key, e = key_err(Q, t);
      rlo = __fsub_rd(t, e);
      rhi = __fadd_ru(t, e);
      rex_ok = false;
      radius_thresholds(Q, rlo, rhi, tin, tout);
    };
    int sp = 0, cur = 0;
    bool overflow = false;
    float4 p = __ldg(nodes);
    for (;;) {
      ++visited;
      int near, far;
      uint32_t axis;
      float split;
      node_children(p, cur, n, Q, near, far, axis, split);
      // the near child is visited next: its node is loaded now, so that the
      // load overlaps this node's work
      float4 pn = p;
      if (kEarlyLoad && near >= 0) pn = __ldg(nodes + near);
      {
        const float d2f = dist2f(p, Q);
        bool inside;
        if (d2f < tin) {
          inside = true;
        } else if (d2f >= tout) {
          inside = false;
        } else {
          inside = point_d2(p, Q) < radius();
        }
        if (inside && (!Q.filter || photon_filter(Q, p, __ldg(nids + cur), dirs))) {
          const FCand c{d2f, cur};
          if (size < k) {
            heap[size++] = c;
            if (size == k) {
              fheap_make(nodes, Q, heap, k);
              new_top();
            }
          } else {
            // pop_heap: the top goes to the back; the back's old value is re-placed
            const FCand back = heap[k - 1];
            heap[k - 1] = heap[0];
            fheap_adjust<KMAX == 0>(nodes, Q, heap, 0, k - 1, back);
            // the popped back slot takes the new point, pushed up
            fheap_push_up(nodes, Q, heap, k - 1, 0, c);
            new_top();
          }
        }
      }
      if (far >= 0) {  // the far child waits on the stack
        if (sp >= S) {
          overflow = true;
          break;
        }
        stk[sp][threadIdx.x] = (uint32_t)cur;
        ++sp;
      }
      if (near >= 0) {
        cur = near;
        p = kEarlyLoad ? pn : __ldg(nodes + near);
        continue;
      }
      int next = -1;
      while (sp > 0) {
        --sp;
        // the reference's pop test: (qa - split)^2 < radius, in double
        const uint32_t par = stk[sp][threadIdx.x];
        int pnear, pfar;
        uint32_t ax;
        float ps;
        const float4 pp = __ldg(nodes + par);
        node_children(pp, (int)par, n, Q, pnear, pfar, ax, ps);
        const float sd = qf_at(Q, ax) - ps, s2 = sd * sd;
        bool take;
        if (s2 < tin) {
          take = true;
        } else if (s2 >= tout) {
          take = false;
        } else {
          const double pd = __dsub_rn(q_at(Q, ax), (double)ps);
          take = __dmul_rn(pd, pd) < radius();
        }
        if (take) {
          next = pfar;
          break;
        }
      }
      if (next < 0) break;
      cur = next;
      p = __ldg(nodes + cur);
    }
    if (overflow) atomicOr(status, 2u);
  }
  out_count[i] = size;
  // the exact squared distances of the output, four chains at a time
  int j = 0;
  for (; j + 4 <= size; j += 4) {
    const int32_t a0 = heap[j].idx, a1 = heap[j + 1].idx, a2 = heap[j + 2].idx, a3 = heap[j + 3].idx;
    const double d0 = point_d2(__ldg(nodes + a0), Q), d1 = point_d2(__ldg(nodes + a1), Q),
                 d2 = point_d2(__ldg(nodes + a2), Q), d3 = point_d2(__ldg(nodes + a3), Q);
    out_idx[i * k + j] = a0;
    out_idx[i * k + j + 1] = a1;
    out_idx[i * k + j + 2] = a2;
    out_idx[i * k + j + 3] = a3;
    out_d2[i * k + j] = d0;
    out_d2[i * k + j + 1] = d1;
    out_d2[i * k + j + 2] = d2;
    out_d2[i * k + j + 3] = d3;
  }
  for (; j < size; ++j) {
    out_idx[i * k + j] = heap[j].idx;
    out_d2[i * k + j] = point_d2(__ldg(nodes + heap[j].idx), Q);
  }
  for (; j < k; ++j) {
    out_idx[i * k + j] = -1;
    out_d2[i * k + j] = 0.0;
  }
  if (out_visited) out_visited[i] = visited;
}

// GetNearestPoint (KDTree.h:495-503) with NearestPointProc (:293-323):
// every accepted point becomes the nearest and shrinks the radius.
template <int S>
__global__ void __launch_bounds__(kKnnBlock, SKW_KNN_MINB) k_nearest(const float4 *__restrict__ nodes, const uint16_t *__restrict__ nids,
                                                 const double *__restrict__ dirs, int n,
                                                 const double *__restrict__ q, const double *__restrict__ qn,
                                                 int64_t nq, double max_dist, double cos_t,
                                                 int32_t *__restrict__ out_idx, unsigned *__restrict__ status,
                                                 const int *__restrict__ nq_dev, const int32_t *__restrict__ order) {
  __shared__ uint32_t stk[S][kKnnBlock];
  int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (nq_dev && *nq_dev < nq) nq = *nq_dev;
  if (i >= nq) return;
  if (order) i = order[i];
  Query Q;
  Q.q[0] = q[3 * i];
  Q.q[1] = q[3 * i + 1];
  Q.q[2] = q[3 * i + 2];
  Q.filter = cos_t >= 0.0;
  if (Q.filter) {
    Q.n[0] = qn[3 * i];
    Q.n[1] = qn[3 * i + 1];
    Q.n[2] = qn[3 * i + 2];
    Q.cos_t = cos_t;
    Q.sin_t = __dsqrt_rn(__dsub_rn(1.0, __dmul_rn(cos_t, cos_t)));
  } else {
    Q.n[0] = Q.n[1] = Q.n[2] = 0.0;
    Q.cos_t = Q.sin_t = 0.0;
  }
  query_float(Q);
  double maxd2 = __dmul_rn(max_dist, max_dist);
  int best = -1;
  const int v = walk<S>(nodes, n, Q, maxd2, stk, [&](int ni, const float4 p, double d2, double &md2) -> bool {
    if (Q.filter && !photon_filter(Q, p, __ldg(nids + ni), dirs)) return false;
    best = ni;
    md2 = d2 < 0.0 ? point_d2(p, Q) : d2;
    return true;
  });
  if (v < 0) atomicOr(status, 2u);
  out_idx[i] = best;
}

// Walk stack entries for a tree of n points (see walk).
constexpr int kShallowStack = 20;
inline bool shallow_tree(int n) { return n < (1 << kShallowStack); }

// k_knn<KMAX, S> with S chosen by the tree's depth.
template <int KMAX>
void knn_kernel(unsigned grid, cudaStream_t stream, const float4 *nodes, const uint16_t *nids, const double *dirs,
                int n, const double *q, const double *qn, int64_t nq, int k, double max_dist, double cos_t,
                int32_t *out_idx, double *out_d2, int32_t *out_count, int32_t *out_visited, FCand *scratch,
                unsigned *status, const int *nq_dev, const int32_t *order) {
  if (shallow_tree(n))
    k_knn<KMAX, kShallowStack><<<grid, kKnnBlock, 0, stream>>>(nodes, nids, dirs, n, q, qn, nq, k, max_dist, cos_t,
                                                               out_idx, out_d2, out_count, out_visited, scratch,
                                                               status, nq_dev, order);
  else
    k_knn<KMAX, 32><<<grid, kKnnBlock, 0, stream>>>(nodes, nids, dirs, n, q, qn, nq, k, max_dist, cos_t, out_idx,
                                                    out_d2, out_count, out_visited, scratch, status, nq_dev, order);
}

// Spatial bins of queries: a box cut into 64^3 cells, each query's cell as
// an 18-bit Morton code; a counting sort by cell (count, one exclusive scan,
// scatter) gives the order in which the lookup kernels take the queries, so
// that a warp's walks start near each other.  The order inside a cell
// follows the atomics; every query's answer is the same whichever thread
// computes it, and it is written at the query's own index.
constexpr int kBinBits = 6, kBins = 1 << (3 * kBinBits);
#ifndef SKW_KNN_SORT_BITS
#define SKW_KNN_SORT_BITS 6  // cell bits per axis of the sorted order (1..10)
#endif
constexpr int kSortCellBits = SKW_KNN_SORT_BITS;
static_assert(kSortCellBits >= 1 && kSortCellBits <= 10, "sorted cells: 1 to 10 bits per axis");

__device__ __forceinline__ uint32_t spread3(uint32_t v) {  // bit b of v (v < 2^10) to bit 3b
  uint32_t r = 0;
#pragma unroll
  for (int b = 0; b < 10; ++b) r |= ((v >> b) & 1u) << (3 * b);
  return r;
}

template <int BITS>
__global__ void k_bin_keys(const double *__restrict__ q, int64_t n, const int *__restrict__ count, float3 lo,
                           float3 scale, uint32_t *__restrict__ key, int *__restrict__ bins) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || (count && i >= *count)) return;
  const float c[3] = {((float)q[3 * i] - lo.x) * scale.x, ((float)q[3 * i + 1] - lo.y) * scale.y,
                      ((float)q[3 * i + 2] - lo.z) * scale.z};
  uint32_t k = 0;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float f = fminf(fmaxf(c[a], 0.0f), (float)((1 << BITS) - 1));  // NaN -> 0
    k |= spread3((uint32_t)f) << a;
  }
  key[i] = k;
  if (bins) atomicAdd(bins + k, 1);
}

// Exclusive scan of the kBins counts in place, one block of 1024 threads.
__global__ void __launch_bounds__(1024) k_bin_scan(int *__restrict__ bins) {
  constexpr int per = kBins / 1024;
  __shared__ int part[1024];
  int local[per];
  int sum = 0;
  for (int j = 0; j < per; ++j) {
    local[j] = sum;
    sum += bins[threadIdx.x * per + j];
  }
  part[threadIdx.x] = sum;
  __syncthreads();
  for (int off = 1; off < 1024; off <<= 1) {  // inclusive Hillis-Steele scan of the parts
    const int v = threadIdx.x >= (unsigned)off ? part[threadIdx.x - off] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  const int base = part[threadIdx.x] - sum;
  for (int j = 0; j < per; ++j) bins[threadIdx.x * per + j] = base + local[j];
}

__global__ void k_bin_scatter(const uint32_t *__restrict__ key, int64_t n, const int *__restrict__ count,
                              int *__restrict__ bins, int32_t *__restrict__ order) {
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || (count && i >= *count)) return;
  // the lanes of one cell take consecutive slots in lane order (one atomic
  // per cell and warp), so runs of neighbouring queries stay in order
  const uint32_t k = key[i];
  const unsigned grp = __match_any_sync(__activemask(), k);
  const int lane = threadIdx.x & 31, leader = __ffs(grp) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(bins + k, __popc(grp));
  base = __shfl_sync(grp, base, leader);
  order[base + __popc(grp & ((1u << lane) - 1u))] = (int32_t)i;
}

// A stable LSD radix sort of the cell keys (3 × SKW_KNN_SORT_BITS bits, 6-bit
// digits, one pass per digit) carrying the query indices: per block of 256 keys, each digit's
// count (lanes of a warp grouped by digit with __match_any_sync), one
// exclusive scan of the counts digit-major (all blocks of digit 0, then
// digit 1, ...), and a scatter that ranks a key after the block's earlier
// warps and the warp's earlier lanes with the same digit.  Stable, so the
// queries of a cell keep their image order.
constexpr int kSortBlock = 256, kDigitBits = 6, kDigits = 1 << kDigitBits;

__device__ __forceinline__ void digit_counts(uint32_t d, bool valid, unsigned &grp, int (*wcnt)[kDigits]) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  grp = __match_any_sync(0xffffffffu, valid ? d : 0xFFFFFFFFu);
  if (valid && lane == __ffs(grp) - 1) wcnt[w][d] = __popc(grp);
}

__global__ void __launch_bounds__(kSortBlock) k_sort_hist(const uint32_t *__restrict__ key, int64_t n, int shift,
                                                          uint64_t *__restrict__ hist, int64_t nblocks) {
  __shared__ int wcnt[kSortBlock / 32][kDigits];
  for (int j = threadIdx.x; j < (kSortBlock / 32) * kDigits; j += kSortBlock) (&wcnt[0][0])[j] = 0;
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * kSortBlock + threadIdx.x;
  const bool valid = i < n;
  const uint32_t d = valid ? (key[i] >> shift) & (kDigits - 1) : 0u;
  unsigned grp;
  digit_counts(d, valid, grp, wcnt);
  __syncthreads();
  if (threadIdx.x < kDigits) {
    int c = 0;
    for (int w = 0; w < kSortBlock / 32; ++w) c += wcnt[w][threadIdx.x];
    hist[(int64_t)threadIdx.x * nblocks + blockIdx.x] = (uint64_t)c;
  }
}

__global__ void __launch_bounds__(kSortBlock) k_sort_scatter(const uint32_t *__restrict__ key,
                                                             const int32_t *__restrict__ val, int64_t n, int shift,
                                                             const uint64_t *__restrict__ offs, int64_t nblocks,
                                                             uint32_t *__restrict__ key2, int32_t *__restrict__ val2) {
  __shared__ int wcnt[kSortBlock / 32][kDigits];
  for (int j = threadIdx.x; j < (kSortBlock / 32) * kDigits; j += kSortBlock) (&wcnt[0][0])[j] = 0;
  __syncthreads();
  const int64_t i = (int64_t)blockIdx.x * kSortBlock + threadIdx.x;
  const bool valid = i < n;
  const uint32_t k = valid ? key[i] : 0u, d = (k >> shift) & (kDigits - 1);
  unsigned grp;
  digit_counts(d, valid, grp, wcnt);
  __syncthreads();
  if (!valid) return;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int before = 0;
  for (int v = 0; v < w; ++v) before += wcnt[v][d];
  const int64_t dst = (int64_t)offs[(int64_t)d * nblocks + blockIdx.x] + before + __popc(grp & ((1u << lane) - 1u));
  key2[dst] = k;
  val2[dst] = val ? val[i] : (int32_t)i;
}

}  // namespace

int64_t bin_order_bins() { return kBins; }

size_t sort_order_bytes(int64_t n) {
  const int64_t nb = (n + kSortBlock - 1) / kSortBlock, m = nb * kDigits;
  auto al = [](int64_t x) { return (size_t)((x + 255) & ~(int64_t)255); };
  return 3 * al(n * 4) + al(m * 8) + al(((m + 255) / 256) * 8);
}

cudaError_t launch_sort_order(const double *q, int64_t n, const float lo[3], const float hi[3], void *scratch,
                              int32_t *order, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const int64_t nb = (n + kSortBlock - 1) / kSortBlock, m = nb * kDigits;
  auto al = [](int64_t x) { return (size_t)((x + 255) & ~(int64_t)255); };
  char *w = (char *)scratch;
  uint32_t *ka = (uint32_t *)w, *kb = (uint32_t *)(w + al(n * 4));
  int32_t *va = (int32_t *)(w + 2 * al(n * 4)), *vb = order;
  uint64_t *hist = (uint64_t *)(w + 3 * al(n * 4));
  uint64_t *sums = (uint64_t *)((char *)hist + al(m * 8));
  float sc[3];
  for (int a = 0; a < 3; ++a) {
    const float ext = hi[a] - lo[a];
    sc[a] = ext > 0.0f && ext < INFINITY ? (float)(1 << kSortCellBits) / ext : 0.0f;
  }
  k_bin_keys<kSortCellBits><<<(unsigned)((n + 255) / 256), 256, 0, st>>>(
      q, n, nullptr, make_float3(lo[0], lo[1], lo[2]), make_float3(sc[0], sc[1], sc[2]), ka, nullptr);
  // passes alternate ka/kb for the keys and va/vb for the indices, the
  // indices' parity chosen so that the last pass lands in order (vb)
  constexpr int passes = (3 * kSortCellBits + kDigitBits - 1) / kDigitBits;
  const int32_t *vin = nullptr;
  for (int pass = 0; pass < passes; ++pass) {
    const int shift = pass * kDigitBits;
    uint32_t *kin = pass % 2 ? kb : ka, *kout = pass % 2 ? ka : kb;
    int32_t *vout = (passes - 1 - pass) % 2 ? va : vb;
    k_sort_hist<<<(unsigned)nb, kSortBlock, 0, st>>>(kin, n, shift, hist, nb);
    cudaError_t e = scan64(hist, m, sums, st);
    if (e != cudaSuccess) return e;
    k_sort_scatter<<<(unsigned)nb, kSortBlock, 0, st>>>(kin, vin, n, shift, hist, nb, kout, vout);
    vin = vout;
  }
  return cudaGetLastError();
}

cudaError_t launch_bin_order(const double *q, int64_t n, const int *count_dev, const float lo[3], const float hi[3],
                             uint32_t *keys, int *bins, int32_t *order, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  float sc[3];
  for (int a = 0; a < 3; ++a) {
    const float ext = hi[a] - lo[a];
    sc[a] = ext > 0.0f && ext < INFINITY ? (float)(1 << kBinBits) / ext : 0.0f;
  }
  const unsigned grid = (unsigned)((n + 255) / 256);
  cudaError_t e = cudaMemsetAsync(bins, 0, (size_t)kBins * 4, st);
  if (e != cudaSuccess) return e;
  k_bin_keys<kBinBits><<<grid, 256, 0, st>>>(q, n, count_dev, make_float3(lo[0], lo[1], lo[2]),
                                   make_float3(sc[0], sc[1], sc[2]), keys, bins);
  k_bin_scan<<<1, 1024, 0, st>>>(bins);
  k_bin_scatter<<<grid, 256, 0, st>>>(keys, n, count_dev, bins, order);
  return cudaGetLastError();
}

#ifndef SKW_KNN_GHEAP
#define SKW_KNN_GHEAP 129  // smallest k whose heaps live in global scratch
#endif
size_t knn_scratch_bytes(int64_t nq, int k) {
  return k >= SKW_KNN_GHEAP ? (size_t)nq * (size_t)knn_heap_stride(k) * sizeof(FCand) : 0;
}

cudaError_t launch_knn(const void *nodes, const uint16_t *nids, const double *dirs, int n, const double *q,
                       const double *qn, int64_t nq, int k, double max_dist, double cos_t, int32_t *out_idx,
                       double *out_d2, int32_t *out_count, int32_t *out_visited, void *scratch, unsigned *status,
                       cudaStream_t stream, const int *nq_dev, const int32_t *order) {
  if (nq <= 0) return cudaSuccess;
  const int block = kKnnBlock;
  const unsigned grid = (unsigned)((nq + block - 1) / block);
  const float4 *nd = (const float4 *)nodes;
  if (scratch && k >= SKW_KNN_GHEAP) {
    knn_kernel<0>(grid, stream, nd, nids, dirs, n, q, qn, nq, k, max_dist, cos_t, out_idx, out_d2, out_count,
                  out_visited, (FCand *)scratch, status, nq_dev, order);
  } else if (k <= 32) {
    knn_kernel<32>(grid, stream, nd, nids, dirs, n, q, qn, nq, k, max_dist, cos_t, out_idx, out_d2, out_count,
                   out_visited, nullptr, status, nq_dev, order);
  } else if (k <= 128) {
    knn_kernel<128>(grid, stream, nd, nids, dirs, n, q, qn, nq, k, max_dist, cos_t, out_idx, out_d2, out_count,
                    out_visited, nullptr, status, nq_dev, order);
  } else {
    if (!scratch) return cudaErrorInvalidValue;
    knn_kernel<0>(grid, stream, nd, nids, dirs, n, q, qn, nq, k, max_dist, cos_t, out_idx, out_d2, out_count,
                  out_visited, (FCand *)scratch, status, nq_dev, order);
  }
  return cudaGetLastError();
}

int64_t knn_noalloc_capacity() { return SKW_KNN_NOALLOC_ENTRIES; }

// The calling thread's current CUDA context (the driver's cuCtxGetCurrent,
// reached through the runtime so that the library needs no link against the
// driver library); null where the driver does not offer it.
static void *current_context() {
  using Fn = CUresult (*)(CUcontext *);
  static const Fn fn = [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      p = nullptr;
    return (Fn)p;
  }();
  CUcontext c = nullptr;
  if (!fn || fn(&c) != CUDA_SUCCESS) return nullptr;
  return (void *)c;
}

// Device address of the static scratch for the current device, looked up
// once per device (cudaGetSymbolAddress with that device current; the first
// lookup may load this module on the device) and again whenever the
// device's current context has changed since (a device reset destroys the
// context and the module with it; the next context loads the module anew).
static cudaError_t knn_noalloc_scratch(void **out) {
  static std::mutex mu;
  static void *addr[64] = {nullptr};
  static void *owner[64] = {nullptr};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  // make the device's primary context current (a no-op when it already is)
  if ((e = cudaFree(nullptr)) != cudaSuccess) return e;
  void *ctx = current_context();
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev] || owner[dev] != ctx) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_knn_noalloc_scratch);
    if (e != cudaSuccess) return e;
    addr[dev] = p;
    owner[dev] = ctx;
  }
  *out = addr[dev];
  return cudaSuccess;
}

cudaError_t launch_knn_noalloc(const void *nodes, const uint16_t *nids, const double *dirs, int n, const double *q,
                               const double *qn, int64_t nq, int k, double max_dist, double cos_t,
                               int32_t *out_idx, double *out_d2, int32_t *out_count, unsigned *status,
                               cudaStream_t stream) {
  if (nq <= 0) return cudaSuccess;
  if (nq * (int64_t)k > SKW_KNN_NOALLOC_ENTRIES) return cudaErrorInvalidValue;
  void *scratch = nullptr;
  cudaError_t e = knn_noalloc_scratch(&scratch);
  if (e != cudaSuccess) return e;
  // Every heap slot is written before it is read, so the array needs no
  // clearing between calls.
  const int block = kKnnBlock;
  const unsigned grid = (unsigned)((nq + block - 1) / block);
  knn_kernel<0>(grid, stream, (const float4 *)nodes, nids, dirs, n, q, qn, nq, k, max_dist, cos_t, out_idx, out_d2,
                out_count, nullptr, (FCand *)scratch, status, nullptr, nullptr);
  return cudaGetLastError();
}

cudaError_t launch_nearest(const void *nodes, const uint16_t *nids, const double *dirs, int n, const double *q,
                           const double *qn, int64_t nq, double max_dist, double cos_t, int32_t *out_idx,
                           unsigned *status, cudaStream_t stream, const int *nq_dev, const int32_t *order) {
  if (nq <= 0) return cudaSuccess;
  const int block = kKnnBlock;
  const unsigned grid = (unsigned)((nq + block - 1) / block);
  if (shallow_tree(n))
    k_nearest<kShallowStack><<<grid, block, 0, stream>>>((const float4 *)nodes, nids, dirs, n, q, qn, nq, max_dist,
                                                         cos_t, out_idx, status, nq_dev, order);
  else
    k_nearest<32><<<grid, block, 0, stream>>>((const float4 *)nodes, nids, dirs, n, q, qn, nq, max_dist, cos_t,
                                              out_idx, status, nq_dev, order);
  return cudaGetLastError();
}

}  // namespace skw
