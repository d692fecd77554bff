// Photon kd-tree construction on the GPU: the same tree as the host's
// build_photon_tree (KDTree::_Build, Raytracer/Core/KDTree.h:428-473)
// wherever no node's median ties on its split axis.
//
// The reference's tree is a function of each node's point set when the
// median is unique: a node over positions [b, e) holds the point of rank
// m = floor((e - b) / 2) along the longest axis of the set's box (x, then y,
// then z on equal extents), its left subtree the points of smaller rank at
// [b + 1, b + m + 1), its right subtree the larger ones at [b + m + 1, e).
// (With ties at the median, which of the equal points std::nth_element puts
// at the median and how it splits the others is the standard library's own
// choice; the builder reports the tie nodes, and the host remakes their
// subtrees and the paths to them from the input order, repair_photon_tree.)
//
// GPU form: the points are sorted once per axis (a stable radix sort of
// order-preserving 32-bit keys, one bit per pass), then the tree is built
// level by level over the three sorted lists.  A node's box is the first
// and last key of its segment in each list; its median is the element of
// rank m in the split axis's list; every list is then stably partitioned
// within the segment into the left and right ranks (one packed 64-bit scan
// counts both), which keeps each child's segment sorted on every axis.  A
// level is a fixed sequence of launches over all positions; the number of
// levels follows from n alone, so nothing is read back until the end.
#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

#include "kernels.h"
#include "photon_tree.h"

namespace skw {
namespace {

constexpr int kBlock = 256;
constexpr uint32_t kNoRight = (1u << 29) - 1u;

__device__ __forceinline__ uint32_t fkey(float f) {  // order-preserving bits of a float
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// ------------------------------------------------------------ scans --
// Exclusive scan of n 64-bit values in three launches: per-block scans
// (warp shuffles) with the block totals, a one-block scan of the totals,
// and the totals added back.
__global__ void k_scan64_blocks(uint64_t *__restrict__ v, int64_t n, uint64_t *__restrict__ sums) {
  __shared__ uint64_t warp_tot[kBlock / 32];
  const int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  const uint64_t x = i < n ? v[i] : 0ull;
  uint64_t s = x;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int o = 1; o < 32; o <<= 1) {
    const uint64_t t = __shfl_up_sync(0xffffffffu, s, o);
    if (lane >= o) s += t;
  }
  if (lane == 31) warp_tot[w] = s;
  __syncthreads();
  if (w == 0) {
    uint64_t t = lane < kBlock / 32 ? warp_tot[lane] : 0ull;
    for (int o = 1; o < 32; o <<= 1) {
      const uint64_t u = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += u;
    }
    if (lane < kBlock / 32) warp_tot[lane] = t;  // inclusive
  }
  __syncthreads();
  const uint64_t before = w > 0 ? warp_tot[w - 1] : 0ull;
  if (i < n) v[i] = before + s - x;
  if (threadIdx.x == kBlock - 1) sums[blockIdx.x] = before + s;
}

__global__ void k_scan64_sums(uint64_t *__restrict__ sums, int nb) {
  __shared__ uint64_t part[1024];
  __shared__ uint64_t carry;
  if (threadIdx.x == 0) carry = 0ull;
  __syncthreads();
  for (int base = 0; base < nb; base += 1024) {
    const int i = base + threadIdx.x;
    const uint64_t x = i < nb ? sums[i] : 0ull;
    part[threadIdx.x] = x;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      const uint64_t t = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0ull;
      __syncthreads();
      part[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < nb) sums[i] = carry + part[threadIdx.x] - x;
    __syncthreads();
    if (threadIdx.x == 1023) carry += part[1023];
    __syncthreads();
  }
}

__global__ void k_scan64_add(uint64_t *__restrict__ v, int64_t n, const uint64_t *__restrict__ sums) {
  const int64_t i = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  if (i < n) v[i] += sums[blockIdx.x];
}

}  // namespace

cudaError_t scan64(uint64_t *v, int64_t n, uint64_t *sums, cudaStream_t st) {
  const int nb = (int)((n + kBlock - 1) / kBlock);
  k_scan64_blocks<<<nb, kBlock, 0, st>>>(v, n, sums);
  k_scan64_sums<<<1, 1024, 0, st>>>(sums, nb);
  k_scan64_add<<<nb, kBlock, 0, st>>>(v, n, sums);
  return cudaGetLastError();
}

namespace {

// ------------------------------------------------------------ sort --
// The three lists (axis a at [a n, a n + n)): key and point index.
__global__ void k_lists_init(const float *__restrict__ pos, int64_t n, uint32_t *__restrict__ key,
                             int32_t *__restrict__ id) {
  const int64_t q = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  if (q >= 3 * n) return;
  const int a = (int)(q / n);
  const int64_t i = q - a * n;
  key[q] = fkey(pos[3 * i + a]);
  id[q] = (int32_t)i;
}

// One stable split pass of the radix sort on bit `bit`: the zero flags.
__global__ void k_sort_flags(const uint32_t *__restrict__ key, int64_t m, int bit, uint64_t *__restrict__ cnt) {
  const int64_t q = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  if (q < m) cnt[q] = ((key[q] >> bit) & 1u) ? 0ull : 1ull;
}

// Scatter of the pass: zeros first, ones after, each in order, per list.
__global__ void k_sort_scatter(const uint32_t *__restrict__ key, const int32_t *__restrict__ id, int64_t n, int bit,
                               const uint64_t *__restrict__ excl, uint32_t *__restrict__ key2,
                               int32_t *__restrict__ id2) {
  const int64_t q = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  if (q >= 3 * n) return;
  const int a = (int)(q / n);
  const int64_t s = (int64_t)a * n, p = q - s;
  const uint64_t z0 = excl[s];
  const uint64_t zeros_before = excl[q] - z0;
  // zeros of the whole list: the scan at the next list's start, or the last element's
  const uint64_t zeros_total =
      (a < 2 ? excl[s + n] : excl[3 * n - 1] + (((key[3 * n - 1] >> bit) & 1u) ? 0ull : 1ull)) - z0;
  const uint32_t k = key[q];
  const int64_t dst = ((k >> bit) & 1u) ? s + (int64_t)zeros_total + (p - (int64_t)zeros_before)
                                        : s + (int64_t)zeros_before;
  key2[dst] = k;
  id2[dst] = id[q];
}

// ------------------------------------------------------------ levels --
// Segment of every position: seg[p] = (b, e), b = -1 once p's node is made.
// Heads (p == b) make their node: a leaf for a one-point segment, else the
// median of the longest axis (a tie at the median is counted in tie[0] and
// the first kTieCap tie nodes' positions kept in tie[1..]).
__global__ void k_level_nodes(const float *__restrict__ pos, int64_t n, const int2 *__restrict__ seg,
                              const int32_t *__restrict__ id, KdNode *__restrict__ nodes,
                              int32_t *__restrict__ perm, int *__restrict__ seg_axis, int *__restrict__ tie) {
  const int64_t p = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  if (p >= n) return;
  const int2 s = seg[p];
  if (s.x != (int)p) return;
  const int b = s.x, e = s.y;
  if (e - b == 1) {
    const int32_t i = id[b];
    nodes[b] = KdNode{pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], 3u};
    perm[b] = i;
    return;
  }
  double ext[3];
#pragma unroll
  for (int a = 0; a < 3; ++a)
    ext[a] = (double)pos[3 * id[a * n + e - 1] + a] - (double)pos[3 * id[a * n + b] + a];
  int axis = 0;
  if (ext[1] > ext[axis]) axis = 1;
  if (ext[2] > ext[axis]) axis = 2;
  const int m = (e - b) / 2, split = b + m;
  const int32_t *L = id + (int64_t)axis * n;
  const int32_t med = L[split];
  const float mk = pos[3 * med + axis];
  if ((m > 0 && pos[3 * L[split - 1] + axis] == mk) || (split + 1 < e && pos[3 * L[split + 1] + axis] == mk)) {
    const int slot = atomicAdd(tie, 1);
    if (slot < kTieCap) tie[1 + slot] = b;
  }
  const uint32_t right = split + 1 < e ? (uint32_t)(split + 1) : kNoRight;
  nodes[b] = KdNode{pos[3 * med], pos[3 * med + 1], pos[3 * med + 2], (right << 3) | 4u | (uint32_t)axis};
  perm[b] = med;
  seg_axis[b] = axis;
}

// Side of every point of an open segment: 0 left (rank < m), 1 the median,
// 2 right; read off the split axis's list.
__global__ void k_level_sides(int64_t n, const int2 *__restrict__ seg, const int32_t *__restrict__ id,
                              const int *__restrict__ seg_axis, uint8_t *__restrict__ side) {
  const int64_t p = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  if (p >= n) return;
  const int2 s = seg[p];
  if (s.x < 0 || s.y - s.x < 2) return;
  const int m = (s.y - s.x) / 2, r = (int)p - s.x;
  side[id[(int64_t)seg_axis[s.x] * n + p]] = r < m ? 0 : (r == m ? 1 : 2);
}

// Packed left / right flags of every list position of an open segment.
__global__ void k_level_flags(int64_t n, const int2 *__restrict__ seg, const int32_t *__restrict__ id,
                              const uint8_t *__restrict__ side, uint64_t *__restrict__ cnt) {
  const int64_t q = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  if (q >= 3 * n) return;
  const int64_t p = q % n;
  const int2 s = seg[p];
  uint64_t v = 0ull;
  if (s.x >= 0 && s.y - s.x >= 2) {
    const uint8_t sd = side[id[q]];
    v = sd == 0 ? 1ull : (sd == 2 ? (1ull << 32) : 0ull);
  }
  cnt[q] = v;
}

// Stable partition of every open segment of every list: the left ranks to
// [b + 1, b + m + 1), the right ones to [b + m + 1, e), in list order; the
// next level's segments.
__global__ void k_level_scatter(int64_t n, const int2 *__restrict__ seg, const uint32_t *__restrict__ key,
                                const int32_t *__restrict__ id, const uint8_t *__restrict__ side,
                                const uint64_t *__restrict__ excl, uint32_t *__restrict__ key2,
                                int32_t *__restrict__ id2) {
  const int64_t q = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  if (q >= 3 * n) return;
  const int64_t a = q / n, p = q - a * n;
  const int2 s = seg[p];
  if (s.x < 0 || s.y - s.x < 2) {  // finished or a leaf-to-be: stays
    key2[q] = key[q];
    id2[q] = id[q];
    return;
  }
  const int32_t i = id[q];
  const uint8_t sd = side[i];
  if (sd == 1) return;  // the median: its node is made
  const uint64_t before = excl[q] - excl[a * n + s.x];
  const int m = (s.y - s.x) / 2;
  const int64_t dst = sd == 0 ? s.x + 1 + (int64_t)(uint32_t)before : s.x + m + 1 + (int64_t)(before >> 32);
  key2[a * n + dst] = key[q];
  id2[a * n + dst] = i;
}

__global__ void k_level_segments(int64_t n, const int2 *__restrict__ seg, int2 *__restrict__ seg2) {
  const int64_t p = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  if (p >= n) return;
  const int2 s = seg[p];
  if (s.x < 0 || (int)p == s.x) {  // finished, or this level's node
    seg2[p] = make_int2(-1, -1);
    return;
  }
  const int split = s.x + (s.y - s.x) / 2;
  seg2[p] = (int)p <= split ? make_int2(s.x + 1, split + 1) : make_int2(split + 1, s.y);
}

__global__ void k_seg_init(int64_t n, int2 *__restrict__ seg) {
  const int64_t p = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  if (p < n) seg[p] = make_int2(0, (int)n);
}

inline size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace

size_t photon_tree_gpu_scratch(int64_t n) {
  const size_t m = (size_t)(3 * n);
  const size_t nb = (m + kBlock - 1) / kBlock;
  return 2 * al256(m * 4) + 2 * al256(m * 4) + al256(m * 8) + al256(nb * 8) + 2 * al256((size_t)n * 8) +
         al256((size_t)n * 4) + al256((size_t)n) + 256;
}

int photon_tree_levels(int64_t n) {
  int h = 0;
  while (n >= 1) {  // the left child holds floor(n / 2) points, the larger share
    ++h;
    n /= 2;
  }
  return h;
}

cudaError_t build_photon_tree_gpu(const float *pos, int64_t n, KdNode *nodes, int32_t *perm, int *tie,
                                  void *scratch, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  if (n > (int64_t)INT32_MAX / 4) return cudaErrorInvalidValue;
  const int64_t m = 3 * n;
  char *w = (char *)scratch;
  auto take = [&](size_t b) {
    char *r = w;
    w += al256(b);
    return r;
  };
  uint32_t *key = (uint32_t *)take(m * 4), *key2 = (uint32_t *)take(m * 4);
  int32_t *id = (int32_t *)take(m * 4), *id2 = (int32_t *)take(m * 4);
  uint64_t *cnt = (uint64_t *)take(m * 8);
  uint64_t *sums = (uint64_t *)take(((m + kBlock - 1) / kBlock) * 8);
  int2 *seg = (int2 *)take(n * 8), *seg2 = (int2 *)take(n * 8);
  int *seg_axis = (int *)take(n * 4);
  uint8_t *side = (uint8_t *)take(n);
  const unsigned gm = (unsigned)((m + kBlock - 1) / kBlock), gn = (unsigned)((n + kBlock - 1) / kBlock);
  cudaError_t e = cudaMemsetAsync(tie, 0, sizeof(int), st);
  if (e != cudaSuccess) return e;
  k_lists_init<<<gm, kBlock, 0, st>>>(pos, n, key, id);
  for (int bit = 0; bit < 32; ++bit) {
    k_sort_flags<<<gm, kBlock, 0, st>>>(key, m, bit, cnt);
    if ((e = scan64(cnt, m, sums, st)) != cudaSuccess) return e;
    k_sort_scatter<<<gm, kBlock, 0, st>>>(key, id, n, bit, cnt, key2, id2);
    uint32_t *tk = key;
    key = key2;
    key2 = tk;
    int32_t *ti = id;
    id = id2;
    id2 = ti;
  }
  k_seg_init<<<gn, kBlock, 0, st>>>(n, seg);
  const int levels = photon_tree_levels(n);
  for (int l = 0; l < levels; ++l) {
    k_level_nodes<<<gn, kBlock, 0, st>>>(pos, n, seg, id, nodes, perm, seg_axis, tie);
    k_level_sides<<<gn, kBlock, 0, st>>>(n, seg, id, seg_axis, side);
    k_level_flags<<<gm, kBlock, 0, st>>>(n, seg, id, side, cnt);
    if ((e = scan64(cnt, m, sums, st)) != cudaSuccess) return e;
    k_level_scatter<<<gm, kBlock, 0, st>>>(n, seg, key, id, side, cnt, key2, id2);
    k_level_segments<<<gn, kBlock, 0, st>>>(n, seg, seg2);
    uint32_t *tk = key;
    key = key2;
    key2 = tk;
    int32_t *ti = id;
    id = id2;
    id2 = ti;
    int2 *ts = seg;
    seg = seg2;
    seg2 = ts;
  }
  return cudaGetLastError();
}

namespace {
__global__ void k_gather_tree_order(const int32_t *__restrict__ perm, int64_t n, const uint16_t *__restrict__ nrm_in,
                                    const uint16_t *__restrict__ dir_in, const float *__restrict__ w_in,
                                    uint16_t *__restrict__ nrm_out, uint16_t *__restrict__ dir_out,
                                    float *__restrict__ w_out) {
  const int64_t t = (int64_t)blockIdx.x * kBlock + threadIdx.x;
  if (t >= n) return;
  const int32_t i = perm[t];
  if (nrm_out) nrm_out[t] = nrm_in[i];
  if (dir_out) dir_out[t] = dir_in[i];
  if (w_out) {
    w_out[3 * t] = w_in[3 * (int64_t)i];
    w_out[3 * t + 1] = w_in[3 * (int64_t)i + 1];
    w_out[3 * t + 2] = w_in[3 * (int64_t)i + 2];
  }
}
}  // namespace

cudaError_t gather_tree_order(const int32_t *perm, int64_t n, const uint16_t *nrm_in, const uint16_t *dir_in,
                              const float *w_in, uint16_t *nrm_out, uint16_t *dir_out, float *w_out,
                              cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  k_gather_tree_order<<<(unsigned)((n + kBlock - 1) / kBlock), kBlock, 0, st>>>(perm, n, nrm_in, dir_in, w_in,
                                                                               nrm_out, dir_out, w_out);
  return cudaGetLastError();
}

// Below this many points the host build is as quick as the launches.
constexpr int64_t kGpuTreeMin = 16384;

cudaError_t build_photon_tree_device(const float *pos, int64_t n, cudaStream_t st, KdNode **d_nodes,
                                     std::vector<int32_t> &perm, int32_t **d_perm, bool *on_gpu) {
  *d_nodes = nullptr;
  *d_perm = nullptr;
  *on_gpu = false;
  const size_t nb = (size_t)(n > 0 ? n : 1) * sizeof(KdNode);
  cudaError_t e = cudaMalloc((void **)d_nodes, nb);
  if (e != cudaSuccess) return e;
  if (n >= kGpuTreeMin) {
    float *d_pos = nullptr;
    void *scratch = nullptr;
    int *d_tie = nullptr;
    std::vector<int> tie(1 + kTieCap, 0);
    tie[0] = kTieCap + 1;
    if ((e = cudaMalloc((void **)&d_pos, (size_t)n * 12)) == cudaSuccess &&
        (e = cudaMalloc((void **)d_perm, (size_t)n * 4)) == cudaSuccess &&
        (e = cudaMalloc(&scratch, photon_tree_gpu_scratch(n))) == cudaSuccess &&
        (e = cudaMalloc((void **)&d_tie, tie.size() * sizeof(int))) == cudaSuccess &&
        (e = cudaMemcpyAsync(d_pos, pos, (size_t)n * 12, cudaMemcpyHostToDevice, st)) == cudaSuccess &&
        (e = build_photon_tree_gpu(d_pos, n, *d_nodes, *d_perm, d_tie, scratch, st)) == cudaSuccess &&
        (e = cudaMemcpyAsync(tie.data(), d_tie, tie.size() * sizeof(int), cudaMemcpyDeviceToHost, st)) ==
            cudaSuccess)
      e = cudaStreamSynchronize(st);
    if (e == cudaSuccess && tie[0] <= kTieCap) {
      perm.resize((size_t)n);
      e = cudaMemcpyAsync(perm.data(), *d_perm, (size_t)n * 4, cudaMemcpyDeviceToHost, st);
      if (tie[0] > 0) {
        // the few subtrees below tied medians, and the paths to them, on the host
        std::vector<KdNode> nodes((size_t)n);
        if (e == cudaSuccess)
          e = cudaMemcpyAsync(nodes.data(), *d_nodes, (size_t)n * sizeof(KdNode), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e == cudaSuccess) {
          repair_photon_tree(pos, n, std::vector<int32_t>(tie.begin() + 1, tie.begin() + 1 + tie[0]), nodes, perm);
          if ((e = cudaMemcpyAsync(*d_nodes, nodes.data(), (size_t)n * sizeof(KdNode), cudaMemcpyHostToDevice,
                                   st)) == cudaSuccess)
            e = cudaMemcpyAsync(*d_perm, perm.data(), (size_t)n * 4, cudaMemcpyHostToDevice, st);
        }
      }
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
      *on_gpu = e == cudaSuccess;
    }
    cudaFree(d_pos);
    cudaFree(scratch);
    cudaFree(d_tie);
    if (e != cudaSuccess || *on_gpu) return e;
    cudaFree(*d_perm);
    *d_perm = nullptr;
  }
  // the host build: small trees, and trees with more than kTieCap tied medians
  std::vector<KdNode> nodes;
  build_photon_tree(pos, n, 0, nodes, perm);
  if (n > 0) e = cudaMemcpyAsync(*d_nodes, nodes.data(), (size_t)n * sizeof(KdNode), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  return e;
}

}  // namespace skw
