// Ray binning before traversal: a one-pass counting sort of the rays by a
// 16-bit coherence key, so that the 32 rays of a warp share their direction
// octant (hence the child visit order at every node), an origin cell and a
// direction sub-cone.  Results are written back in the caller's ray order,
// so binning changes only which rays run side by side, never an answer.
//
// key = octant (3 bits) | Morton code of the origin's cell in an 8x8x8 grid
//       over the scene box (9 bits) | direction bin within the octant from
//       the octahedral coordinates |dx|/s, |dy|/s, s = |dx|+|dy|+|dz|
//       (2 + 2 bits)
//
// Passes (all linear, HBM-bound): histogram (atomics on 65,536 bins),
// exclusive scan of the bins (one block), scatter (each ray copied to its
// slot, plus its original index).  Order inside a bin is whatever the atomics
// give; it affects speed only.
#include <cuda_runtime.h>
#include <cstdint>

#include "kernels.h"

namespace skw {
namespace {

constexpr int kBins = 1 << 16;

__device__ __forceinline__ uint32_t spread3(uint32_t v) {  // 3 bits -> every third bit
  return (v & 1u) | ((v & 2u) << 2) | ((v & 4u) << 4);
}

__device__ __forceinline__ uint32_t ray_key(const float4 a, const float4 b, const float3 lo, const float3 scale) {
  const float dx = a.w, dy = b.x, dz = b.y;
  const uint32_t oct = (dx < 0.0f ? 1u : 0u) | (dy < 0.0f ? 2u : 0u) | (dz < 0.0f ? 4u : 0u);
  const int cx = min(7, max(0, (int)((a.x - lo.x) * scale.x)));
  const int cy = min(7, max(0, (int)((a.y - lo.y) * scale.y)));
  const int cz = min(7, max(0, (int)((a.z - lo.z) * scale.z)));
  const uint32_t cell = spread3((uint32_t)cx) | (spread3((uint32_t)cy) << 1) | (spread3((uint32_t)cz) << 2);
  const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
  const float inv = 1.0f / fmaxf(ax + ay + az, 1e-30f);
  const uint32_t u = (uint32_t)min(3, (int)(ax * inv * 4.0f));
  const uint32_t v = (uint32_t)min(3, (int)(ay * inv * 4.0f));
  return (oct << 13) | (cell << 4) | (u << 2) | v;
}

__global__ void k_ray_hist(const float4 *__restrict__ rays, int64_t n, float3 lo, float3 scale,
                           uint16_t *__restrict__ keys, uint32_t *__restrict__ hist) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float4 a = __ldcs(rays + 2 * i), b = __ldcs(rays + 2 * i + 1);
    const uint32_t k = ray_key(a, b, lo, scale);
    keys[i] = (uint16_t)k;
    atomicAdd(hist + k, 1u);
  }
}

// Exclusive scan of kBins counters in place, one block of 1024 threads.
__global__ void __launch_bounds__(1024) k_hist_scan(uint32_t *__restrict__ hist) {
  constexpr int kPer = kBins / 1024;
  __shared__ uint32_t warp_sums[32];
  uint32_t local[kPer];
  const int t = threadIdx.x;
  uint32_t sum = 0;
#pragma unroll
  for (int j = 0; j < kPer; ++j) {
    local[j] = hist[t * kPer + j];
    sum += local[j];
  }
  // inclusive scan of per-thread sums across the block
  uint32_t x = sum;
  const int lane = t & 31, warp = t >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = warp_sums[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    warp_sums[lane] = w;
  }
  __syncthreads();
  uint32_t run = x - sum + (warp > 0 ? warp_sums[warp - 1] : 0u);
#pragma unroll
  for (int j = 0; j < kPer; ++j) {
    hist[t * kPer + j] = run;
    run += local[j];
  }
}

__global__ void k_ray_scatter(const float4 *__restrict__ rays, int64_t n, const uint16_t *__restrict__ keys,
                              uint32_t *__restrict__ offsets, float4 *__restrict__ sorted,
                              int32_t *__restrict__ index) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t pos = atomicAdd(offsets + keys[i], 1u);
    const float4 a = __ldcs(rays + 2 * i), b = __ldcs(rays + 2 * i + 1);
    sorted[2 * (int64_t)pos] = a;
    sorted[2 * (int64_t)pos + 1] = b;
    index[pos] = (int32_t)i;
  }
}

}  // namespace

size_t ray_sort_workspace_bytes(int64_t n) {
  // hist | keys (2 B per ray) | index (4 B per ray) | sorted rays (32 B per ray), each 256-B aligned
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  return al(kBins * sizeof(uint32_t)) + al((size_t)n * 2) + al((size_t)n * 4) + al((size_t)n * 32);
}

cudaError_t launch_ray_sort(const void *rays, int64_t n, const float *bounds, void *workspace, const void **sorted_out,
                            const int32_t **index_out, int sms, cudaStream_t stream, int *launches) {
  auto al = [](size_t x) { return (x + 255) & ~(size_t)255; };
  char *w = (char *)workspace;
  uint32_t *hist = (uint32_t *)w;
  w += al(kBins * sizeof(uint32_t));
  uint16_t *keys = (uint16_t *)w;
  w += al((size_t)n * 2);
  int32_t *index = (int32_t *)w;
  w += al((size_t)n * 4);
  float4 *sorted = (float4 *)w;
  const float3 lo = make_float3(bounds[0], bounds[1], bounds[2]);
  auto sc = [](float a, float b) { return b > a ? 8.0f / (b - a) : 0.0f; };
  const float3 scale = make_float3(sc(bounds[0], bounds[3]), sc(bounds[1], bounds[4]), sc(bounds[2], bounds[5]));
  cudaError_t e = cudaMemsetAsync(hist, 0, kBins * sizeof(uint32_t), stream);
  if (e != cudaSuccess) return e;
  const int block = 256;
  int64_t grid = (n + block - 1) / block;
  if (grid > (int64_t)sms * 16) grid = (int64_t)sms * 16;
  k_ray_hist<<<(unsigned)grid, block, 0, stream>>>((const float4 *)rays, n, lo, scale, keys, hist);
  k_hist_scan<<<1, 1024, 0, stream>>>(hist);
  k_ray_scatter<<<(unsigned)grid, block, 0, stream>>>((const float4 *)rays, n, keys, hist, sorted, index);
  *launches += 3;
  *sorted_out = sorted;
  *index_out = index;
  return cudaGetLastError();
}

}  // namespace skw
