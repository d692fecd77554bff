// Launch wrappers exported by the .cu translation units to the host layer.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

namespace skw {

// Smallest compiled traversal stack capacity that covers a tree of the given
// depth (root = 0): 2 * depth + 1 entries suffice for the ternary tree.
int traversal_stack_capacity(int max_depth);

// closest = true: hits is skw_hit[n] (int4); false: out is uint8_t[n].
// status: device word; bit 0 is set if a stack ever overflowed.
// scene_abs: the largest absolute coordinate of any vertex in the tree (it
// bounds the slab-test rounding error).
// out_index (may be null): result of ray j goes to slot out_index[j].
cudaError_t launch_traversal(bool closest, int stack_cap, const void *nodes, const void *tris, const void *rays,
                             int64_t n, float scene_abs, const int32_t *out_index, void *out, unsigned *status,
                             cudaStream_t stream);

// Ray binning (raysort.cu): bytes of workspace for n rays, and the launch
// that fills it.  bounds: scene box (min xyz, max xyz).  On return
// *sorted_out / *index_out point into the workspace.
size_t ray_sort_workspace_bytes(int64_t n);
cudaError_t launch_ray_sort(const void *rays, int64_t n, const float *bounds, void *workspace, const void **sorted_out,
                            const int32_t **index_out, int sms, cudaStream_t stream, int *launches);

// Rays per query at or above which the binning pre-pass runs.
#ifndef SKW_RAY_SORT_MIN
#define SKW_RAY_SORT_MIN 65536
#endif

}  // namespace skw
