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



}  // namespace skw
