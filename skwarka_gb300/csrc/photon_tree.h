// Host construction of the photon kd-tree (one point per node, median
// split on the longest axis) and the 16-bit direction codec table.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <vector>

namespace skw {

// One tree node = the node's own photon position and the reference's packed
// node word (KDTree<T>::Node, Raytracer/Core/KDTree.h:188-246): bits 0-1 split
// axis or 3 for a leaf, bit 2 has-left-child, bits 3-31 right child index
// ((1 << 29) - 1 when absent).  The node's split coordinate is its own
// position on the split axis (KDTree.h:455), so it is not stored twice.
// The left child, when present, is the next node.  16 bytes, one vector load.
struct alignas(16) KdNode {
  float x, y, z;
  uint32_t word;
};
static_assert(sizeof(KdNode) == 16, "KdNode must be 16 bytes");

// Builds the tree over n points (float xyz): nodes in tree order and perm[i]
// = input index of the point at tree position i.  The order equals the
// reference's KDTree::_Build (KDTree.h:428-473) for the same standard
// library, since it makes the same std::nth_element calls.  Subtrees are
// built on several threads (`threads` <= 0: all hardware threads).
void build_photon_tree(const float *pos, int64_t n, int threads, std::vector<KdNode> &nodes,
                       std::vector<int32_t> &perm);

// The same tree built on the GPU (photon_tree_gpu.cu) from device positions
// (n x 3 floats): nodes and perm in device memory, and the tie record
// (device, 1 + kTieCap ints): [0] = the number of nodes whose median ties
// on its split axis, then the tree positions of the first kTieCap of them.
// Below a tie node the reference's tree depends on std::nth_element's
// choice among the equal points (repair_photon_tree rebuilds those parts);
// elsewhere the tree equals build_photon_tree's node for node.  scratch:
// photon_tree_gpu_scratch(n) bytes.
constexpr int kTieCap = 256;
size_t photon_tree_gpu_scratch(int64_t n);
int photon_tree_levels(int64_t n);
cudaError_t build_photon_tree_gpu(const float *pos, int64_t n, KdNode *nodes, int32_t *perm, int *tie,
                                  void *scratch, cudaStream_t st);
// Makes a GPU-built tree (nodes, perm: host copies, overwritten in place)
// equal to build_photon_tree's, given the tree positions of all its tie
// nodes: the nodes on the paths from the root to the tie nodes, and the tie
// nodes' whole subtrees, are made on the host from the input order, as
// _Build makes them; every other subtree holds the same points as the
// reference's (no tie above it), so it is already the reference's.
void repair_photon_tree(const float *pos, int64_t n, std::vector<int32_t> ties, std::vector<KdNode> &nodes,
                        std::vector<int32_t> &perm);
// Gathers per-photon attributes into tree order: out[t] = in[perm[t]]
// (normal ids, direction ids and 3-float weights; any may be null).
cudaError_t gather_tree_order(const int32_t *perm, int64_t n, const uint16_t *nrm_in, const uint16_t *dir_in,
                              const float *w_in, uint16_t *nrm_out, uint16_t *dir_out, float *w_out,
                              cudaStream_t st);
// Builds the reference's tree on the GPU (repaired on the host where medians
// tie, up to kTieCap tie nodes), else on the host: the device nodes
// (allocated here, freed by the caller with cudaFree), the permutation on
// the host, and *on_gpu.  pos: host positions.
cudaError_t build_photon_tree_device(const float *pos, int64_t n, cudaStream_t st, KdNode **d_nodes,
                                     std::vector<int32_t> &perm, int32_t **d_perm, bool *on_gpu);

// CompressedDirection table (Math/CompressedDirection.cpp:21-41): unit vector
// of every 16-bit direction id, as 3 doubles per id.
const std::vector<double> &direction_table();

// The device copy of the table: the 3 << 16 doubles of direction_table()
// followed by the same values rounded to float (3 floats per id, packed
// into the vector's last (3 << 16) / 2 doubles).  Kernels that pre-test in
// float read the float part and never convert a double.
const std::vector<double> &direction_table_device();

// CompressedDirection(Vector3D) encoder (Math/CompressedDirection.h:107-133).
uint16_t compress_direction(double x, double y, double z);

}  // namespace skw
