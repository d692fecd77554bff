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
// (n x 3 floats): nodes and perm in device memory, *tie (device int) set
// when some node's median ties on its split axis -- there the reference's
// tree depends on std::nth_element's choice among equal points, and the
// host build is the one to use.  Otherwise the tree equals
// build_photon_tree's node for node.  scratch: photon_tree_gpu_scratch(n)
// bytes.
size_t photon_tree_gpu_scratch(int64_t n);
int photon_tree_levels(int64_t n);
cudaError_t build_photon_tree_gpu(const float *pos, int64_t n, KdNode *nodes, int32_t *perm, int *tie,
                                  void *scratch, cudaStream_t st);
// Gathers per-photon attributes into tree order: out[t] = in[perm[t]]
// (normal ids, direction ids and 3-float weights; any may be null).
cudaError_t gather_tree_order(const int32_t *perm, int64_t n, const uint16_t *nrm_in, const uint16_t *dir_in,
                              const float *w_in, uint16_t *nrm_out, uint16_t *dir_out, float *w_out,
                              cudaStream_t st);
// Builds on the GPU where that gives the reference's tree, else on the host:
// the device nodes (allocated here, freed by the caller with cudaFree), the
// permutation on the host, and *on_gpu.  pos: host positions.
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
