// Host-side construction of the ternary bbox kd-tree and its flattening into
// the device layout used by the traversal kernels.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <vector>

namespace skw {

// One node of the device tree: 32 bytes, 32-byte aligned, read as two
// 16-byte vector loads.
//   lo/hi : float AABB of the node's triangles (the reference's Node::m_bbox)
//   a     : internal -> index of the first child (children are contiguous, in
//           left, middle, right order, absent ones skipped)
//           leaf     -> index of the first triangle slot
//   b     : bits 0-1 type (0 = leaf, 1..3 = internal with split axis + 1,
//           the reference's Node::m_flags & 3)
//           internal -> bits 2-4 child-present mask (1 left, 2 middle, 4 right)
//           leaf     -> bits 8-31 triangle count
struct alignas(32) DevNode {
  float lo[3];
  float hi[3];
  uint32_t a;
  uint32_t b;
};
static_assert(sizeof(DevNode) == 32, "DevNode must be 32 bytes");

// One triangle slot: 48 bytes = 3 x float4 (v0, prim), (v1, tri), (v2, slot)
// with the integer ids stored in the .w lanes as raw bits.
struct alignas(16) DevTri {
  float v0[3];
  int32_t prim;
  float v1[3];
  int32_t tri;
  float v2[3];
  int32_t slot;
};
static_assert(sizeof(DevTri) == 48, "DevTri must be 48 bytes");

struct MeshIn {
  const float *vertices;
  int64_t n_vertices;
  const int32_t *triangles;
  int64_t n_triangles;
};

struct PrimIn {
  int32_t mesh;
  const double *mesh_to_world;  // row-major 4x4 or null
};

// An instance of a mesh shared by several primitives (the reference's
// m_instance_nodes / m_instance_to_world_transformations /
// m_instance_primitive_indices, TriangleAccelerator.cpp:54-102): the
// world-to-mesh matrix of its primitive (row-major; the inverse that
// Matrix4x4::Inverted computes, which the traversal applies to rays), the
// node index of its mesh's subtree and its primitive.  144 bytes.
struct alignas(16) DevInst {
  double world_to_mesh[16];
  uint32_t root;
  int32_t prim;
  uint32_t pad[2];
};
static_assert(sizeof(DevInst) == 144, "DevInst must be 144 bytes");

// A leaf holding instances: DevNode.b has kLeafExt set and DevNode.a indexes
// the tree's leaf_ext table (its triangle and instance ranges).
constexpr uint32_t kLeafExt = 1u << 7;
struct LeafExt {
  uint32_t tri_first, tri_count, inst_first, inst_count;
};

struct FlatTree {
  std::vector<DevNode> nodes;    // the tree (root 0), then every shared mesh's subtree
  std::vector<DevTri> tris;      // shared meshes' triangles (mesh space, prim -1) first
  std::vector<DevInst> inst;     // in the final (partitioned) order
  std::vector<LeafExt> leaf_ext;
  std::vector<uint32_t> subtree_roots;  // one per shared mesh, in mesh order
  int32_t max_depth = 0;         // over the tree and the subtrees
  int64_t n_leaves = 0;
  float bounds[6] = {0, 0, 0, 0, 0, 0};
};

// Matrix4x4<double>::Inverted (Math/Matrix4x4.h:240-316): Gauss-Jordan
// elimination with full pivoting, row-major 4x4; false if singular.
bool invert4(const double *m, double *out);

// The tree built on the GPU over triangle boxes (build_accel_tree_gpu):
// node records by node id (level by level from the root), and the final
// slot order.
struct AccelTreeGpu {
  std::vector<float> box;       // 6 floats per node: lo xyz, hi xyz
  std::vector<uint32_t> tb, te; // triangle-slot range per node
  std::vector<uint8_t> flags;   // 0 leaf, 1..3 split axis + 1
  std::vector<int32_t> child;   // 3 per node (left, middle, right), -1 if absent
  std::vector<uint32_t> perm;   // triangle (input order) of each final slot
  int64_t n_nodes = 0, n_leaves = 0;
  int32_t max_depth = 0;
  bool inconsistent = false;    // the partition's step map was not a permutation
};

// Builds the tree of the host build over n triangle boxes (6 floats each:
// lo xyz, hi xyz, host memory, in the order the host build starts from) on
// the current device, on stream st (waits for it).
cudaError_t build_accel_tree_gpu(const float *tbox, int64_t n, cudaStream_t st, AccelTreeGpu &out);

// build_accel for accelerators without instancing, the tree built on the
// GPU (the same tree; meshes shared by several primitives, or fewer than
// min_gpu triangles, build on the host).  *on_gpu tells which.
std::string build_accel_device(const MeshIn *meshes, int32_t n_meshes, const PrimIn *prims, int32_t n_prims,
                               int threads, cudaStream_t st, int64_t min_gpu, FlatTree &out, bool *on_gpu);

// Builds the tree (same split search, partition order and leaf rule as the
// reference TriangleAccelerator, instancing included: a mesh used by several
// primitives gets one subtree in mesh space and each of its primitives an
// instance) and flattens it.  `threads` <= 0 uses all
// hardware threads.  Returns an empty string on success, else an error.
std::string build_accel(const MeshIn *meshes, int32_t n_meshes, const PrimIn *prims, int32_t n_prims,
                        int threads, FlatTree &out);

}  // namespace skw
