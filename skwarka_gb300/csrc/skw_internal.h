// Definitions shared by the host translation units of the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/skw.h"
#include "accel_build.h"
#include "render_scene.h"

struct skw_ctx {
  int device = 0;
  int sms = 0;
  std::string err;
  std::atomic<int64_t> launches{0};
  // Stream-ordered pool for per-call workspaces; it keeps freed memory
  // (release threshold = max) so repeated calls do not remap.
  cudaMemPool_t pool = nullptr;
  // The host-buffer queries' two streams and events, made on first use and
  // kept (creating and destroying them per call cost ~0.1 ms).
  cudaStream_t host_st[2] = {nullptr, nullptr};
  cudaEvent_t host_ev[2] = {nullptr, nullptr};
  // The renders' side streams (a level's shadow and BSDF traversals), made
  // on first use under aux_mu and kept.
  std::mutex aux_mu;
  cudaStream_t aux_st[2] = {nullptr, nullptr};
};

// A device-resident accelerator (skw_accel_create / _from_flat).
struct skw_accel {
  skw_ctx *ctx = nullptr;
  skw::DevNode *d_nodes = nullptr;
  skw::DevTri *d_tris = nullptr;
  skw::DevInst *d_inst = nullptr;     // instances (null: none)
  skw::LeafExt *d_leaf_ext = nullptr; // leaves holding instances
  unsigned *d_status = nullptr;
  unsigned long long *d_traced = nullptr;  // rays traced by all launches on this accelerator
  int stack_cap = 0;
  float scene_abs = 0.0f;  // largest absolute vertex coordinate
  skw_accel_info info{};
  std::vector<skw::DevNode> h_nodes;
  std::vector<skw::DevTri> h_tris;
  std::vector<skw::DevInst> h_inst;
  std::vector<skw::LeafExt> h_leaf_ext;
  std::vector<uint32_t> h_subtree_roots;
};

// A render scene (skw_scene_create): its accelerator plus the shading data.
struct skw_scene {
  skw_ctx *ctx = nullptr;
  skw_accel *accel = nullptr;
  int64_t n_triangles = 0;  // mesh order, over all primitives
  double total_area = 0.0;  // sum of the primitives' mesh areas (TriangleMesh::GetArea, mesh space)
  std::vector<void *> buffers;  // device allocations owned by the scene
  skw::SceneDev dev{};
};

namespace skw {

// Records `msg` as the context's last error and returns `code`.
int fail(skw_ctx *ctx, int code, const std::string &msg);
// Maps a CUDA error to SKW_ERR_OOM / SKW_ERR_CUDA with a message.
int cuda_fail(skw_ctx *ctx, cudaError_t e, const char *what);
// Creates the context's workspace pool on first use.
cudaError_t ctx_pool(skw_ctx *ctx, cudaMemPool_t *pool);

}  // namespace skw
