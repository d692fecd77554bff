// Definitions shared by the host translation units of the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <string>

struct skw_ctx {
  int device = 0;
  std::string err;
  std::atomic<int64_t> launches{0};
};

namespace skw {

// Records `msg` as the context's last error and returns `code`.
int fail(skw_ctx *ctx, int code, const std::string &msg);
// Maps a CUDA error to SKW_ERR_OOM / SKW_ERR_CUDA with a message.
int cuda_fail(skw_ctx *ctx, cudaError_t e, const char *what);

}  // namespace skw
