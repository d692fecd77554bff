// Photon kd-tree build and direction codec; see photon_tree.h.
#include "photon_tree.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <mutex>
#include <thread>

namespace skw {
namespace {

struct Pt {
  float p[3];
  int32_t orig;
};

struct Build {
  std::vector<Pt> pts;
  std::vector<uint32_t> word;
  std::atomic<int> threads_left{0};

  // KDTree::_Build (KDTree.h:428-473).
  void build(size_t b, size_t e) {
    if (b + 1 == e) {
      word[b] = (word[b] & ~3u) + 3u;  // SetLeaf
      return;
    }
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (size_t i = b; i < e; ++i)
      for (int k = 0; k < 3; ++k) {
        lo[k] = std::min(lo[k], (double)pts[i].p[k]);
        hi[k] = std::max(hi[k], (double)pts[i].p[k]);
      }
    int axis = 0;
    if (hi[1] - lo[1] > hi[axis] - lo[axis]) axis = 1;
    if (hi[2] - lo[2] > hi[axis] - lo[axis]) axis = 2;
    const size_t split = (b + e) / 2;
    std::nth_element(pts.begin() + (long)b, pts.begin() + (long)split, pts.begin() + (long)e,
                     [axis](const Pt &u, const Pt &v) { return u.p[axis] < v.p[axis]; });
    std::swap(pts[b], pts[split]);
    word[b] = (word[b] & ~3u) + (uint32_t)axis;  // SetSplitAxis
    std::thread left_worker;
    bool spawned = false;
    if (b < split) {
      word[b] = (word[b] & ~4u) + 4u;  // SetHasLeftChild(true)
      if (split - b > 50000 && threads_left.fetch_sub(1) > 0) {
        spawned = true;
        left_worker = std::thread([this, b, split]() { build(b + 1, split + 1); });
      } else {
        build(b + 1, split + 1);
      }
    } else {
      word[b] = word[b] & ~4u;
    }
    if (split + 1 < e) {
      word[b] = ((uint32_t)(split + 1) << 3) + (word[b] & 7u);  // SetRightChild
      build(split + 1, e);
    } else {
      word[b] = (((1u << 29) - 1u) << 3) + (word[b] & 7u);
    }
    if (spawned) left_worker.join();
  }
};

}  // namespace

void build_photon_tree(const float *pos, int64_t n, int threads, std::vector<KdNode> &nodes,
                       std::vector<int32_t> &perm) {
  Build B;
  B.pts.resize((size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    for (int k = 0; k < 3; ++k) B.pts[(size_t)i].p[k] = pos[3 * i + k];
    B.pts[(size_t)i].orig = (int32_t)i;
  }
  B.word.assign((size_t)n, 0u);
  unsigned hw = std::thread::hardware_concurrency();
  B.threads_left = (threads > 0 ? threads : (int)(hw ? hw : 1)) - 1;
  if (n > 0) B.build(0, (size_t)n);
  nodes.resize((size_t)n);
  perm.resize((size_t)n);
  for (size_t i = 0; i < (size_t)n; ++i) {
    nodes[i] = KdNode{B.pts[i].p[0], B.pts[i].p[1], B.pts[i].p[2], B.word[i]};
    perm[i] = B.pts[i].orig;
  }
}

const std::vector<double> &direction_table() {
  static std::vector<double> table;
  static std::once_flag once;
  std::call_once(once, []() {
    table.resize(3u << 16);
    for (int i = 0; i < (1 << 16); ++i) {
      unsigned x = (unsigned)((i >> 6) & 0x7F), y = (unsigned)(i & 0x3F);
      if (x + y >= 127) {
        x = 127 - x;
        y = 127 - y;
      }
      double v[3] = {x + 0.5, y + 0.5, 126.0 - x - y};
      const double ls = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
      if (ls > 0.0) {
        const double inv = 1.0 / std::sqrt(ls);
        for (double &c : v) c *= inv;
      }
      if (i & (1 << 13)) v[0] = -v[0];
      if (i & (1 << 14)) v[1] = -v[1];
      if (i & (1 << 15)) v[2] = -v[2];
      for (int k = 0; k < 3; ++k) table[3 * (size_t)i + k] = v[k];
    }
  });
  return table;
}

const std::vector<double> &direction_table_device() {
  static std::vector<double> table;
  static std::once_flag once;
  std::call_once(once, []() {
    const std::vector<double> &t = direction_table();
    table.assign(t.begin(), t.end());
    table.resize(t.size() + t.size() / 2);
    float *f = reinterpret_cast<float *>(table.data() + t.size());
    for (size_t i = 0; i < t.size(); ++i) f[i] = (float)t[i];
  });
  return table;
}

uint16_t compress_direction(double x, double y, double z) {
  unsigned data = 0;
  if (x < 0) {
    data |= 1u << 13;
    x = -x;
  }
  if (y < 0) {
    data |= 1u << 14;
    y = -y;
  }
  if (z < 0) {
    data |= 1u << 15;
    z = -z;
  }
  const double scale = 126.999 / (x + y + z);
  unsigned char qx = (unsigned char)(x * scale), qy = (unsigned char)(y * scale);
  if (qy >= 64) {
    qx = (unsigned char)(127 - qx);
    qy = (unsigned char)(127 - qy);
  }
  data |= ((unsigned)qx << 6) | qy;
  return (uint16_t)data;
}

}  // namespace skw
