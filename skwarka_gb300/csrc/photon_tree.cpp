// Photon kd-tree build and direction codec; see photon_tree.h.
#include "photon_tree.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <mutex>
#include <thread>
#include <utility>

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

  // One inner node of KDTree::_Build (KDTree.h:436-470) over pts[b, e),
  // e - b >= 2: the median of the longest axis (`known_axis` when the
  // caller knows it, else from the points' box) moved to b, its node word
  // (split axis, left child, right child) set; returns the split position.
  size_t node(size_t b, size_t e, int known_axis = -1) {
    int axis = known_axis;
    if (axis < 0 || axis > 2) {
      double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
      for (size_t i = b; i < e; ++i)
        for (int k = 0; k < 3; ++k) {
          lo[k] = std::min(lo[k], (double)pts[i].p[k]);
          hi[k] = std::max(hi[k], (double)pts[i].p[k]);
        }
      axis = 0;
      if (hi[1] - lo[1] > hi[axis] - lo[axis]) axis = 1;
      if (hi[2] - lo[2] > hi[axis] - lo[axis]) axis = 2;
    }
    const size_t split = (b + e) / 2;
    std::nth_element(pts.begin() + (long)b, pts.begin() + (long)split, pts.begin() + (long)e,
                     [axis](const Pt &u, const Pt &v) { return u.p[axis] < v.p[axis]; });
    std::swap(pts[b], pts[split]);
    word[b] = (word[b] & ~3u) + (uint32_t)axis;  // SetSplitAxis
    if (b < split)
      word[b] = (word[b] & ~4u) + 4u;  // SetHasLeftChild(true)
    else
      word[b] = word[b] & ~4u;
    if (split + 1 < e)
      word[b] = ((uint32_t)(split + 1) << 3) + (word[b] & 7u);  // SetRightChild
    else
      word[b] = (((1u << 29) - 1u) << 3) + (word[b] & 7u);
    return split;
  }

  // KDTree::_Build (KDTree.h:428-473).
  void build(size_t b, size_t e) {
    if (b + 1 == e) {
      word[b] = (word[b] & ~3u) + 3u;  // SetLeaf
      return;
    }
    const size_t split = node(b, e);
    std::thread left_worker;
    bool spawned = false;
    if (b < split) {
      if (split - b > 50000 && threads_left.fetch_sub(1) > 0) {
        spawned = true;
        left_worker = std::thread([this, b, split]() { build(b + 1, split + 1); });
      } else {
        build(b + 1, split + 1);
      }
    }
    if (split + 1 < e) build(split + 1, e);
    if (spawned) left_worker.join();
  }

  // The repair of a tree built on the GPU (repair_photon_tree): pts[b, e)
  // holds the range as _Build sees it.  A range without a tie node is the
  // GPU's; a tie node's subtree is built whole; any other node is made here
  // (its split axis is the GPU's: the node's point set is the reference's)
  // and its children repaired.  `done` collects the ranges made here.
  bool has_tie(size_t b, size_t e, const std::vector<int32_t> &ties) const {
    const auto it = std::lower_bound(ties.begin(), ties.end(), (int32_t)b);
    return it != ties.end() && (size_t)*it < e;
  }
  void repair(size_t b, size_t e, const std::vector<int32_t> &ties, const std::vector<KdNode> &gpu,
              std::vector<std::pair<size_t, size_t>> &done) {
    if (!has_tie(b, e, ties)) return;
    if (std::binary_search(ties.begin(), ties.end(), (int32_t)b)) {
      build(b, e);
      done.emplace_back(b, e);
      return;
    }
    const size_t split = node(b, e, (int)(gpu[b].word & 3u));
    done.emplace_back(b, b + 1);
    std::vector<std::pair<size_t, size_t>> left_done;
    std::thread left_worker;
    bool spawned = false;
    if (has_tie(b + 1, split + 1, ties)) {
      if (split - b > 50000 && has_tie(split + 1, e, ties) && threads_left.fetch_sub(1) > 0) {
        spawned = true;
        left_worker = std::thread([&, b, split]() { repair(b + 1, split + 1, ties, gpu, left_done); });
      } else {
        repair(b + 1, split + 1, ties, gpu, done);
      }
    }
    if (split + 1 < e) repair(split + 1, e, ties, gpu, done);
    if (spawned) {
      left_worker.join();
      done.insert(done.end(), left_done.begin(), left_done.end());
    }
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

void repair_photon_tree(const float *pos, int64_t n, std::vector<int32_t> ties, std::vector<KdNode> &nodes,
                        std::vector<int32_t> &perm) {
  if (n <= 0 || ties.empty()) return;
  std::sort(ties.begin(), ties.end());
  Build B;
  B.pts.resize((size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    for (int k = 0; k < 3; ++k) B.pts[(size_t)i].p[k] = pos[3 * i + k];
    B.pts[(size_t)i].orig = (int32_t)i;
  }
  B.word.assign((size_t)n, 0u);
  unsigned hw = std::thread::hardware_concurrency();
  B.threads_left = (int)(hw ? hw : 1) - 1;
  std::vector<std::pair<size_t, size_t>> done;
  B.repair(0, (size_t)n, ties, nodes, done);
  for (const auto &r : done)
    for (size_t i = r.first; i < r.second; ++i) {
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
