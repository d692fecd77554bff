// Host construction of the ternary bbox kd-tree, restating the reference
// TriangleAccelerator build (Raytracer/Core/TriangleAccelerator.cpp):
//   * meshes shared by several primitives (instancing, ctor step 2,
//     :54-102): one subtree over the mesh-space triangles per mesh, and per
//     primitive an instance with the world box of the subtree box's
//     transformed corners, weighted by the subtree's triangle count in the
//     split search and partitioned like triangles;
//   * world-space float triangles per primitive, in primitive order
//     (ctor steps 3-4, :104-139; the transform is Transform::operator()
//     on Point3D_f, Math/Transform.h:219-230);
//   * per node: float AABB of its triangles (_ConstructBBox, :470-481);
//     leaf if <= 4 triangles, three middle splits on the path, or depth >= 200
//     (Node::Node, :630-636);
//   * split search over min(200, 2n) uniform candidate planes per axis with
//     bucketed left/middle/right boxes and counts, cost
//     sum(n_child * area_child / area_node) with a 0.8 bonus for an empty
//     side, first strict minimum per axis, axis ties to the lower axis
//     (_DetermineBestSplit, :505-617);
//   * in-place three-way partition with the same swap sequence
//     (Node::Node, :644-673), so leaves own contiguous triangle ranges.
// The arithmetic keeps the reference's float/double mix operation by
// operation (for example the candidate-plane position is computed in float),
// so that the same input gives the same tree.  Subtrees are built in parallel
// on disjoint triangle ranges; this changes no result.
//
// The tree is then flattened into DevNode/DevTri arrays: pre-order, each
// internal node's present children stored contiguously.
#include "accel_build.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <limits>
#include <memory>
#include <thread>

namespace skw {
namespace {

constexpr size_t kMaxTrianglesInLeaf = 4;  // TriangleAccelerator.h:128
constexpr size_t kMaxSplitTries = 200;     // TriangleAccelerator.h:131
constexpr size_t kMaxTreeDepth = 200;      // TriangleAccelerator.h:134

constexpr float kInfF = std::numeric_limits<float>::infinity();
constexpr double kInfD = std::numeric_limits<double>::infinity();

struct BoxF {
  float lo[3] = {kInfF, kInfF, kInfF};
  float hi[3] = {-kInfF, -kInfF, -kInfF};
  void unite(const BoxF &o) {
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], o.lo[k]);
      hi[k] = std::max(hi[k], o.hi[k]);
    }
  }
  // BBox3D<float>::Area (Math/BBox3D.h:141-147): all in float.
  float area() const {
    float x = std::fabs(hi[0] - lo[0]);
    float y = std::fabs(hi[1] - lo[1]);
    float z = std::fabs(hi[2] - lo[2]);
    return 2.0f * (x * y + x * z + y * z);
  }
};

struct BoxD {
  double lo[3] = {kInfD, kInfD, kInfD};
  double hi[3] = {-kInfD, -kInfD, -kInfD};
  void unite(const BoxF &o) {
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], (double)o.lo[k]);
      hi[k] = std::max(hi[k], (double)o.hi[k]);
    }
  }
  void unite(const BoxD &o) {
    for (int k = 0; k < 3; ++k) {
      lo[k] = std::min(lo[k], o.lo[k]);
      hi[k] = std::max(hi[k], o.hi[k]);
    }
  }
  double area() const {
    double x = std::fabs(hi[0] - lo[0]);
    double y = std::fabs(hi[1] - lo[1]);
    double z = std::fabs(hi[2] - lo[2]);
    return 2.0 * (x * y + x * z + y * z);
  }
};

// double -> size_t with the result x86-64 g++ code gives for the reference's
// (size_t) casts: NaN -> 2^63, +inf and values >= 2^64 -> 0.  NaN arises for a
// node of zero extent along the tested axis (0 * inf).
inline size_t cast_size(double v) {
  if (std::isnan(v)) return (size_t)1 << 63;
  if (v >= 18446744073709551616.0) return 0;
  if (v >= 9223372036854775808.0) return (size_t)(v - 9223372036854775808.0) + ((size_t)1 << 63);
  return (size_t)(int64_t)v;
}

struct BNode {
  BoxF box;
  uint32_t tb = 0, te = 0;  // triangle range
  uint32_t ib = 0, ie = 0;  // instance range
  uint8_t flags = 0;        // 0 leaf, 1..3 axis + 1
  std::unique_ptr<BNode> child[3];
};

struct Builder {
  std::vector<float> tv;      // 9 floats per triangle (world space)
  std::vector<int32_t> prim;  // primitive index per triangle
  std::vector<int32_t> tidx;  // mesh triangle index per triangle
  std::vector<BoxF> tbox;     // per-triangle AABB, in the build's current order
  std::vector<uint32_t> order;  // the triangle (index into tv, prim, tidx) in each slot
  // Instances of shared meshes (TriangleAccelerator.cpp:54-102): world box
  // of the instance, triangles of its mesh's subtree (the split search's
  // weight), its primitive and the subtree it instances.
  std::vector<BoxF> ibox;
  std::vector<size_t> icount;
  std::vector<int32_t> iprim;
  std::vector<int32_t> isub;
  std::atomic<int> threads_left{0};
  int threads = 1;  // the build's thread budget
  std::atomic<int32_t> max_depth{0};
  std::atomic<int64_t> n_leaves{0};

  // The partition's swaps move the box the split search reads and the
  // slot's triangle index; the triangles themselves are gathered in the
  // final order once, when the tree is flattened.
  void swap_tris(size_t a, size_t b) {
    std::swap(order[a], order[b]);
    std::swap(tbox[a], tbox[b]);
  }
  // _SwapInstances (TriangleAccelerator.cpp:495-503)
  void swap_inst(size_t a, size_t b) {
    std::swap(ibox[a], ibox[b]);
    std::swap(icount[a], icount[b]);
    std::swap(iprim[a], iprim[b]);
    std::swap(isub[a], isub[b]);
  }

  // One axis's buckets of _DetermineBestSplit over triangles [ib, ie):
  // left / middle / right boxes and counts per candidate plane.  Box unions
  // (min / max) and counts do not depend on the order the triangles come
  // in, so partial buckets over slices of the range merge exactly.
  struct Buckets {
    BoxD L[kMaxSplitTries], M[kMaxSplitTries], R[kMaxSplitTries];
    size_t Ln[kMaxSplitTries] = {0}, Mn[kMaxSplitTries] = {0}, Rn[kMaxSplitTries] = {0};
    // Empties the first `tries` candidates (the only ones a node uses).
    void reset(size_t tries) {
      for (size_t i = 0; i < tries; ++i) {
        L[i] = M[i] = R[i] = BoxD();
        Ln[i] = Mn[i] = Rn[i] = 0;
      }
    }
    void merge(const Buckets &o, size_t tries) {
      for (size_t i = 0; i < tries; ++i) {
        L[i].unite(o.L[i]);
        M[i].unite(o.M[i]);
        R[i].unite(o.R[i]);
        Ln[i] += o.Ln[i];
        Mn[i] += o.Mn[i];
        Rn[i] += o.Rn[i];
      }
    }
  };
  static void add_bucket(const BoxF &nb, int axis, const BoxF &b, size_t count, size_t tries, double coef,
                         Buckets &k) {
    const float dmax = b.hi[axis] - nb.lo[axis];
    const float dmin = b.lo[axis] - nb.lo[axis];
    const size_t lefts_begin = std::min(tries, cast_size((double)dmax * coef + 1.0));
    const size_t rights_end = std::min(tries, cast_size((double)dmin * coef + 1.0));
    if (rights_end > 0) {
      k.R[rights_end - 1].unite(b);
      k.Rn[rights_end - 1] += count;
    }
    if (lefts_begin < tries) {
      k.L[lefts_begin].unite(b);
      k.Ln[lefts_begin] += count;
    }
    for (size_t j = rights_end; j < lefts_begin; ++j) {
      k.M[j].unite(b);
      k.Mn[j] += count;
    }
  }
  void fill_buckets(const BoxF &nb, int axis, size_t ib, size_t ie, size_t tries, double coef, Buckets &k) const {
    for (size_t i = ib; i < ie; ++i) add_bucket(nb, axis, tbox[i], 1, tries, coef, k);
  }
  // An instance counts as its subtree's triangles (TriangleAccelerator.cpp:553).
  void fill_inst_buckets(const BoxF &nb, int axis, size_t ib, size_t ie, size_t tries, double coef,
                         Buckets &k) const {
    for (size_t i = ib; i < ie; ++i) add_bucket(nb, axis, ibox[i], icount[i], tries, coef, k);
  }

  // _DetermineBestSplit (TriangleAccelerator.cpp:505-617).
  // Nodes of at least kParallelSplit triangles (the top of the tree, where
  // few subtrees run side by side) fill their buckets on several threads,
  // one slice of the triangles and one axis each.
  static constexpr size_t kParallelSplit = (size_t)1 << 17;
  void best_split(const BoxF &nb, size_t tb, size_t te, size_t ib, size_t ie, unsigned mask, int &axis_out,
                  double &pos_out) const {
    const size_t n = te - tb;
    double best_pos[3] = {0, 0, 0}, best_cost[3] = {kInfD, kInfD, kInfD};
    const size_t tries = std::min(kMaxSplitTries, 2 * n + 2 * (ie - ib));
    double coefs[3] = {0, 0, 0};
    for (int axis = 0; axis < 3; ++axis) {
      const float ext = nb.hi[axis] - nb.lo[axis];
      // size_t / float converts the count to float: float division.
      coefs[axis] = (double)((float)tries / ext);
    }
    // The reference's cost of every candidate plane of one axis (prefix
    // unions of the left boxes, suffix unions of the right ones).
    auto score = [&](int axis, Buckets &k) {
      const float ext = nb.hi[axis] - nb.lo[axis];
      BoxD *L = k.L, *M = k.M, *R = k.R;
      size_t *Ln = k.Ln, *Mn = k.Mn, *Rn = k.Rn;
      for (size_t i = 1; i < tries; ++i) {
        L[i].unite(L[i - 1]);
        Ln[i] += Ln[i - 1];
      }
      for (int i = (int)tries - 2; i >= 0; --i) {
        R[i].unite(R[i + 1]);
        Rn[i] += Rn[i + 1];
      }
      const double inv_area = 1.0 / (double)nb.area();
      for (size_t i = 0; i < tries; ++i) {
        const double p1 = std::min(1.0, L[i].area() * inv_area);
        const double p2 = std::min(1.0, M[i].area() * inv_area);
        const double p3 = std::min(1.0, R[i].area() * inv_area);
        double cost = (double)Ln[i] * p1 + (double)Mn[i] * p2 + (double)Rn[i] * p3;
        if (Ln[i] == 0 || Rn[i] == 0) cost *= 0.8;
        if (cost < best_cost[axis]) {
          best_cost[axis] = cost;
          // min + i*(max-min)/tries, evaluated in float.
          best_pos[axis] = (double)(nb.lo[axis] + ((float)i * ext) / (float)tries);
        }
      }
    };
    const size_t slices = n >= kParallelSplit && threads > 1 ? std::min<size_t>(std::max(1, threads / 3), 16) : 1;
    if (slices > 1) {
      std::vector<Buckets> part(3 * slices);
      std::vector<std::thread> pool;
      for (int axis = 0; axis < 3; ++axis) {
        if (mask & (1u << axis)) continue;
        for (size_t c = 0; c < slices; ++c) {
          const size_t ib = tb + n * c / slices, ie = tb + n * (c + 1) / slices;
          pool.emplace_back([this, &nb, &part, axis, ib, ie, tries, c, slices, coef = coefs[axis]]() {
            fill_buckets(nb, axis, ib, ie, tries, coef, part[(size_t)axis * slices + c]);
          });
        }
      }
      for (std::thread &t : pool) t.join();
      for (int axis = 0; axis < 3; ++axis) {
        if (mask & (1u << axis)) continue;
        Buckets &k = part[(size_t)axis * slices];
        for (size_t c = 1; c < slices; ++c) k.merge(part[(size_t)axis * slices + c], tries);
        fill_inst_buckets(nb, axis, ib, ie, tries, coefs[axis], k);
        score(axis, k);
      }
    } else {
      // one bucket set per thread, emptied over the node's own candidates
      static thread_local Buckets k;
      for (int axis = 0; axis < 3; ++axis) {
        if (mask & (1u << axis)) continue;
        k.reset(tries);
        fill_buckets(nb, axis, tb, te, tries, coefs[axis], k);
        fill_inst_buckets(nb, axis, ib, ie, tries, coefs[axis], k);
        score(axis, k);
      }
    }
    if (best_cost[0] <= best_cost[1] && best_cost[0] <= best_cost[2]) {
      axis_out = 0;
    } else if (best_cost[1] <= best_cost[0] && best_cost[1] <= best_cost[2]) {
      axis_out = 1;
    } else {
      axis_out = 2;
    }
    pos_out = best_pos[axis_out];
  }

  // Node::Node (TriangleAccelerator.cpp:621-729): triangles [tb, te) and
  // instances [ib, ie).
  std::unique_ptr<BNode> build(size_t tb, size_t te, size_t ib, size_t ie, unsigned mask, size_t depth) {
    auto node = std::make_unique<BNode>();
    node->tb = (uint32_t)tb;
    node->te = (uint32_t)te;
    node->ib = (uint32_t)ib;
    node->ie = (uint32_t)ie;
    for (size_t i = tb; i < te; ++i) node->box.unite(tbox[i]);
    for (size_t i = ib; i < ie; ++i) node->box.unite(ibox[i]);
    int32_t d = (int32_t)depth;
    int32_t cur = max_depth.load();
    while (d > cur && !max_depth.compare_exchange_weak(cur, d)) {
    }
    if ((te - tb) + (ie - ib) <= kMaxTrianglesInLeaf || mask == 7u || depth >= kMaxTreeDepth) {
      node->flags = 0;
      n_leaves.fetch_add(1);
      return node;
    }
    int axis;
    double split;
    best_split(node->box, tb, te, ib, ie, mask, axis, split);
    node->flags = (uint8_t)(axis + 1);

    size_t mid_begin = tb, right_begin = te, i = tb;
    while (i < right_begin) {
      const BoxF &b = tbox[i];
      if ((double)b.hi[axis] < split) {
        swap_tris(mid_begin, i);
        ++mid_begin;
        ++i;
      } else if ((double)b.lo[axis] > split) {
        --right_begin;
        swap_tris(i, right_begin);
      } else {
        ++i;
      }
    }
    // the instances, partitioned the same way (TriangleAccelerator.cpp:677-700)
    size_t imid = ib, iright = ie;
    i = ib;
    while (i < iright) {
      const BoxF &b = ibox[i];
      if ((double)b.hi[axis] < split) {
        swap_inst(imid, i);
        ++imid;
        ++i;
      } else if ((double)b.lo[axis] > split) {
        --iright;
        swap_inst(i, iright);
      } else {
        ++i;
      }
    }
    struct Range {
      size_t b, e, ib, ie;
      unsigned m;
    } ranges[3] = {{tb, mid_begin, ib, imid, mask},
                   {mid_begin, right_begin, imid, iright, mask | (1u << axis)},
                   {right_begin, te, iright, ie, mask}};
    // Large subtrees run on their own thread while the budget lasts.
    std::thread workers[3];
    bool spawned[3] = {false, false, false};
    for (int c = 0; c < 3; ++c) {
      if (ranges[c].b >= ranges[c].e && ranges[c].ib >= ranges[c].ie) continue;
      bool spawn = false;
      if (ranges[c].e - ranges[c].b > 20000) {
        spawn = threads_left.fetch_sub(1) > 0;
        if (!spawn) threads_left.fetch_add(1);
      }
      if (spawn) {
        spawned[c] = true;
        workers[c] = std::thread([this, node_ptr = node.get(), c, r = ranges[c], depth]() {
          node_ptr->child[c] = build(r.b, r.e, r.ib, r.ie, r.m, depth + 1);
          threads_left.fetch_add(1);  // the thread goes back to the budget
        });
      } else {
        node->child[c] = build(ranges[c].b, ranges[c].e, ranges[c].ib, ranges[c].ie, ranges[c].m, depth + 1);
      }
    }
    for (int c = 0; c < 3; ++c)
      if (spawned[c]) workers[c].join();
    return node;
  }
};

// Transform::operator()(const Point3D<float>&) (Math/Transform.h:219-230).
inline void transform_point(const double *m, const float *p, float *out) {
  const float x = p[0], y = p[1], z = p[2];
  float xp = (float)(m[0] * x + m[1] * y + m[2] * z + m[3]);
  float yp = (float)(m[4] * x + m[5] * y + m[6] * z + m[7]);
  float zp = (float)(m[8] * x + m[9] * y + m[10] * z + m[11]);
  float wp = (float)(m[12] * x + m[13] * y + m[14] * z + m[15]);
  if (wp == 1.0f) {
    out[0] = xp;
    out[1] = yp;
    out[2] = zp;
  } else {
    // Point3D<float>::operator/(double): multiply by the double reciprocal.
    double inv = 1.0 / (double)wp;
    out[0] = (float)(xp * inv);
    out[1] = (float)(yp * inv);
    out[2] = (float)(zp * inv);
  }
}

}  // namespace

bool invert4(const double *m, double *out) {
  int indxc[4], indxr[4];
  int ipiv[4] = {0, 0, 0, 0};
  double minv[4][4];
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) minv[r][c] = m[4 * r + c];
  bool singular = false;
  for (int i = 0; i < 4; ++i) {
    int irow = -1, icol = -1;
    double big = 0.0;
    for (int j = 0; j < 4; ++j) {
      if (ipiv[j] == 1) continue;
      for (int k = 0; k < 4; ++k) {
        if (ipiv[k] == 0) {
          if (std::fabs(minv[j][k]) >= big) {
            big = std::fabs(minv[j][k]);
            irow = j;
            icol = k;
          }
        } else if (ipiv[k] > 1) {
          singular = true;
        }
      }
    }
    if (irow < 0 || icol < 0) return false;  // NaN entries
    ++ipiv[icol];
    if (irow != icol)
      for (int k = 0; k < 4; ++k) std::swap(minv[irow][k], minv[icol][k]);
    indxr[i] = irow;
    indxc[i] = icol;
    if (minv[icol][icol] == 0.0) singular = true;
    const double pivinv = 1.0 / minv[icol][icol];
    minv[icol][icol] = 1.0;
    for (int j = 0; j < 4; ++j) minv[icol][j] *= pivinv;
    for (int j = 0; j < 4; ++j) {
      if (j == icol) continue;
      const double save = minv[j][icol];
      minv[j][icol] = 0;
      for (int k = 0; k < 4; ++k) minv[j][k] -= minv[icol][k] * save;
    }
  }
  for (int j = 3; j >= 0; --j)
    if (indxr[j] != indxc[j])
      for (int k = 0; k < 4; ++k) std::swap(minv[k][indxr[j]], minv[k][indxc[j]]);
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) out[4 * r + c] = minv[r][c];
  return !singular;
}

namespace {

// A mesh's triangles, dropping those TriangleMesh drops (an out-of-range or
// repeated vertex index, TriangleMesh.cpp:176-182; mesh triangle indices
// count the kept ones), in mesh space or through `m` (Transform on
// Point3D_f), appended to the builder with primitive id `prim`.
struct MeshJob {
  const MeshIn *m;
  const double *xf;
  int32_t prim;
};

inline bool dropped(const MeshIn &m, int64_t t) {
  const int32_t *ix = m.triangles + 3 * t;
  for (int k = 0; k < 3; ++k)
    if (ix[k] < 0 || (int64_t)ix[k] >= m.n_vertices) return true;
  return ix[0] == ix[1] || ix[0] == ix[2] || ix[1] == ix[2];
}

// Runs f(c) for c in [0, n) on up to `threads` threads.
template <class F>
void parallel_for(size_t n, int threads, F &&f) {
  const size_t nt = std::min<size_t>(n, (size_t)std::max(threads, 1));
  if (nt <= 1) {
    for (size_t c = 0; c < n; ++c) f(c);
    return;
  }
  std::atomic<size_t> next{0};
  std::vector<std::thread> pool;
  for (size_t w = 0; w < nt; ++w)
    pool.emplace_back([&]() {
      for (size_t c; (c = next.fetch_add(1)) < n;) f(c);
    });
  for (std::thread &t : pool) t.join();
}

// The meshes' triangles, dropping those TriangleMesh drops (an
// out-of-range or repeated vertex index, TriangleMesh.cpp:176-182; mesh
// triangle indices count the kept ones), in mesh space or through each
// job's matrix (Transform on Point3D_f), appended to the builder in job
// order with the job's primitive id.  Chunks of triangles are counted,
// then filled, on several threads; the result is the sequential one.
void add_meshes(Builder &B, const std::vector<MeshJob> &jobs, int threads) {
  constexpr int64_t kChunk = 1 << 15;
  struct Chunk {
    size_t job;
    int64_t t0, t1;
    size_t out = 0;
    int32_t kept_before = 0;  // kept triangles of the job before the chunk
    int64_t kept = 0;
  };
  std::vector<Chunk> chunks;
  for (size_t j = 0; j < jobs.size(); ++j)
    for (int64_t t0 = 0; t0 < jobs[j].m->n_triangles; t0 += kChunk)
      chunks.push_back(Chunk{j, t0, std::min(jobs[j].m->n_triangles, t0 + kChunk)});
  parallel_for(chunks.size(), threads, [&](size_t c) {
    Chunk &k = chunks[c];
    int64_t kept = 0;
    for (int64_t t = k.t0; t < k.t1; ++t) kept += dropped(*jobs[k.job].m, t) ? 0 : 1;
    k.kept = kept;
  });
  size_t total = B.prim.size();
  for (size_t c = 0; c < chunks.size(); ++c) {
    chunks[c].out = total;
    chunks[c].kept_before = (c > 0 && chunks[c - 1].job == chunks[c].job)
                                ? chunks[c - 1].kept_before + (int32_t)chunks[c - 1].kept
                                : 0;
    total += (size_t)chunks[c].kept;
  }
  const size_t base = B.prim.size();
  B.tv.resize(9 * total);
  B.prim.resize(total);
  B.tidx.resize(total);
  B.tbox.resize(total);
  B.order.resize(total);
  for (size_t i = base; i < total; ++i) B.order[i] = (uint32_t)i;
  parallel_for(chunks.size(), threads, [&](size_t c) {
    const Chunk &k = chunks[c];
    const MeshJob &jb = jobs[k.job];
    const MeshIn &m = *jb.m;
    size_t o = k.out;
    int32_t kept = k.kept_before;
    for (int64_t t = k.t0; t < k.t1; ++t) {
      if (dropped(m, t)) continue;
      const int32_t *ix = m.triangles + 3 * t;
      float *v = &B.tv[9 * o];
      for (int q = 0; q < 3; ++q) {
        const float *src = m.vertices + 3 * (int64_t)ix[q];
        if (jb.xf) {
          transform_point(jb.xf, src, v + 3 * q);
        } else {
          v[3 * q] = src[0];
          v[3 * q + 1] = src[1];
          v[3 * q + 2] = src[2];
        }
      }
      BoxF b;
      for (int q = 0; q < 3; ++q) {
        for (int a = 0; a < 3; ++a) {
          b.lo[a] = std::min(b.lo[a], v[3 * q + a]);
          b.hi[a] = std::max(b.hi[a], v[3 * q + a]);
        }
      }
      B.prim[o] = jb.prim;
      B.tidx[o] = kept++;
      B.tbox[o] = b;
      ++o;
    }
  });
}

void add_mesh_triangles(Builder &B, const MeshIn &m, const double *xf, int32_t prim) {
  add_meshes(B, {MeshJob{&m, xf, prim}}, B.threads);
}

// Pre-order flattening of one tree into out.nodes; a node's present
// children occupy consecutive slots.  Returns the root's index.
uint32_t flatten(const BNode *root, FlatTree &out) {
  const uint32_t root_idx = (uint32_t)out.nodes.size();
  out.nodes.emplace_back();
  std::vector<std::pair<const BNode *, uint32_t>> stack{{root, root_idx}};
  while (!stack.empty()) {
    auto [bn, idx] = stack.back();
    stack.pop_back();
    DevNode dn{};
    for (int k = 0; k < 3; ++k) {
      dn.lo[k] = bn->box.lo[k];
      dn.hi[k] = bn->box.hi[k];
    }
    if (bn->flags == 0) {
      if (bn->ie > bn->ib) {
        dn.a = (uint32_t)out.leaf_ext.size();
        dn.b = kLeafExt;
        out.leaf_ext.push_back(LeafExt{bn->tb, bn->te - bn->tb, bn->ib, bn->ie - bn->ib});
      } else {
        dn.a = bn->tb;
        dn.b = (uint32_t)(bn->te - bn->tb) << 8;
      }
    } else {
      uint32_t first = (uint32_t)out.nodes.size(), mask = 0, slot = first;
      std::pair<const BNode *, uint32_t> kids[3];
      int nk = 0;
      for (int c = 0; c < 3; ++c)
        if (bn->child[c]) {
          mask |= 1u << c;
          kids[nk++] = {bn->child[c].get(), slot++};
          out.nodes.emplace_back();
        }
      dn.a = first;
      dn.b = (uint32_t)bn->flags | (mask << 2);
      for (int k = nk - 1; k >= 0; --k) stack.push_back(kids[k]);
    }
    out.nodes[idx] = dn;
  }
  return root_idx;
}

// The same pre-order flattening over the GPU build's node records.
uint32_t flatten_records(const AccelTreeGpu &g, FlatTree &out) {
  const uint32_t root_idx = (uint32_t)out.nodes.size();
  out.nodes.emplace_back();
  std::vector<std::pair<int64_t, uint32_t>> stack{{0, root_idx}};
  while (!stack.empty()) {
    auto [id, idx] = stack.back();
    stack.pop_back();
    DevNode dn{};
    for (int k = 0; k < 3; ++k) {
      dn.lo[k] = g.box[(size_t)id * 6 + k];
      dn.hi[k] = g.box[(size_t)id * 6 + 3 + k];
    }
    if (g.flags[(size_t)id] == 0) {
      dn.a = g.tb[(size_t)id];
      dn.b = (g.te[(size_t)id] - g.tb[(size_t)id]) << 8;
    } else {
      uint32_t first = (uint32_t)out.nodes.size(), mask = 0, slot = first;
      std::pair<int64_t, uint32_t> kids[3];
      int nk = 0;
      for (int c = 0; c < 3; ++c) {
        const int32_t ch = g.child[(size_t)id * 3 + c];
        if (ch >= 0) {
          mask |= 1u << c;
          kids[nk++] = {ch, slot++};
          out.nodes.emplace_back();
        }
      }
      dn.a = first;
      dn.b = (uint32_t)g.flags[(size_t)id] | (mask << 2);
      for (int k = nk - 1; k >= 0; --k) stack.push_back(kids[k]);
    }
    out.nodes[idx] = dn;
  }
  return root_idx;
}

const double kIdentity[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};

}  // namespace

std::string build_accel_device(const MeshIn *meshes, int32_t n_meshes, const PrimIn *prims, int32_t n_prims,
                               int threads, cudaStream_t st, int64_t min_gpu, FlatTree &out, bool *on_gpu) {
  if (on_gpu) *on_gpu = false;
  if (n_prims < 0 || n_meshes < 0) return "negative primitive or mesh count";
  std::vector<int> uses((size_t)n_meshes, 0);
  int64_t n_tris = 0;
  for (int32_t p = 0; p < n_prims; ++p) {
    if (prims[p].mesh < 0 || prims[p].mesh >= n_meshes) return "primitive references a mesh index out of range";
    ++uses[(size_t)prims[p].mesh];
    n_tris += meshes[prims[p].mesh].n_triangles;
  }
  bool shared = false;
  for (int u : uses) shared = shared || u > 1;
  if (shared || n_tris < std::max<int64_t>(min_gpu, 1))
    return build_accel(meshes, n_meshes, prims, n_prims, threads, out);
  for (int32_t p = 0; p < n_prims; ++p) {
    const MeshIn &m = meshes[prims[p].mesh];
    if (m.n_triangles > 0 && (!m.triangles || !m.vertices)) return "mesh has triangles but null arrays";
  }
  // Steps 3-4 of the reference's constructor: the primitives' triangles in
  // world space, then the tree over them (on the GPU).
  Builder B;
  unsigned hw = std::thread::hardware_concurrency();
  B.threads = threads > 0 ? threads : (int)(hw ? hw : 1);
  {
    std::vector<MeshJob> jobs;
    for (int32_t p = 0; p < n_prims; ++p) jobs.push_back(MeshJob{&meshes[prims[p].mesh], prims[p].mesh_to_world, p});
    add_meshes(B, jobs, B.threads);
  }
  const size_t n = B.prim.size();
  if (n > (size_t)INT32_MAX / 2) return "too many triangles";
  if (n < (size_t)std::max<int64_t>(min_gpu, 1)) return build_accel(meshes, n_meshes, prims, n_prims, threads, out);
  static_assert(sizeof(BoxF) == 24, "BoxF is 6 floats");
  AccelTreeGpu g;
  cudaError_t e = build_accel_tree_gpu(reinterpret_cast<const float *>(B.tbox.data()), (int64_t)n, st, g);
  if (e != cudaSuccess) return std::string("GPU tree build: ") + cudaGetErrorString(e);
  if (g.inconsistent) return build_accel(meshes, n_meshes, prims, n_prims, threads, out);
  out = FlatTree();
  out.nodes.reserve((size_t)g.n_nodes);
  flatten_records(g, out);
  out.tris.resize(n);
  const size_t gchunks = (n + 65535) / 65536;
  parallel_for(gchunks, B.threads, [&](size_t c) {
    for (size_t i = c * 65536; i < std::min(n, (c + 1) * 65536); ++i) {
      DevTri &t = out.tris[i];
      const size_t o = g.perm[i];
      std::memcpy(t.v0, &B.tv[9 * o], 12);
      std::memcpy(t.v1, &B.tv[9 * o + 3], 12);
      std::memcpy(t.v2, &B.tv[9 * o + 6], 12);
      t.prim = B.prim[o];
      t.tri = B.tidx[o];
      t.slot = (int32_t)i;
    }
  });
  out.max_depth = g.max_depth;
  out.n_leaves = g.n_leaves;
  for (int k = 0; k < 6; ++k) out.bounds[k] = g.box[(size_t)k];
  if (on_gpu) *on_gpu = true;
  return "";
}

std::string build_accel(const MeshIn *meshes, int32_t n_meshes, const PrimIn *prims, int32_t n_prims, int threads,
                        FlatTree &out) {
  if (n_prims < 0 || n_meshes < 0) return "negative primitive or mesh count";
  std::vector<int> uses((size_t)n_meshes, 0);
  for (int32_t p = 0; p < n_prims; ++p) {
    if (prims[p].mesh < 0 || prims[p].mesh >= n_meshes) return "primitive references a mesh index out of range";
    ++uses[(size_t)prims[p].mesh];
    const MeshIn &m = meshes[prims[p].mesh];
    if (m.n_triangles > 0 && (!m.triangles || !m.vertices)) return "mesh has triangles but null arrays";
  }
  Builder B;
  unsigned hw = std::thread::hardware_concurrency();
  B.threads = threads > 0 ? threads : (int)(hw ? hw : 1);
  B.threads_left = B.threads - 1;
  out = FlatTree();

  // Step 2 of the reference's constructor: every mesh used by more than one
  // primitive gets a subtree over its mesh-space triangles, and each of its
  // primitives an instance whose world box is the union of the subtree
  // box's eight corners transformed to world space.  Meshes in index order
  // (the reference orders them by address, which follows creation order).
  std::vector<std::unique_ptr<BNode>> subtrees;
  std::vector<std::vector<double>> inverses((size_t)n_prims);
  for (int32_t mi = 0; mi < n_meshes; ++mi) {
    if (uses[(size_t)mi] < 2) continue;
    const size_t tb = B.prim.size();
    add_mesh_triangles(B, meshes[mi], nullptr, -1);
    const size_t te = B.prim.size();
    subtrees.push_back(B.build(tb, te, 0, 0, 0u, 0));
    const BNode *sub = subtrees.back().get();
    for (int32_t p = 0; p < n_prims; ++p) {
      if (prims[p].mesh != mi) continue;
      const double *xf = prims[p].mesh_to_world ? prims[p].mesh_to_world : kIdentity;
      BoxF ib;
      for (int j = 0; j < 8; ++j) {
        const float corner[3] = {(j & 1) ? sub->box.lo[0] : sub->box.hi[0], (j & 2) ? sub->box.lo[1] : sub->box.hi[1],
                                 (j & 4) ? sub->box.lo[2] : sub->box.hi[2]};
        float w[3];
        transform_point(xf, corner, w);
        for (int c = 0; c < 3; ++c) {
          ib.lo[c] = std::min(ib.lo[c], w[c]);
          ib.hi[c] = std::max(ib.hi[c], w[c]);
        }
      }
      std::vector<double> inv(16);
      if (!invert4(xf, inv.data())) return "a primitive's mesh-to-world matrix is singular";
      inverses[(size_t)p] = inv;
      B.ibox.push_back(ib);
      B.icount.push_back(te - tb);
      B.iprim.push_back(p);
      B.isub.push_back((int32_t)subtrees.size() - 1);
    }
  }
  // Step 3: the primitives that own their mesh, in world space.
  const size_t shared_end = B.prim.size();
  {
    std::vector<MeshJob> jobs;
    for (int32_t p = 0; p < n_prims; ++p)
      if (uses[(size_t)prims[p].mesh] < 2) jobs.push_back(MeshJob{&meshes[prims[p].mesh], prims[p].mesh_to_world, p});
    add_meshes(B, jobs, B.threads);
  }
  const size_t n = B.prim.size(), n_inst = B.ibox.size();
  if (n > (size_t)INT32_MAX) return "too many triangles";

  if (n == shared_end && n_inst == 0) {
    // An empty accelerator: a single empty leaf whose box culls every ray.
    DevNode leaf{};
    for (int k = 0; k < 3; ++k) {
      leaf.lo[k] = kInfF;
      leaf.hi[k] = -kInfF;
    }
    leaf.a = 0;
    leaf.b = 0;
    out.nodes.push_back(leaf);
    out.max_depth = 0;
    out.n_leaves = 1;
    for (int k = 0; k < 6; ++k) out.bounds[k] = 0.f;
    return "";
  }
  // Step 4: the tree over the world triangles and the instances.
  std::unique_ptr<BNode> root = B.build(shared_end, n, 0, n_inst, 0u, 0);
  out.nodes.reserve(n + 1);
  flatten(root.get(), out);
  for (const auto &sub : subtrees) out.subtree_roots.push_back(flatten(sub.get(), out));
  out.tris.resize(n);
  for (size_t i = 0; i < n; ++i) {
    DevTri &t = out.tris[i];
    const size_t o = B.order[i];
    std::memcpy(t.v0, &B.tv[9 * o], 12);
    std::memcpy(t.v1, &B.tv[9 * o + 3], 12);
    std::memcpy(t.v2, &B.tv[9 * o + 6], 12);
    t.prim = B.prim[o];
    t.tri = B.tidx[o];
    t.slot = (int32_t)i;
  }
  out.inst.resize(n_inst);
  for (size_t i = 0; i < n_inst; ++i) {
    DevInst &d = out.inst[i];
    std::memcpy(d.world_to_mesh, inverses[(size_t)B.iprim[i]].data(), sizeof(d.world_to_mesh));
    d.root = out.subtree_roots[(size_t)B.isub[i]];
    d.prim = B.iprim[i];
    d.pad[0] = d.pad[1] = 0;
  }
  out.max_depth = B.max_depth.load();
  out.n_leaves = B.n_leaves.load();
  for (int k = 0; k < 3; ++k) {
    out.bounds[k] = root->box.lo[k];
    out.bounds[3 + k] = root->box.hi[k];
  }
  return "";
}

}  // namespace skw
