// ORACLE -- test infrastructure only.  A CPU restatement of the reference's
// ray-query and photon-lookup algorithms, used by tests/, smoke() and the
// CPU-baseline leg of bench.py as the checker.  The product never links,
// loads or calls it.
//
// Parity is pinned (tests/test_oracle_pins.py) against the reference itself,
// built from its own sources into oracle/_ref by oracle/build_ref.py, and
// against golden vectors generated from that build (tests/golden/).
//
// Every function names the reference code it restates (paths in the Skwarka
// source tree).  Arithmetic is double over float data exactly where the
// reference's is; this file is compiled with -ffp-contract=off.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <limits>
#include <memory>
#include <thread>
#include <type_traits>
#include <vector>

namespace {

const double kInfD = std::numeric_limits<double>::infinity();
const float kInfF = std::numeric_limits<float>::infinity();
const double kDblEps = std::numeric_limits<double>::epsilon();

void for_ranges(int64_t n, int threads, const std::function<void(int64_t, int64_t)> &fn) {
  unsigned nt = threads > 0 ? (unsigned)threads : std::max(1u, std::thread::hardware_concurrency());
  if (nt <= 1 || n < 512) {
    fn(0, n);
    return;
  }
  std::atomic<int64_t> next(0);
  std::vector<std::thread> th;
  auto work = [&]() {
    for (;;) {
      int64_t s = next.fetch_add(128);
      if (s >= n) break;
      fn(s, std::min(n, s + 128));
    }
  };
  for (unsigned i = 1; i < nt; ++i) th.emplace_back(work);
  work();
  for (auto &t : th) t.join();
}

// ------------------------------------------------------------------ tree --
// BBox3D<float> / BBox3D<double> (Math/BBox3D.h:121-215).
struct BoxF {
  float lo[3] = {kInfF, kInfF, kInfF}, hi[3] = {-kInfF, -kInfF, -kInfF};
};
struct BoxD {
  double lo[3] = {kInfD, kInfD, kInfD}, hi[3] = {-kInfD, -kInfD, -kInfD};
};
template <class A, class B>
void unite(A &a, const B &b) {
  typedef typename std::remove_reference<decltype(a.lo[0])>::type T;
  for (int k = 0; k < 3; ++k) {
    a.lo[k] = std::min(a.lo[k], (T)b.lo[k]);
    a.hi[k] = std::max(a.hi[k], (T)b.hi[k]);
  }
}
float areaf(const BoxF &b) {
  float x = std::fabs(b.hi[0] - b.lo[0]), y = std::fabs(b.hi[1] - b.lo[1]), z = std::fabs(b.hi[2] - b.lo[2]);
  return (float)2.0 * (x * y + x * z + y * z);
}
double aread(const BoxD &b) {
  double x = std::fabs(b.hi[0] - b.lo[0]), y = std::fabs(b.hi[1] - b.lo[1]), z = std::fabs(b.hi[2] - b.lo[2]);
  return 2.0 * (x * y + x * z + y * z);
}
// (size_t)double with the x86-64 g++ results for NaN (2^63) and +inf (0).
size_t to_size(double v) {
  if (std::isnan(v)) return (size_t)1 << 63;
  if (v >= 18446744073709551616.0) return 0;
  if (v >= 9223372036854775808.0) return (size_t)(v - 9223372036854775808.0) + ((size_t)1 << 63);
  return (size_t)(int64_t)v;
}

struct Node {
  BoxF box;
  int child[3] = {-1, -1, -1};
  size_t tb = 0, te = 0;
  unsigned char flags = 0;  // (TriangleAccelerator.h:193-213): 0 leaf, axis+1 internal
};

struct Accel {
  std::vector<float> tv;  // 9 floats per triangle
  std::vector<int32_t> prim, tidx;
  std::vector<BoxF> tbox;
  std::vector<Node> nodes;  // nodes[0] = root
  int root = -1;

  void swap_tris(size_t a, size_t b) {  // _SwapTriangles (TriangleAccelerator.cpp:483-492)
    for (int k = 0; k < 9; ++k) std::swap(tv[9 * a + k], tv[9 * b + k]);
    std::swap(prim[a], prim[b]);
    std::swap(tidx[a], tidx[b]);
    std::swap(tbox[a], tbox[b]);
  }

  // _DetermineBestSplit (TriangleAccelerator.cpp:505-617), no instances.
  std::pair<int, double> best_split(const BoxF &nb, size_t tb, size_t te, unsigned mask) const {
    const size_t n = te - tb;
    double best_pos[3] = {0, 0, 0}, best_cost[3] = {kInfD, kInfD, kInfD};
    for (int axis = 0; axis < 3; ++axis) {
      if (mask & (1u << axis)) continue;
      BoxD L[200], M[200], R[200];
      size_t Ln[200] = {0}, Mn[200] = {0}, Rn[200] = {0};
      size_t tries = std::min((size_t)200, 2 * n);
      double coef = tries / (nb.hi[axis] - nb.lo[axis]);  // size_t / float -> float division
      for (size_t i = 0; i < n; ++i) {
        const BoxF &b = tbox[tb + i];
        size_t lb = std::min(tries, to_size((b.hi[axis] - nb.lo[axis]) * coef + 1.0));
        size_t re = std::min(tries, to_size((b.lo[axis] - nb.lo[axis]) * coef + 1.0));
        if (re > 0) {
          unite(R[re - 1], b);
          Rn[re - 1] += 1;
        }
        if (lb < tries) {
          unite(L[lb], b);
          Ln[lb] += 1;
        }
        for (size_t j = re; j < lb; ++j) {
          unite(M[j], b);
          Mn[j] += 1;
        }
      }
      for (size_t i = 1; i < tries; ++i) {
        unite(L[i], L[i - 1]);
        Ln[i] += Ln[i - 1];
      }
      for (int i = (int)tries - 2; i >= 0; --i) {
        unite(R[i], R[i + 1]);
        Rn[i] += Rn[i + 1];
      }
      double inv_area = 1.0 / areaf(nb);
      for (size_t i = 0; i < tries; ++i) {
        double p1 = std::min(1.0, aread(L[i]) * inv_area);
        double p2 = std::min(1.0, aread(M[i]) * inv_area);
        double p3 = std::min(1.0, aread(R[i]) * inv_area);
        double cost = Ln[i] * p1 + Mn[i] * p2 + Rn[i] * p3;
        if (Ln[i] == 0 || Rn[i] == 0) cost *= 0.8;
        if (cost < best_cost[axis]) {
          best_cost[axis] = cost;
          best_pos[axis] = nb.lo[axis] + i * (nb.hi[axis] - nb.lo[axis]) / tries;  // float arithmetic
        }
      }
    }
    if (best_cost[0] <= best_cost[1] && best_cost[0] <= best_cost[2]) return {0, best_pos[0]};
    if (best_cost[1] <= best_cost[0] && best_cost[1] <= best_cost[2]) return {1, best_pos[1]};
    return {2, best_pos[2]};
  }

  // Node::Node (TriangleAccelerator.cpp:621-729), no instances.
  int build(size_t tb, size_t te, unsigned mask, size_t depth) {
    int id = (int)nodes.size();
    nodes.emplace_back();
    BoxF box;
    for (size_t i = tb; i < te; ++i) unite(box, tbox[i]);
    nodes[id].box = box;
    nodes[id].tb = tb;
    nodes[id].te = te;
    if (te - tb <= 4 || mask == 7u || depth >= 200) return id;
    std::pair<int, double> sp = best_split(box, tb, te, mask);
    int axis = sp.first;
    double split = sp.second;
    nodes[id].flags = (unsigned char)(axis + 1);
    size_t mb = tb, rb = te, i = tb;
    while (i < rb) {
      const BoxF &b = tbox[i];
      if (b.hi[axis] < split) {
        swap_tris(mb, i);
        ++mb;
        ++i;
      } else if (b.lo[axis] > split) {
        --rb;
        swap_tris(i, rb);
      } else {
        ++i;
      }
    }
    int c0 = tb < mb ? build(tb, mb, mask, depth + 1) : -1;
    int c1 = mb < rb ? build(mb, rb, mask | (1u << axis), depth + 1) : -1;
    int c2 = rb < te ? build(rb, te, mask, depth + 1) : -1;
    nodes[id].child[0] = c0;
    nodes[id].child[1] = c1;
    nodes[id].child[2] = c2;
    return id;
  }
};

struct RayD {
  double o[3], d[3], tmin, tmax;
};

RayD ray_from(const float *r) {
  RayD ray;
  for (int k = 0; k < 3; ++k) {
    ray.o[k] = r[k];
    ray.d[k] = r[3 + k];
  }
  ray.tmin = r[6];
  ray.tmax = r[7];
  return ray;
}

RayD ray_from_d(const double *r) {
  RayD ray;
  for (int k = 0; k < 3; ++k) {
    ray.o[k] = r[k];
    ray.d[k] = r[3 + k];
  }
  ray.tmin = r[6];
  ray.tmax = r[7];
  return ray;
}

// Slab test of _NodeIntersect (TriangleAccelerator.cpp:176-192); true = culled.
bool culled(const BoxF &b, const RayD &ray, const double inv[3], double tmin, double tmax) {
  double tn[3], tf[3];
  for (int k = 0; k < 3; ++k) {
    tn[k] = (b.lo[k] - ray.o[k]) * inv[k];
    tf[k] = (b.hi[k] - ray.o[k]) * inv[k];
    if (tn[k] > tf[k]) std::swap(tn[k], tf[k]);
  }
  return tmin > tf[0] || tn[0] > tf[1] || tn[1] > tf[0] || tn[2] > tf[0] || tmin > tf[1] || tn[0] > tf[2] ||
         tn[1] > tf[2] || tn[2] > tf[1] || tmin > tf[2] || tn[0] > tmax || tn[1] > tmax || tn[2] > tmax;
}

// Moller-Trumbore in double (TriangleAccelerator.cpp:240-273): returns true
// and t when the reference accepts the triangle for [tmin, tmax].
bool tri_hit(const float *v, const RayD &ray, double tmin, double tmax, double &t_out) {
  double v0[3] = {v[0], v[1], v[2]}, v1[3] = {v[3], v[4], v[5]}, v2[3] = {v[6], v[7], v[8]};
  double e1[3], e2[3], d[3];
  for (int k = 0; k < 3; ++k) {
    e1[k] = v1[k] - v0[k];
    e2[k] = v2[k] - v0[k];
    d[k] = ray.o[k] - v0[k];
  }
  const double *dir = ray.d;
  double s1[3] = {dir[1] * e2[2] - dir[2] * e2[1], dir[2] * e2[0] - dir[0] * e2[2], dir[0] * e2[1] - dir[1] * e2[0]};
  double divisor = s1[0] * e1[0] + s1[1] * e1[1] + s1[2] * e1[2];
  double inv_divisor = 1.0 / divisor;
  double b1 = (d[0] * s1[0] + d[1] * s1[1] + d[2] * s1[2]) * inv_divisor;
  if (b1 > -kDblEps && b1 < (1.0 + kDblEps)) {
    double s2[3] = {d[1] * e1[2] - d[2] * e1[1], d[2] * e1[0] - d[0] * e1[2], d[0] * e1[1] - d[1] * e1[0]};
    double b2 = (dir[0] * s2[0] + dir[1] * s2[1] + dir[2] * s2[2]) * inv_divisor;
    if (b2 > -kDblEps && b1 + b2 < (1.0 + kDblEps)) {
      double t = (e2[0] * s2[0] + e2[1] * s2[1] + e2[2] * s2[2]) * inv_divisor;
      if (t >= tmin && t <= tmax) {
        t_out = t;
        return true;
      }
    }
  }
  return false;
}

// ---------------------------------------------------------------- photons --
// KDTree<T>::Node (Raytracer/Core/KDTree.h:188-246): float split, union of
// right-child index (bits 3..31) and flags (bits 0-1 axis or 3 = leaf,
// bit 2 = has left child).
struct KNode {
  float split;
  uint32_t word;
};
struct KPoint {
  float p[3];
  int32_t orig;
  uint16_t normal_id;
};

struct KDTreeO {
  std::vector<KPoint> pts;
  std::vector<KNode> nodes;

  // _Build (KDTree.h:428-473) -- std::nth_element with the same comparator,
  // so the permutation equals the reference's for the same standard library.
  void build(size_t b, size_t e) {
    if (b + 1 == e) {
      nodes[b].word = (nodes[b].word & ~3u) + 3u;
      return;
    }
    BoxD box;
    for (size_t i = b; i < e; ++i) {
      BoxD pb;
      for (int k = 0; k < 3; ++k) pb.lo[k] = pb.hi[k] = (double)pts[i].p[k];
      unite(box, pb);
    }
    int axis = 0;
    if (box.hi[1] - box.lo[1] > box.hi[axis] - box.lo[axis]) axis = 1;
    if (box.hi[2] - box.lo[2] > box.hi[axis] - box.lo[axis]) axis = 2;
    size_t split_index = (b + e) / 2;
    std::nth_element(pts.begin() + b, pts.begin() + split_index, pts.begin() + e,
                     [axis](const KPoint &a, const KPoint &c) { return a.p[axis] < c.p[axis]; });
    std::swap(pts[b], pts[split_index]);
    nodes[b].word = (nodes[b].word & ~3u) + (uint32_t)axis;
    nodes[b].split = pts[b].p[axis];
    if (b < split_index) {
      nodes[b].word = (nodes[b].word & ~4u) + 4u;
      build(b + 1, split_index + 1);
    } else {
      nodes[b].word = nodes[b].word & ~4u;
    }
    if (split_index + 1 < e) {
      nodes[b].word = ((uint32_t)(split_index + 1) << 3) + (nodes[b].word & 7u);
      build(split_index + 1, e);
    } else {
      nodes[b].word = (((1u << 29) - 1) << 3) + (nodes[b].word & 7u);
    }
  }
};

// CompressedDirection table (Math/CompressedDirection.cpp:21-41).
std::vector<double> g_dir_table;
void init_dir_table() {
  if (!g_dir_table.empty()) return;
  g_dir_table.resize(3 << 16);
  for (int i = 0; i < (1 << 16); ++i) {
    unsigned char x = (unsigned char)((i & 0x1FC0) >> 6), y = (unsigned char)(i & 0x3F);
    if (x + y >= 127) {
      x = (unsigned char)(127 - x);
      y = (unsigned char)(127 - y);
    }
    double v[3] = {x + 0.5, y + 0.5, 126.0 - x - y};
    double ls = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    if (ls > 0.0) {  // Vector3D::Normalize (Math/Vector3D.h:260-270): multiply by 1/len
      double inv = 1.0 / std::sqrt(ls);
      for (int k = 0; k < 3; ++k) v[k] *= inv;
    }
    if (i & (1 << 13)) v[0] = -v[0];
    if (i & (1 << 14)) v[1] = -v[1];
    if (i & (1 << 15)) v[2] = -v[2];
    for (int k = 0; k < 3; ++k) g_dir_table[3 * i + k] = v[k];
  }
}

struct Cand {
  int32_t idx;
  double d2;
  bool operator<(const Cand &o) const { return d2 == o.d2 ? idx < o.idx : d2 < o.d2; }  // KDTree.h:174-177
};

// PhotonFilter (PhotonInternalTypes.h:113-137).
struct Filter {
  bool on;
  double q[3], n[3], cos_t, sin_t;
  bool pass(const KPoint &p) const {
    if (!on) return true;
    const double *pn = &g_dir_table[3 * p.normal_id];
    double to[3] = {(double)p.p[0] - q[0], (double)p.p[1] - q[1], (double)p.p[2] - q[2]};
    double len = std::sqrt(to[0] * to[0] + to[1] * to[1] + to[2] * to[2]);
    return (pn[0] * n[0] + pn[1] * n[1] + pn[2] * n[2]) > cos_t &&
           std::fabs(to[0] * n[0] + to[1] * n[1] + to[2] * n[2]) < sin_t * len;
  }
};

// _Lookup (KDTree.h:537-576) with NearestPointsProc (KDTree.h:331-387).
struct KnnProc {
  const Filter *f;
  size_t k;
  std::vector<Cand> heap;
  int64_t visited = 0;
  void visit(const KDTreeO &t, size_t ni, const double q[3], double &maxd2) {
    ++visited;
    const KPoint &pt = t.pts[ni];
    double dx = pt.p[0] - q[0], dy = pt.p[1] - q[1], dz = pt.p[2] - q[2];
    double d2 = dx * dx + dy * dy + dz * dz;
    if (d2 < maxd2 && f->pass(pt)) {
      if (heap.size() < k) {
        heap.push_back(Cand{(int32_t)ni, d2});
        if (heap.size() == k) {
          std::make_heap(heap.begin(), heap.end());
          maxd2 = heap[0].d2;
        }
      } else {
        std::pop_heap(heap.begin(), heap.end());
        heap[k - 1] = Cand{(int32_t)ni, d2};
        std::push_heap(heap.begin(), heap.end());
        maxd2 = heap[0].d2;
      }
    }
    uint32_t w = t.nodes[ni].word;
    if ((w & 3u) != 3u) {
      unsigned axis = w & 3u;
      double split = t.nodes[ni].split;
      double pd = (q[axis] - split) * (q[axis] - split);
      size_t right = w >> 3;
      bool has_left = (w & 4u) != 0;
      if (q[axis] <= split) {
        if (has_left) visit(t, ni + 1, q, maxd2);
        if (pd < maxd2 && right < t.nodes.size()) visit(t, right, q, maxd2);
      } else {
        if (right < t.nodes.size()) visit(t, right, q, maxd2);
        if (pd < maxd2 && has_left) visit(t, ni + 1, q, maxd2);
      }
    }
  }
};

}  // namespace

extern "C" {

int oracle_version(void) { return 1; }

// -------------------------------------------------------------- accelerator
// Triangles come as world-space float xyz (9 per triangle) with their
// primitive / mesh-triangle ids, in primitive order (TriangleAccelerator ctor
// steps 3-4, TriangleAccelerator.cpp:104-139).
void *oracle_accel_create(const float *tris, const int32_t *prim, const int32_t *tidx, int64_t n) {
  auto *a = new Accel();
  a->tv.assign(tris, tris + 9 * n);
  a->prim.assign(prim, prim + n);
  a->tidx.assign(tidx, tidx + n);
  a->tbox.resize((size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    BoxF b;
    for (int v = 0; v < 3; ++v)
      for (int k = 0; k < 3; ++k) {
        b.lo[k] = std::min(b.lo[k], tris[9 * i + 3 * v + k]);
        b.hi[k] = std::max(b.hi[k], tris[9 * i + 3 * v + k]);
      }
    a->tbox[(size_t)i] = b;
  }
  if (n > 0) a->root = a->build(0, (size_t)n, 0u, 0);
  return a;
}

void oracle_accel_destroy(void *a) { delete (Accel *)a; }
int64_t oracle_accel_num_nodes(void *a) { return (int64_t)((Accel *)a)->nodes.size(); }

// Same export layout as the reference driver: pre-order, children L, M, R.
void oracle_accel_export(void *ap, float *node_bbox, int32_t *node_info, int32_t *tri_prim, int32_t *tri_idx) {
  Accel &a = *(Accel *)ap;
  std::vector<int> order, pos(a.nodes.size(), -1);
  std::vector<int> st;
  if (a.root >= 0) st.push_back(a.root);
  while (!st.empty()) {
    int id = st.back();
    st.pop_back();
    pos[(size_t)id] = (int)order.size();
    order.push_back(id);
    for (int c = 2; c >= 0; --c)
      if (a.nodes[(size_t)id].child[c] >= 0) st.push_back(a.nodes[(size_t)id].child[c]);
  }
  for (size_t i = 0; i < order.size(); ++i) {
    const Node &nd = a.nodes[(size_t)order[i]];
    for (int k = 0; k < 3; ++k) {
      node_bbox[6 * i + k] = nd.box.lo[k];
      node_bbox[6 * i + 3 + k] = nd.box.hi[k];
    }
    int32_t *info = node_info + 8 * i;
    info[0] = nd.flags;
    for (int c = 0; c < 3; ++c) info[1 + c] = nd.child[c] >= 0 ? pos[(size_t)nd.child[c]] : -1;
    info[4] = (int32_t)nd.tb;
    info[5] = (int32_t)nd.te;
    info[6] = 0;
    info[7] = 0;
  }
  for (size_t i = 0; i < a.prim.size(); ++i) {
    tri_prim[i] = a.prim[i];
    tri_idx[i] = a.tidx[i];
  }
}

// Closest hit: _NodeIntersect (TriangleAccelerator.cpp:154-293).
// counters (optional): per ray nodes popped, triangles tested.
// rays_d (if rays is null): 8 doubles per ray, the reference's own Ray.
static void intersect_impl(void *ap, const float *rays, const double *rays_d, int64_t n, int32_t *prim, int32_t *tri,
                           double *t_out, int32_t *nodes_visited, int32_t *tris_tested, int threads) {
  const Accel &a = *(Accel *)ap;
  for_ranges(n, threads, [&](int64_t b, int64_t e) {
    std::vector<int> todo(401);
    for (int64_t i = b; i < e; ++i) {
      RayD ray = rays ? ray_from(rays + 8 * i) : ray_from_d(rays_d + 8 * i);
      double inv[3] = {1.0 / ray.d[0], 1.0 / ray.d[1], 1.0 / ray.d[2]};
      int sp = 0, nv = 0, nt = 0;
      if (a.root >= 0) todo[(size_t)sp++] = a.root;
      long best = -1;
      while (sp > 0) {
        const Node &nd = a.nodes[(size_t)todo[(size_t)--sp]];
        ++nv;
        if (culled(nd.box, ray, inv, ray.tmin, ray.tmax)) continue;
        if (nd.flags) {
          int axis = nd.flags - 1;
          if (ray.d[axis] > 0.0) {
            for (int c = 2; c >= 0; --c)
              if (nd.child[c] >= 0) todo[(size_t)sp++] = nd.child[c];
          } else {
            for (int c = 0; c < 3; ++c)
              if (nd.child[c] >= 0) todo[(size_t)sp++] = nd.child[c];
          }
        } else {
          for (size_t k = nd.tb; k < nd.te; ++k) {
            ++nt;
            double th;
            if (tri_hit(&a.tv[9 * k], ray, ray.tmin, ray.tmax, th)) {
              ray.tmax = th;
              best = (long)k;
            }
          }
        }
      }
      prim[i] = best >= 0 ? a.prim[(size_t)best] : -1;
      tri[i] = best >= 0 ? a.tidx[(size_t)best] : -1;
      t_out[i] = best >= 0 ? ray.tmax : kInfD;
      if (nodes_visited) nodes_visited[i] = nv;
      if (tris_tested) tris_tested[i] = nt;
    }
  });
}

void oracle_intersect(void *ap, const float *rays, int64_t n, int32_t *prim, int32_t *tri, double *t_out,
                      int32_t *nodes_visited, int32_t *tris_tested, int threads) {
  intersect_impl(ap, rays, nullptr, n, prim, tri, t_out, nodes_visited, tris_tested, threads);
}

void oracle_intersect_d(void *ap, const double *rays, int64_t n, int32_t *prim, int32_t *tri, double *t_out,
                        int threads) {
  intersect_impl(ap, nullptr, rays, n, prim, tri, t_out, nullptr, nullptr, threads);
}

// Any hit: _NodeIntersectTest (TriangleAccelerator.cpp:354-462).
static void intersect_test_impl(void *ap, const float *rays, const double *rays_d, int64_t n, uint8_t *occluded,
                                int32_t *nodes_visited, int32_t *tris_tested, int threads) {
  const Accel &a = *(Accel *)ap;
  for_ranges(n, threads, [&](int64_t b, int64_t e) {
    std::vector<int> todo(401);
    for (int64_t i = b; i < e; ++i) {
      RayD ray = rays ? ray_from(rays + 8 * i) : ray_from_d(rays_d + 8 * i);
      double inv[3] = {1.0 / ray.d[0], 1.0 / ray.d[1], 1.0 / ray.d[2]};
      int sp = 0, nv = 0, nt = 0;
      if (a.root >= 0) todo[(size_t)sp++] = a.root;
      bool hit = false;
      while (sp > 0 && !hit) {
        const Node &nd = a.nodes[(size_t)todo[(size_t)--sp]];
        ++nv;
        if (culled(nd.box, ray, inv, ray.tmin, ray.tmax)) continue;
        if (nd.flags) {
          int axis = nd.flags - 1;
          if (ray.d[axis] > 0.0) {
            for (int c = 2; c >= 0; --c)
              if (nd.child[c] >= 0) todo[(size_t)sp++] = nd.child[c];
          } else {
            for (int c = 0; c < 3; ++c)
              if (nd.child[c] >= 0) todo[(size_t)sp++] = nd.child[c];
          }
        } else {
          for (size_t k = nd.tb; k < nd.te && !hit; ++k) {
            ++nt;
            double th;
            if (tri_hit(&a.tv[9 * k], ray, ray.tmin, ray.tmax, th)) hit = true;
          }
        }
      }
      occluded[i] = hit ? 1 : 0;
      if (nodes_visited) nodes_visited[i] = nv;
      if (tris_tested) tris_tested[i] = nt;
    }
  });
}

void oracle_intersect_test(void *ap, const float *rays, int64_t n, uint8_t *occluded, int32_t *nodes_visited,
                           int32_t *tris_tested, int threads) {
  intersect_test_impl(ap, rays, nullptr, n, occluded, nodes_visited, tris_tested, threads);
}

void oracle_intersect_test_d(void *ap, const double *rays, int64_t n, uint8_t *occluded, int threads) {
  intersect_test_impl(ap, nullptr, rays, n, occluded, nullptr, nullptr, threads);
}

// Brute force over all triangles in input order, the unit test's check
// (UnitTests/MainTests/Raytracer/Core/TriangleAccelerator.test.h:213-269):
// nearest accepted t, ties to the later triangle.
void oracle_brute_force(const float *tris, const int32_t *prim, const int32_t *tidx, int64_t nt, const float *rays,
                        int64_t n, int32_t *prim_out, int32_t *tri_out, double *t_out, int threads) {
  for_ranges(n, threads, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      RayD ray = ray_from(rays + 8 * i);
      long best = -1;
      for (int64_t k = 0; k < nt; ++k) {
        double th;
        if (tri_hit(tris + 9 * k, ray, ray.tmin, ray.tmax, th)) {
          ray.tmax = th;
          best = (long)k;
        }
      }
      prim_out[i] = best >= 0 ? prim[best] : -1;
      tri_out[i] = best >= 0 ? tidx[best] : -1;
      t_out[i] = best >= 0 ? ray.tmax : kInfD;
    }
  });
}

// ----------------------------------------------------------------- photons
void *oracle_kdtree_create(const float *pos, const uint16_t *normal_ids, int64_t n, int32_t *perm_out,
                           uint32_t *node_words) {
  init_dir_table();
  auto *t = new KDTreeO();
  t->pts.resize((size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    KPoint &p = t->pts[(size_t)i];
    for (int k = 0; k < 3; ++k) p.p[k] = pos[3 * i + k];
    p.orig = (int32_t)i;
    p.normal_id = normal_ids ? normal_ids[i] : 0;
  }
  t->nodes.assign((size_t)n, KNode{0.f, 0u});
  if (n > 0) t->build(0, (size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    if (perm_out) perm_out[i] = t->pts[(size_t)i].orig;
    if (node_words) {
      std::memcpy(&node_words[2 * i], &t->nodes[(size_t)i].split, 4);
      node_words[2 * i + 1] = t->nodes[(size_t)i].word;
    }
  }
  return t;
}

void oracle_kdtree_destroy(void *t) { delete (KDTreeO *)t; }

// GetNearestPoints (KDTree.h:506-533) with PhotonFilter when cos_threshold >=
// 0.  Output slots hold the heap order; visited (optional) = nodes visited.
void oracle_knn(void *tp, const double *q, const double *qn, int64_t nq, int32_t k, double max_dist,
                double cos_threshold, int32_t *out_idx, double *out_d2, int32_t *out_count, int32_t *visited,
                int threads) {
  init_dir_table();
  const KDTreeO &t = *(KDTreeO *)tp;
  for_ranges(nq, threads, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      Filter f;
      f.on = cos_threshold >= 0;
      for (int c = 0; c < 3; ++c) {
        f.q[c] = q[3 * i + c];
        f.n[c] = qn ? qn[3 * i + c] : 0.0;
      }
      f.cos_t = cos_threshold;
      f.sin_t = f.on ? std::sqrt(1.0 - cos_threshold * cos_threshold) : 0.0;
      KnnProc proc;
      proc.f = &f;
      proc.k = (size_t)k;
      double maxd2 = max_dist * max_dist;
      if (k > 0 && !t.nodes.empty()) proc.visit(t, 0, f.q, maxd2);
      out_count[i] = (int32_t)proc.heap.size();
      for (int32_t j = 0; j < k; ++j) {
        out_idx[i * k + j] = (size_t)j < proc.heap.size() ? proc.heap[(size_t)j].idx : -1;
        out_d2[i * k + j] = (size_t)j < proc.heap.size() ? proc.heap[(size_t)j].d2 : 0.0;
      }
      if (visited) visited[i] = (int32_t)proc.visited;
    }
  });
}

// GetNearestPoint (KDTree.h:485-503) with NearestPointProc (KDTree.h:293-323)
// and, when cos_threshold >= 0, PhotonFilter.
struct NearestProc {
  const Filter *f;
  int32_t best = -1;
  void visit(const KDTreeO &t, size_t ni, const double q[3], double &maxd2) {
    const KPoint &pt = t.pts[ni];
    double dx = pt.p[0] - q[0], dy = pt.p[1] - q[1], dz = pt.p[2] - q[2];
    double d2 = dx * dx + dy * dy + dz * dz;
    if (d2 < maxd2 && f->pass(pt)) {
      best = (int32_t)ni;
      maxd2 = d2;
    }
    uint32_t w = t.nodes[ni].word;
    if ((w & 3u) != 3u) {
      unsigned axis = w & 3u;
      double split = t.nodes[ni].split;
      double pd = (q[axis] - split) * (q[axis] - split);
      size_t right = w >> 3;
      bool has_left = (w & 4u) != 0;
      if (q[axis] <= split) {
        if (has_left) visit(t, ni + 1, q, maxd2);
        if (pd < maxd2 && right < t.nodes.size()) visit(t, right, q, maxd2);
      } else {
        if (right < t.nodes.size()) visit(t, right, q, maxd2);
        if (pd < maxd2 && has_left) visit(t, ni + 1, q, maxd2);
      }
    }
  }
};

void oracle_nearest(void *tp, const double *q, const double *qn, int64_t nq, double max_dist, double cos_threshold,
                    int32_t *out_idx, int threads) {
  init_dir_table();
  const KDTreeO &t = *(KDTreeO *)tp;
  for_ranges(nq, threads, [&](int64_t b, int64_t e) {
    for (int64_t i = b; i < e; ++i) {
      Filter f;
      f.on = cos_threshold >= 0;
      for (int c = 0; c < 3; ++c) {
        f.q[c] = q[3 * i + c];
        f.n[c] = qn ? qn[3 * i + c] : 0.0;
      }
      f.cos_t = cos_threshold;
      f.sin_t = f.on ? std::sqrt(1.0 - cos_threshold * cos_threshold) : 0.0;
      NearestProc proc;
      proc.f = &f;
      double maxd2 = max_dist * max_dist;
      if (!t.nodes.empty()) proc.visit(t, 0, f.q, maxd2);
      out_idx[i] = proc.best;
    }
  });
}

void oracle_compressed_direction_table(double *out) {
  init_dir_table();
  std::memcpy(out, g_dir_table.data(), g_dir_table.size() * sizeof(double));
}

}  // extern "C"
