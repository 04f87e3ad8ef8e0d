/* The reference's kd-tree, restated for the CPU oracle.  TEST
 * INFRASTRUCTURE ONLY: included by oracle.cpp, which tests/, smoke() and
 * bench.py's CPU-baseline leg load.
 *
 * Follows Primitive/KdTree.hs:
 *   - build (mkKdTree / buildTree / trySplit / bestSplit / cost / edges /
 *     partition, KdTree.hs:81-203): exact-event SAH with cT = 1, cI = 80,
 *     empty bonus 0.5, maximum depth round(8 + 3 ln N); axes tried from the
 *     node's largest extent on, the first axis whose cheapest split beats
 *     leaf cost cI * N wins; primitives go left when their start edge lies
 *     before the split edge and right when their end edge lies after it,
 *     in edge order;
 *   - traversal (traverse / traverse', KdTree.hs:209-246): front-to-back
 *     recursion with the split distance tp = (split - o) * (1 / d), the
 *     near side chosen by `o < split || (o == split && d <= 0)`, subtrees
 *     beyond the closest hit so far skipped (`rayMax < tmin`), and leaf
 *     primitives tested against the whole ray in leaf order with the
 *     `nearest'` fold (Primitive.hs:29-43): a later primitive with an equal
 *     distance replaces the earlier one;
 *   - the root interval from intersectAABB (AABB.hs:79-94).
 * Arithmetic is binary32 in the reference's operation order; min/max are
 * GHC's Ord defaults (`if x <= y`).
 *
 * One thing cannot be restated: edges are sorted by vector-algorithms'
 * introsort (Data.Vector.Algorithms.Intro, pinned through stackage lts-8.13;
 * not vendored), which is not stable, so the order of edges with equal
 * position and kind is that library's.  Here such edges keep primitive-ID
 * order.  The choice only moves primitives whose bound lies exactly on a
 * split plane and the order of equal-distance hits within a leaf.
 *
 * The build sorts every axis once and partitions the sorted edge lists
 * (each node's lists equal what sorting its own edges gives), and builds
 * large subtrees on separate threads, as the reference sparks them
 * (`par left`, KdTree.hs:130). */
#pragma once
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <thread>
#include <vector>

namespace kd {

inline float gmin(float x, float y) { return x <= y ? x : y; }
inline float gmax(float x, float y) { return x <= y ? y : x; }

struct Box {
  float lo[3], hi[3];
};

// interior: axis 0..2, split plane, children a (left) and b (right);
// leaf: axis 3, primitives leafPrims[a, a + b)
struct Node {
  int axis;
  float split;
  int32_t a, b;
};

struct Stats {
  int64_t interiors = 0, leaves = 0, empty_leaves = 0, leaf_refs = 0, max_leaf = 0;
  int64_t max_depth = 0, depth_sum = 0;
};

struct Tree {
  Box bounds{};
  int depth_limit = 0;
  std::vector<Node> nodes;  // root is node 0
  std::vector<int32_t> leafPrims;
  Stats stats;
};

// cT, cI (KdTree.hs:81-87)
constexpr float kCT = 1.0f;
constexpr float kCI = 80.0f;

// surfaceArea (AABB.hs:68-71)
inline float surfaceArea(const Box& b) {
  float dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
  return 2.0f * (dx * dy + dx * dz + dy * dz);
}

// maximumExtent = dominant (pmax - pmin) (AABB.hs:49-51, Math.hs:292-301)
inline int maximumExtent(const Box& b) {
  float ax = std::fabs(b.hi[0] - b.lo[0]), ay = std::fabs(b.hi[1] - b.lo[1]),
        az = std::fabs(b.hi[2] - b.lo[2]);
  if (ax > ay && ax > az) return 0;
  if (ay > az) return 1;
  return 2;
}

// the SAH cost (KdTree.hs:187-203)
inline float cost(const Box& b, int a0, float t, int64_t nl, int64_t nr) {
  float d[3] = {b.hi[0] - b.lo[0], b.hi[1] - b.lo[1], b.hi[2] - b.lo[2]};
  int a1 = (a0 + 1) % 3, a2 = (a0 + 2) % 3;
  float dl = t - b.lo[a0], dr = b.hi[a0] - t;
  float sal = 2.0f * (d[a1] * d[a2] + dl * (d[a1] + d[a2]));
  float sar = 2.0f * (d[a1] * d[a2] + dr * (d[a1] + d[a2]));
  float invTotSa = 1.0f / surfaceArea(b);
  float pl = sal * invTotSa, pr = sar * invTotSa;
  float eb = (nl == 0 || nr == 0) ? 0.5f : 1.0f;
  float pI = pl * (float)nl + pr * (float)nr;
  return kCT + kCI * eb * pI;
}

// an edge: position, primitive and kind (start edges sort before end edges
// at equal position, Edge's Ord instance, KdTree.hs:94-100)
struct Edge {
  float t;
  uint32_t code;  // primitive << 1 | (1 for an end edge)
  bool end() const { return code & 1u; }
  int32_t prim() const { return (int32_t)(code >> 1); }
};
inline bool edgeLess(const Edge& x, const Edge& y) {
  if (x.t != y.t) return x.t < y.t;
  if (x.end() != y.end()) return !x.end();
  return x.code < y.code;  // equal position and kind: primitive-ID order
}

class Builder {
 public:
  Builder(const std::vector<Box>& boxes, int nthreads) : boxes_(boxes), budget_(nthreads - 1) {}

  void build(Tree& T) {
    const int64_t n = (int64_t)boxes_.size();
    Box b{{INFINITY, INFINITY, INFINITY}, {-INFINITY, -INFINITY, -INFINITY}};  // mempty
    for (const Box& p : boxes_)  // V.foldl' mappend mempty (KdTree.hs:111)
      for (int k = 0; k < 3; k++) {
        b.lo[k] = gmin(b.lo[k], p.lo[k]);
        b.hi[k] = gmax(b.hi[k], p.hi[k]);
      }
    T.bounds = b;
    // md = round (8 + 3 * log N) in binary32; `round` rounds halves to even
    float md = 8.0f + 3.0f * logf((float)n);
    T.depth_limit = n > 0 ? (int)std::nearbyint(md) : 0;
    std::vector<int32_t> prims(n);
    for (int64_t i = 0; i < n; i++) prims[i] = (int32_t)i;
    std::vector<Edge> es[3];
    for (int a = 0; a < 3; a++) {
      es[a].resize(2 * n);
      for (int64_t i = 0; i < n; i++) {
        es[a][2 * i] = Edge{boxes_[i].lo[a], (uint32_t)i << 1};
        es[a][2 * i + 1] = Edge{boxes_[i].hi[a], ((uint32_t)i << 1) | 1u};
      }
    }
    sortAll(es);
    Frag f;
    buildNode(f, b, std::move(prims), es, T.depth_limit, 0);
    T.nodes = std::move(f.nodes);
    T.leafPrims = std::move(f.leafPrims);
    T.stats = f.stats;
  }

 private:
  struct Frag {
    std::vector<Node> nodes;
    std::vector<int32_t> leafPrims;
    Stats stats;
    std::vector<uint8_t> mark;  // per primitive: 1 left, 2 right (scratch)
  };

  const std::vector<Box>& boxes_;
  std::atomic<int> budget_;  // threads that may still be started

  void sortAll(std::vector<Edge> (&es)[3]) {
    std::vector<std::thread> th;
    for (int a = 1; a < 3; a++)
      if (es[a].size() > 100000 && budget_.fetch_sub(1) > 0)
        th.emplace_back([&es, a] { std::sort(es[a].begin(), es[a].end(), edgeLess); });
      else
        std::sort(es[a].begin(), es[a].end(), edgeLess);
    std::sort(es[0].begin(), es[0].end(), edgeLess);
    for (auto& t : th) {
      t.join();
      budget_.fetch_add(1);
    }
  }

  static void addLeaf(Frag& f, int idx, const std::vector<int32_t>& prims, int level) {
    f.nodes[idx] = Node{3, 0.0f, (int32_t)f.leafPrims.size(), (int32_t)prims.size()};
    f.leafPrims.insert(f.leafPrims.end(), prims.begin(), prims.end());
    f.stats.leaves += 1;
    f.stats.empty_leaves += prims.empty() ? 1 : 0;
    f.stats.leaf_refs += (int64_t)prims.size();
    f.stats.max_leaf = std::max<int64_t>(f.stats.max_leaf, (int64_t)prims.size());
    f.stats.max_depth = std::max<int64_t>(f.stats.max_depth, level);
    f.stats.depth_sum += level;
  }

  // trySplit (KdTree.hs:121-139): the split of the first axis whose
  // cheapest split (bestSplit/allSplits/filterSplits, :141-167) costs less
  // than a leaf.  Returns false for a leaf.
  static bool trySplit(const Box& b, int64_t n, const std::vector<Edge> (&es)[3], int& axis,
                       int64_t& at, float& t) {
    const float oldCost = kCI * (float)n;
    const int a0 = maximumExtent(b);
    for (int k = 0; k < 3; k++) {
      const int a = (a0 + k) % 3;
      const float tmin = b.lo[a], tmax = b.hi[a];
      const std::vector<Edge>& e = es[a];
      bool any = false;
      float best = INFINITY;
      int64_t bi = -1;
      float bt = 0.0f;
      int64_t l = 0, r = n;
      for (int64_t i = 0; i < (int64_t)e.size(); i++) {
        int64_t nl = l, nr = r;
        if (e[i].end()) {
          nr = r - 1;
          r -= 1;
        } else {
          l += 1;
        }
        const float ti = e[i].t;
        if (!(ti > tmin && ti < tmax)) continue;
        any = true;
        float c = cost(b, a, ti, nl, nr);
        if (c < best) {
          best = c;
          bi = i;
          bt = ti;
        }
      }
      if (!any) continue;
      if (best < oldCost) {
        axis = a;
        at = bi;
        t = bt;
        return true;
      }
    }
    return false;
  }

  int buildNode(Frag& f, const Box& b, std::vector<int32_t> prims, std::vector<Edge> (&es)[3],
                int depth, int level) {
    const int idx = (int)f.nodes.size();
    f.nodes.push_back(Node{});
    const int64_t n = (int64_t)prims.size();
    int axis = 0;
    int64_t at = 0;
    float t = 0.0f;
    if (depth == 0 || n <= 1 || !trySplit(b, n, es, axis, at, t)) {  // buildTree (:114-119)
      addLeaf(f, idx, prims, level);
      return idx;
    }
    // partition (:146-150): left = start edges before the split edge, right =
    // end edges after it, both in edge order
    if (f.mark.size() < boxes_.size()) f.mark.assign(boxes_.size(), 0);
    std::vector<int32_t> lp, rp;
    const std::vector<Edge>& e = es[axis];
    for (int64_t i = 0; i < at; i++)
      if (!e[i].end()) {
        lp.push_back(e[i].prim());
        f.mark[e[i].prim()] |= 1;
      }
    for (int64_t i = at + 1; i < (int64_t)e.size(); i++)
      if (e[i].end()) {
        rp.push_back(e[i].prim());
        f.mark[e[i].prim()] |= 2;
      }
    std::vector<Edge> le[3], re[3];
    for (int a = 0; a < 3; a++) {
      le[a].reserve(2 * lp.size());
      re[a].reserve(2 * rp.size());
      for (const Edge& x : es[a]) {
        uint8_t m = f.mark[x.prim()];
        if (m & 1) le[a].push_back(x);
        if (m & 2) re[a].push_back(x);
      }
      std::vector<Edge>().swap(es[a]);
    }
    for (int32_t p : prims) f.mark[p] = 0;
    std::vector<int32_t>().swap(prims);
    // splitAABB (AABB.hs:73-77)
    Box lb = b, rb = b;
    lb.hi[axis] = t;
    rb.lo[axis] = t;
    f.nodes[idx] = Node{axis, t, -1, -1};
    f.stats.interiors += 1;
    int left, right;
    if (lp.size() > 50000 && budget_.fetch_sub(1) > 0) {
      Frag lf;
      std::thread th([&] { buildNode(lf, lb, std::move(lp), le, depth - 1, level + 1); });
      right = buildNode(f, rb, std::move(rp), re, depth - 1, level + 1);
      th.join();
      budget_.fetch_add(1);
      left = append(f, lf);
    } else {
      budget_.fetch_add(lp.size() > 50000 ? 1 : 0);
      left = buildNode(f, lb, std::move(lp), le, depth - 1, level + 1);
      right = buildNode(f, rb, std::move(rp), re, depth - 1, level + 1);
    }
    f.nodes[idx].a = left;
    f.nodes[idx].b = right;
    return idx;
  }

  // moves fragment g (root at its node 0) into f; returns the root's new index
  static int append(Frag& f, Frag& g) {
    const int32_t no = (int32_t)f.nodes.size(), lo = (int32_t)f.leafPrims.size();
    for (Node nd : g.nodes) {
      if (nd.axis == 3) {
        nd.a += lo;
      } else {
        nd.a += no;
        nd.b += no;
      }
      f.nodes.push_back(nd);
    }
    f.leafPrims.insert(f.leafPrims.end(), g.leafPrims.begin(), g.leafPrims.end());
    f.stats.interiors += g.stats.interiors;
    f.stats.leaves += g.stats.leaves;
    f.stats.empty_leaves += g.stats.empty_leaves;
    f.stats.leaf_refs += g.stats.leaf_refs;
    f.stats.max_leaf = std::max(f.stats.max_leaf, g.stats.max_leaf);
    f.stats.max_depth = std::max(f.stats.max_depth, g.stats.max_depth);
    f.stats.depth_sum += g.stats.depth_sum;
    return no;
  }
};

inline void build(Tree& T, const std::vector<Box>& boxes, int nthreads) {
  Builder(boxes, std::max(1, nthreads)).build(T);
}

// visit counts of one query (dbgTraverse's statistic, KdTree.hs:252-281)
struct Counts {
  int64_t nodes = 0, prims = 0;
};

// traverse (KdTree.hs:222-234).  R has o[3], d[3] and tmax (rayMax, lowered
// by each hit as `near` does); hit(p) tests primitive p against R and, on a
// hit, sets R's tmax and records the hit.
template <class R, class HitFn>
void closest(const Tree& T, int ni, R& r, const float inv[3], float tmin, float tmax, HitFn& hit,
             Counts& c) {
  const Node& n = T.nodes[ni];
  c.nodes += 1;
  if (n.axis == 3) {  // nearest' over the leaf, in leaf order
    for (int32_t k = 0; k < n.b; k++) hit(T.leafPrims[n.a + k], r);
    c.prims += n.b;
    return;
  }
  if (r.tmax < tmin) return;
  const int a = n.axis;
  const float o = r.o[a], d = r.d[a];
  const float tp = (n.split - o) * inv[a];
  const bool lf = o < n.split || (o == n.split && d <= 0);
  const int fc = lf ? n.a : n.b, sc = lf ? n.b : n.a;
  if (tp > tmax || tp <= 0) {
    closest(T, fc, r, inv, tmin, tmax, hit, c);
  } else if (tp < tmin) {
    closest(T, sc, r, inv, tmin, tmax, hit, c);
  } else {
    closest(T, fc, r, inv, tmin, tp, hit, c);
    closest(T, sc, r, inv, tp, tmax, hit, c);
  }
}

// traverse' (KdTree.hs:209-220)
template <class R, class AnyFn>
bool any(const Tree& T, int ni, const R& r, const float inv[3], float tmin, float tmax,
         AnyFn& hit, Counts& c) {
  const Node& n = T.nodes[ni];
  c.nodes += 1;
  if (n.axis == 3) {
    for (int32_t k = 0; k < n.b; k++) {
      c.prims += 1;
      if (hit(T.leafPrims[n.a + k], r)) return true;
    }
    return false;
  }
  const int a = n.axis;
  const float o = r.o[a], d = r.d[a];
  const float tp = (n.split - o) * inv[a];
  const bool lf = o < n.split || (o == n.split && d <= 0);
  const int fc = lf ? n.a : n.b, sc = lf ? n.b : n.a;
  if (tp > tmax || tp <= 0) return any(T, fc, r, inv, tmin, tmax, hit, c);
  if (tp < tmin) return any(T, sc, r, inv, tmin, tmax, hit, c);
  return any(T, fc, r, inv, tmin, tp, hit, c) || any(T, sc, r, inv, tp, tmax, hit, c);
}

// intersectAABB of the root box (AABB.hs:79-94): the ray's [tmin, tmax]
// clipped by the slabs, or false
inline bool rootInterval(const Box& b, const float o[3], const float d[3], float tmin, float tmax,
                         float& n_out, float& f_out) {
  float nr = tmin, fr = tmax;
  for (int dim = 0; dim < 3; dim++) {
    if (nr > fr) return false;
    float dInv = 1.0f / d[dim];
    float tFar = (b.hi[dim] - o[dim]) * dInv;
    float tNear = (b.lo[dim] - o[dim]) * dInv;
    float nn = tNear > tFar ? tFar : tNear, ff = tNear > tFar ? tNear : tFar;
    nr = gmax(nr, nn);
    fr = gmin(fr, ff);
  }
  if (nr > fr) return false;
  n_out = nr;
  f_out = fr;
  return true;
}

}  // namespace kd
