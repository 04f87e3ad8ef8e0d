// Binned-SAH BVH builder (host, multi-threaded).  See bvh.h.
#include "bvh.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <future>
#include <thread>

namespace bgpu {
namespace {

struct Box {
  float lo[3], hi[3];
  void reset() {
    for (int k = 0; k < 3; k++) {
      lo[k] = INFINITY;
      hi[k] = -INFINITY;
    }
  }
  void grow(const float* l, const float* h) {
    for (int k = 0; k < 3; k++) {
      lo[k] = std::min(lo[k], l[k]);
      hi[k] = std::max(hi[k], h[k]);
    }
  }
  void grow(const Box& b) { grow(b.lo, b.hi); }
  float area() const {
    float d[3];
    for (int k = 0; k < 3; k++) d[k] = std::max(0.0f, hi[k] - lo[k]);
    return 2.0f * (d[0] * d[1] + d[0] * d[2] + d[1] * d[2]);
  }
};

struct BNode {
  Box box;
  int left = -1, right = -1;  // children (internal)
  int64_t begin = 0, count = 0;  // leaf range in refs when count > 0
};

constexpr int kBins = 32;
constexpr int64_t kParallelGrain = 1 << 15;

struct Builder {
  const BvhBuildInput& in;
  std::vector<int32_t> refs;
  std::vector<float> cen;  // 3n
  std::vector<BNode> nodes;
  std::atomic<int64_t> next{1};
  std::atomic<int> max_depth{0};
  std::atomic<int> live_tasks{0};
  int max_tasks;

  explicit Builder(const BvhBuildInput& i) : in(i) {
    int64_t n = in.n;
    refs.resize(n);
    cen.resize(3 * n);
    for (int64_t k = 0; k < n; k++) {
      refs[k] = (int32_t)k;
      for (int a = 0; a < 3; a++) cen[3 * k + a] = 0.5f * (in.lo[3 * k + a] + in.hi[3 * k + a]);
    }
    nodes.resize(std::max<int64_t>(1, 2 * n));
    unsigned hc = std::thread::hardware_concurrency();
    max_tasks = in.threads > 0 ? in.threads : (hc ? (int)hc : 1);
  }

  void make_leaf(int64_t idx, int64_t b, int64_t e) {
    nodes[idx].begin = b;
    nodes[idx].count = e - b;
  }

  void build(int64_t idx, int64_t b, int64_t e, int depth) {
    int md = max_depth.load();
    while (depth > md && !max_depth.compare_exchange_weak(md, depth)) {
    }
    Box box, cbox;
    box.reset();
    cbox.reset();
    for (int64_t k = b; k < e; k++) {
      int32_t r = refs[k];
      box.grow(&in.lo[3 * r], &in.hi[3 * r]);
      cbox.grow(&cen[3 * r], &cen[3 * r]);
    }
    nodes[idx].box = box;
    int64_t count = e - b;
    if (count <= 1) {
      make_leaf(idx, b, e);
      return;
    }
    int64_t mid = -1;
    bool force_median = depth >= kBvhMaxDepth - 28;  // keeps depth < kBvhMaxDepth for n < 2^27
    if (!force_median) {
      // binned SAH over centroids
      float best_cost = INFINITY;
      int best_axis = -1, best_bin = -1;
      float parent_area = box.area();
      for (int a = 0; a < 3; a++) {
        float ext = cbox.hi[a] - cbox.lo[a];
        if (!(ext > 0)) continue;
        int nb = (int)std::min<int64_t>(kBins, count);
        float k1 = (float)nb * (1.0f - 1e-6f) / ext;
        Box bb[kBins];
        int64_t bc[kBins];
        for (int i = 0; i < nb; i++) {
          bb[i].reset();
          bc[i] = 0;
        }
        for (int64_t k = b; k < e; k++) {
          int32_t r = refs[k];
          int bi = std::min(nb - 1, std::max(0, (int)((cen[3 * r + a] - cbox.lo[a]) * k1)));
          bc[bi]++;
          bb[bi].grow(&in.lo[3 * r], &in.hi[3 * r]);
        }
        float rarea[kBins];
        int64_t rcount[kBins];
        Box acc;
        acc.reset();
        int64_t cnt = 0;
        for (int i = nb - 1; i > 0; i--) {
          acc.grow(bb[i]);
          cnt += bc[i];
          rarea[i] = acc.area();
          rcount[i] = cnt;
        }
        acc.reset();
        cnt = 0;
        for (int i = 0; i < nb - 1; i++) {
          acc.grow(bb[i]);
          cnt += bc[i];
          if (cnt == 0 || rcount[i + 1] == 0) continue;
          float c = acc.area() * (float)cnt + rarea[i + 1] * (float)rcount[i + 1];
          if (c < best_cost) {
            best_cost = c;
            best_axis = a;
            best_bin = i;
          }
        }
      }
      float leaf_cost = (float)count * parent_area;
      float split_cost = parent_area + best_cost;  // traversal step costs one box area
      if (best_axis < 0 || (count <= in.max_leaf && leaf_cost <= split_cost)) {
        if (best_axis < 0 && count > in.max_leaf) {
          force_median = true;  // all centroids coincide
        } else {
          make_leaf(idx, b, e);
          return;
        }
      }
      if (!force_median) {
        int a = best_axis;
        int nb = (int)std::min<int64_t>(kBins, count);
        float k1 = (float)nb * (1.0f - 1e-6f) / (cbox.hi[a] - cbox.lo[a]);
        float lo = cbox.lo[a];
        auto it = std::partition(refs.begin() + b, refs.begin() + e, [&](int32_t r) {
          int bi = std::min(nb - 1, std::max(0, (int)((cen[3 * r + a] - lo) * k1)));
          return bi <= best_bin;
        });
        mid = it - refs.begin();
        if (mid == b || mid == e) force_median = true;
      }
    }
    if (force_median) {
      if (count <= in.max_leaf) {
        make_leaf(idx, b, e);
        return;
      }
      int a = 0;
      for (int k = 1; k < 3; k++)
        if (cbox.hi[k] - cbox.lo[k] > cbox.hi[a] - cbox.lo[a]) a = k;
      mid = b + count / 2;
      std::nth_element(refs.begin() + b, refs.begin() + mid, refs.begin() + e,
                       [&](int32_t x, int32_t y) {
                         float cx = cen[3 * x + a], cy = cen[3 * y + a];
                         return cx < cy || (cx == cy && x < y);
                       });
    }
    int64_t l = next.fetch_add(2);
    nodes[idx].left = (int)l;
    nodes[idx].right = (int)(l + 1);
    if (count > kParallelGrain && live_tasks.load() < max_tasks) {
      live_tasks++;
      auto fut = std::async(std::launch::async, [&, l, b, mid, depth]() { build(l, b, mid, depth + 1); });
      build(l + 1, mid, e, depth + 1);
      fut.get();
      live_tasks--;
    } else {
      build(l, b, mid, depth + 1);
      build(l + 1, mid, e, depth + 1);
    }
  }
};

// ---- 8-wide quantised layout
struct WideItem {
  int64_t bnode;
  int64_t wide;
  int depth;
};

static float box_area(const Box& b) { return b.area(); }

// collapse: replace the internal child of largest area by its two children
// until there are eight children or only leaves
static int collapse(const Builder& B, int64_t b, int64_t kids[8]) {
  int n = 2;
  kids[0] = B.nodes[b].left;
  kids[1] = B.nodes[b].right;
  while (n < 8) {
    int best = -1;
    float best_a = -1;
    for (int i = 0; i < n; i++) {
      const BNode& k = B.nodes[kids[i]];
      if (k.count > 0) continue;
      float a = box_area(k.box);
      if (a > best_a) {
        best_a = a;
        best = i;
      }
    }
    if (best < 0) break;
    int64_t x = kids[best];
    kids[best] = B.nodes[x].left;
    kids[n++] = B.nodes[x].right;
  }
  return n;
}

static bool build_wide(const Builder& B, BvhBuildOutput& out) {
  out.nodes8.clear();
  out.slot_prim8.clear();
  out.slot_last8.clear();
  out.wide_depth = 0;
  auto add_leaf = [&](const BNode& nd) {
    for (int64_t k = 0; k < nd.count; k++) {
      out.slot_prim8.push_back(B.refs[nd.begin + k]);
      out.slot_last8.push_back(k + 1 == nd.count ? 1 : 0);
    }
  };
  const BNode& root = B.nodes[0];
  if (root.count > 0) {
    out.root8 = ~(int32_t)out.slot_prim8.size();
    add_leaf(root);
    return true;
  }
  out.root8 = 0;
  out.nodes8.resize(20);
  std::vector<WideItem> queue;
  queue.push_back(WideItem{0, 0, 1});
  for (size_t qi = 0; qi < queue.size(); qi++) {
    WideItem it = queue[qi];
    out.wide_depth = std::max(out.wide_depth, it.depth);
    int64_t kids[8];
    int n = collapse(B, it.bnode, kids);
    const Box& nb = B.nodes[it.bnode].box;
    // octant slot assignment: slot s gets the child that comes first along the
    // diagonal of octant s (bit k of s set: direction component k negative)
    double nc[3];
    for (int a = 0; a < 3; a++) nc[a] = 0.5 * ((double)nb.lo[a] + nb.hi[a]);
    int64_t slot_kid[8];
    bool used[8] = {false};
    for (int s = 0; s < 8; s++) slot_kid[s] = -1;
    for (int s = 0; s < 8; s++) {
      int best = -1;
      double best_d = 0;
      for (int i = 0; i < n; i++) {
        if (used[i]) continue;
        const Box& kb = B.nodes[kids[i]].box;
        double d = 0;
        for (int a = 0; a < 3; a++) {
          double c = 0.5 * ((double)kb.lo[a] + kb.hi[a]) - nc[a];
          d += (s >> a & 1) ? -c : c;
        }
        if (best < 0 || d < best_d) {
          best = i;
          best_d = d;
        }
      }
      if (best < 0) break;
      used[best] = true;
      slot_kid[s] = kids[best];
    }
    // children: internal ones become consecutive wide nodes, leaves consecutive slots
    uint32_t child_base = (uint32_t)(out.nodes8.size() / 20);
    uint32_t slot_base = (uint32_t)out.slot_prim8.size();
    uint8_t meta[8];
    int rank = 0;
    for (int s = 0; s < 8; s++) {
      meta[s] = 0xFF;
      if (slot_kid[s] < 0) continue;
      const BNode& k = B.nodes[slot_kid[s]];
      if (k.count == 0) {
        meta[s] = (uint8_t)(0x80 | rank);
        queue.push_back(WideItem{slot_kid[s], (int64_t)child_base + rank, it.depth + 1});
        rank++;
      } else {
        size_t off = out.slot_prim8.size() - slot_base;
        if (off > 127) return false;
        meta[s] = (uint8_t)off;
        add_leaf(k);
      }
    }
    out.nodes8.resize(out.nodes8.size() + 20 * (size_t)rank);
    // quantisation: origin p = node minimum, scale 2^e with 255 * 2^e covering the extent
    uint32_t* w = &out.nodes8[20 * it.wide];
    uint8_t q[6][8];
    uint32_t ebits = 0;
    for (int a = 0; a < 3; a++) {
      double lo = nb.lo[a], hi = nb.hi[a];
      double ext = hi - lo;
      int e = -100;
      if (ext > 0) {
        e = (int)std::ceil(std::log2(ext * (1.0 + 1.0 / 1024.0) / 255.0));
        while (std::ldexp(255.0, e) < ext * (1.0 + 1.0 / 1024.0)) e++;
      }
      e = std::max(-126, std::min(127, e));
      ebits |= (uint32_t)(e + 127) << (8 * a);
      double scale = std::ldexp(1.0, e);
      for (int s = 0; s < 8; s++) {
        if (slot_kid[s] < 0) {
          q[a][s] = 255;
          q[3 + a][s] = 0;
          continue;
        }
        const Box& kb = B.nodes[slot_kid[s]].box;
        double ql = std::floor(((double)kb.lo[a] - lo) / scale) - 1;
        double qh = std::ceil(((double)kb.hi[a] - lo) / scale) + 1;
        ql = std::max(0.0, std::min(255.0, ql));
        qh = std::max(0.0, std::min(255.0, qh));
        // the decoded box must contain the child box
        if (lo + ql * scale > (double)kb.lo[a] || lo + qh * scale < (double)kb.hi[a]) return false;
        q[a][s] = (uint8_t)ql;
        q[3 + a][s] = (uint8_t)qh;
      }
    }
    float p[3] = {nb.lo[0], nb.lo[1], nb.lo[2]};
    memcpy(&w[0], p, 12);
    w[3] = ebits;
    w[4] = child_base;
    w[5] = slot_base;
    memcpy(&w[6], meta, 8);
    // qlo.x qlo.y qlo.z qhi.x qhi.y qhi.z, 8 bytes each
    for (int r = 0; r < 6; r++) memcpy(&w[8 + 2 * r], q[r], 8);
  }
  return out.wide_depth <= kWideStack / 7 - 1;
}

// ---- 32-byte quantised binary layout
// quantises child box kb into the node frame (origin lo, scales 2^e[a]) with
// one quantum of margin; false if the decoded box would not contain kb
static bool quantise(const Box& nb, const int e[3], const Box& kb, uint8_t qlo[3],
                     uint8_t qhi[3]) {
  for (int a = 0; a < 3; a++) {
    double lo = nb.lo[a], scale = std::ldexp(1.0, e[a]);
    double ql = std::floor(((double)kb.lo[a] - lo) / scale) - 1;
    double qh = std::ceil(((double)kb.hi[a] - lo) / scale) + 1;
    ql = std::max(0.0, std::min(255.0, ql));
    qh = std::max(0.0, std::min(255.0, qh));
    if (lo + ql * scale > (double)kb.lo[a] || lo + qh * scale < (double)kb.hi[a]) return false;
    qlo[a] = (uint8_t)ql;
    qhi[a] = (uint8_t)qh;
  }
  return true;
}

static bool emit_compact(const Builder& B, int64_t bnode, BvhBuildOutput& out) {
  const size_t me = out.nodesC.size() / 8;
  out.nodesC.resize(out.nodesC.size() + 8, 0u);
  const BNode& nd = B.nodes[bnode];
  int64_t c[2] = {nd.left, nd.right};
  bool leaf[2] = {B.nodes[c[0]].count > 0, B.nodes[c[1]].count > 0};
  if (!leaf[0] && leaf[1]) {  // a leaf child goes first
    std::swap(c[0], c[1]);
    std::swap(leaf[0], leaf[1]);
  }
  auto add_leaf = [&](const BNode& k) {
    for (int64_t i = 0; i < k.count; i++) {
      out.slot_primC.push_back(B.refs[k.begin + i]);
      out.slot_lastC.push_back(i + 1 == k.count ? 1 : 0);
    }
  };
  uint32_t meta = (leaf[0] ? 1u : 0u) | (leaf[1] ? 2u : 0u);
  uint32_t w7 = 0;
  if (leaf[0]) {
    const BNode& k0 = B.nodes[c[0]];
    if (k0.count > 63) return false;
    meta |= (uint32_t)k0.count << 2;
    w7 = (uint32_t)out.slot_primC.size();
    add_leaf(k0);
    if (leaf[1]) add_leaf(B.nodes[c[1]]);
  }
  // the node frame: origin = the node's box minimum, 255 quanta cover the extent
  const Box& nb = nd.box;
  int e[3];
  uint32_t ebits = 0;
  for (int a = 0; a < 3; a++) {
    double ext = (double)nb.hi[a] - nb.lo[a];
    int ea = -100;
    if (ext > 0) {
      ea = (int)std::ceil(std::log2(ext * (1.0 + 1.0 / 1024.0) / 255.0));
      while (std::ldexp(255.0, ea) < ext * (1.0 + 1.0 / 1024.0)) ea++;
    }
    e[a] = std::max(-126, std::min(127, ea));
    ebits |= (uint32_t)(e[a] + 127) << (8 * a);
  }
  uint8_t q[12];
  for (int k = 0; k < 2; k++)
    if (!quantise(nb, e, B.nodes[c[k]].box, &q[6 * k], &q[6 * k + 3])) return false;
  {
    uint32_t* w = &out.nodesC[8 * me];
    memcpy(&w[0], nb.lo, 12);
    w[3] = ebits | (meta << 24);
    memcpy(&w[4], q, 12);
  }
  if (!leaf[0]) {  // both inner: child 0 next, child 1 after child 0's subtree
    if (!emit_compact(B, c[0], out)) return false;
    w7 = (uint32_t)(out.nodesC.size() / 8);
    if (!emit_compact(B, c[1], out)) return false;
  } else if (!leaf[1]) {  // leaf child 0, inner child 1 next
    if (!emit_compact(B, c[1], out)) return false;
  }
  out.nodesC[8 * me + 7] = w7;
  return true;
}

static bool build_compact(const Builder& B, BvhBuildOutput& out) {
  out.nodesC.clear();
  out.slot_primC.clear();
  out.slot_lastC.clear();
  const BNode& root = B.nodes[0];
  if (root.count > 0) {
    out.rootC = ~(int32_t)0;
    for (int64_t i = 0; i < root.count; i++) {
      out.slot_primC.push_back(B.refs[root.begin + i]);
      out.slot_lastC.push_back(i + 1 == root.count ? 1 : 0);
    }
    return true;
  }
  out.rootC = 0;
  return emit_compact(B, 0, out);
}

}  // namespace

int build_bvh(const BvhBuildInput& in, BvhBuildOutput& out) {
  if (in.n <= 0 || !in.lo || !in.hi || in.n >= (int64_t(1) << 27)) return -1;
  Builder B(in);
  B.build(0, 0, in.n, 0);
  out.max_depth = B.max_depth.load();
  if (out.max_depth >= kBvhMaxDepth) return -1;
  if (!in.wide || !build_wide(B, out)) {
    out.nodes8.clear();
    out.slot_prim8.clear();
    out.slot_last8.clear();
    out.wide_depth = -1;  // the wide layout is not available for this tree
  }
  out.compact_ok = in.compact && build_compact(B, out);
  if (!out.compact_ok) {
    out.nodesC.clear();
    out.slot_primC.clear();
    out.slot_lastC.clear();
  }
  out.nodes.clear();
  out.slot_prim.clear();
  out.slot_last.clear();
  out.leaves = 0;
  // depth-first flatten; leaves become slot ranges referenced by their parent
  auto leaf_ref = [&](const BNode& nd) {
    int32_t first = (int32_t)out.slot_prim.size();
    for (int64_t k = 0; k < nd.count; k++) {
      out.slot_prim.push_back(B.refs[nd.begin + k]);
      out.slot_last.push_back(k + 1 == nd.count ? 1 : 0);
    }
    out.leaves++;
    return ~first;
  };
  const BNode& root = B.nodes[0];
  if (root.count > 0) {
    out.root_ref = leaf_ref(root);
    return 0;
  }
  out.root_ref = 0;
  struct Item {
    int64_t bnode;
    int64_t out_index;
  };
  std::vector<Item> stack;
  out.nodes.resize(16);
  stack.push_back(Item{0, 0});
  while (!stack.empty()) {
    Item it = stack.back();
    stack.pop_back();
    const BNode& nd = B.nodes[it.bnode];
    int32_t refs[2];
    const BNode* ch[2] = {&B.nodes[nd.left], &B.nodes[nd.right]};
    int64_t pending[2] = {-1, -1};
    for (int c = 0; c < 2; c++) {
      if (ch[c]->count > 0) {
        refs[c] = leaf_ref(*ch[c]);
      } else {
        int64_t oi = (int64_t)out.nodes.size() / 16;
        out.nodes.resize(out.nodes.size() + 16);
        refs[c] = (int32_t)oi;
        pending[c] = oi;
      }
    }
    float* o = &out.nodes[16 * it.out_index];
    const Box& b0 = ch[0]->box;
    const Box& b1 = ch[1]->box;
    o[0] = b0.lo[0];
    o[1] = b0.hi[0];
    o[2] = b0.lo[1];
    o[3] = b0.hi[1];
    o[4] = b1.lo[0];
    o[5] = b1.hi[0];
    o[6] = b1.lo[1];
    o[7] = b1.hi[1];
    o[8] = b0.lo[2];
    o[9] = b0.hi[2];
    o[10] = b1.lo[2];
    o[11] = b1.hi[2];
    memcpy(&o[12], &refs[0], 4);
    memcpy(&o[13], &refs[1], 4);
    o[14] = 0;
    o[15] = 0;
    // siblings are allocated together, so both children of a node are adjacent
    if (pending[1] >= 0) stack.push_back(Item{nd.right, pending[1]});
    if (pending[0] >= 0) stack.push_back(Item{nd.left, pending[0]});
  }
  return 0;
}

namespace {

struct DBox {
  double lo[3], hi[3];
  void reset() {
    for (int k = 0; k < 3; k++) {
      lo[k] = INFINITY;
      hi[k] = -INFINITY;
    }
  }
  void grow(const DBox& b) {
    for (int k = 0; k < 3; k++) {
      lo[k] = std::min(lo[k], b.lo[k]);
      hi[k] = std::max(hi[k], b.hi[k]);
    }
  }
  bool contains(const DBox& b) const {
    for (int k = 0; k < 3; k++)
      if (b.lo[k] < lo[k] || b.hi[k] > hi[k]) return false;
    return true;
  }
};

struct Validator {
  const BvhBuildInput& in;
  const std::vector<int32_t>& slot_prim;
  const std::vector<uint8_t>& slot_last;
  std::vector<int> prim_seen;
  std::vector<int> slot_seen;
  int err = 0;

  Validator(const BvhBuildInput& i, const std::vector<int32_t>& sp, const std::vector<uint8_t>& sl)
      : in(i), slot_prim(sp), slot_last(sl), prim_seen(i.n, 0), slot_seen(sp.size(), 0) {}

  DBox leaf(int32_t ref) {
    DBox b;
    b.reset();
    int64_t s = ~(int64_t)ref;
    for (;;) {
      if (s < 0 || s >= (int64_t)slot_prim.size()) {
        err = -10;
        return b;
      }
      if (slot_seen[s]++) err = -11;
      int32_t p = slot_prim[s];
      if (p < 0 || p >= in.n) {
        err = -12;
        return b;
      }
      prim_seen[p]++;
      DBox pb;
      for (int k = 0; k < 3; k++) {
        pb.lo[k] = in.lo[3 * p + k];
        pb.hi[k] = in.hi[3 * p + k];
      }
      b.grow(pb);
      if (slot_last[s]) break;
      s++;
    }
    return b;
  }

  int finish() {
    if (err) return err;
    for (int v : prim_seen)
      if (v != 1) return -13;
    for (int v : slot_seen)
      if (v != 1) return -14;
    return 0;
  }
};

DBox validate_binary(Validator& V, const BvhBuildOutput& out, int32_t ref, int depth) {
  if (ref < 0) return V.leaf(ref);
  DBox un;
  un.reset();
  if (depth > kBvhMaxDepth || (int64_t)ref * 16 + 16 > (int64_t)out.nodes.size()) {
    V.err = -20;
    return un;
  }
  const float* o = &out.nodes[16 * (size_t)ref];
  int32_t refs[2];
  memcpy(&refs[0], &o[12], 4);
  memcpy(&refs[1], &o[13], 4);
  for (int c = 0; c < 2; c++) {
    DBox cb = validate_binary(V, out, refs[c], depth + 1);
    DBox stored;
    const int xo = c ? 4 : 0, zo = c ? 10 : 8;
    stored.lo[0] = o[xo];
    stored.hi[0] = o[xo + 1];
    stored.lo[1] = o[xo + 2];
    stored.hi[1] = o[xo + 3];
    stored.lo[2] = o[zo];
    stored.hi[2] = o[zo + 1];
    if (!stored.contains(cb)) V.err = -21;
    un.grow(cb);
  }
  return un;
}

DBox validate_wide(Validator& V, const BvhBuildOutput& out, int32_t ref, int depth) {
  if (ref < 0) return V.leaf(ref);
  DBox un;
  un.reset();
  size_t n_nodes = out.nodes8.size() / 20;
  if (depth > out.wide_depth || (size_t)ref >= n_nodes) {
    V.err = -30;
    return un;
  }
  const uint32_t* w = &out.nodes8[20 * (size_t)ref];
  float p[3];
  memcpy(p, w, 12);
  uint8_t meta[8], q[6][8];
  memcpy(meta, &w[6], 8);
  for (int r = 0; r < 6; r++) memcpy(q[r], &w[8 + 2 * r], 8);
  int internal = 0;
  for (int s = 0; s < 8; s++)
    if (meta[s] != 0xFF && (meta[s] & 0x80)) internal++;
  for (int s = 0; s < 8; s++) {
    if (meta[s] == 0xFF) continue;
    int32_t cref;
    if (meta[s] & 0x80) {
      int rank = meta[s] & 0x7f;
      if (rank >= internal) {
        V.err = -31;
        return un;
      }
      cref = (int32_t)(w[4] + rank);
    } else {
      cref = ~(int32_t)(w[5] + meta[s]);
    }
    DBox cb = validate_wide(V, out, cref, depth + 1);
    DBox dec;
    for (int a = 0; a < 3; a++) {
      double scale = std::ldexp(1.0, (int)((w[3] >> (8 * a)) & 0xff) - 127);
      dec.lo[a] = (double)p[a] + q[a][s] * scale;
      dec.hi[a] = (double)p[a] + q[3 + a][s] * scale;
    }
    if (!dec.contains(cb)) V.err = -32;
    un.grow(cb);
  }
  return un;
}

DBox validate_compact(Validator& V, const BvhBuildOutput& out, int32_t ref, int depth) {
  if (ref < 0) return V.leaf(ref);
  DBox un;
  un.reset();
  size_t n_nodes = out.nodesC.size() / 8;
  if (depth > kBvhMaxDepth || (size_t)ref >= n_nodes) {
    V.err = -40;
    return un;
  }
  const uint32_t* w = &out.nodesC[8 * (size_t)ref];
  float p[3];
  memcpy(p, w, 12);
  uint8_t q[12];
  memcpy(q, &w[4], 12);
  uint32_t meta = w[3] >> 24;
  bool l0 = meta & 1u, l1 = meta & 2u;
  if (!l0 && l1) {
    V.err = -41;  // a leaf child must come first
    return un;
  }
  int32_t refs[2];
  refs[0] = l0 ? ~(int32_t)w[7] : ref + 1;
  refs[1] = l1 ? ~(int32_t)(w[7] + (meta >> 2)) : (l0 ? ref + 1 : (int32_t)w[7]);
  for (int c = 0; c < 2; c++) {
    DBox cb = validate_compact(V, out, refs[c], depth + 1);
    DBox dec;
    for (int a = 0; a < 3; a++) {
      double scale = std::ldexp(1.0, (int)((w[3] >> (8 * a)) & 0xff) - 127);
      dec.lo[a] = (double)p[a] + q[6 * c + a] * scale;
      dec.hi[a] = (double)p[a] + q[6 * c + 3 + a] * scale;
    }
    if (!dec.contains(cb)) V.err = -42;
    un.grow(cb);
  }
  return un;
}

}  // namespace

int validate_bvh(const BvhBuildInput& in, const BvhBuildOutput& out) {
  {
    Validator V(in, out.slot_prim, out.slot_last);
    validate_binary(V, out, out.root_ref, 0);
    int rc = V.finish();
    if (rc) return rc;
  }
  if (out.wide_depth >= 0 && !out.nodes8.empty()) {
    Validator V(in, out.slot_prim8, out.slot_last8);
    validate_wide(V, out, out.root8, 1);
    int rc = V.finish();
    if (rc) return rc - 100;
  } else if (out.wide_depth >= 0 && out.root8 < 0) {
    Validator V(in, out.slot_prim8, out.slot_last8);
    V.leaf(out.root8);
    int rc = V.finish();
    if (rc) return rc - 100;
  }
  if (out.compact_ok) {
    Validator V(in, out.slot_primC, out.slot_lastC);
    validate_compact(V, out, out.rootC, 0);
    int rc = V.finish();
    if (rc) return rc - 200;
  }
  return 0;
}

}  // namespace bgpu
