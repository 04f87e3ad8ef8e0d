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

}  // namespace

int build_bvh(const BvhBuildInput& in, BvhBuildOutput& out) {
  if (in.n <= 0 || !in.lo || !in.hi || in.n >= (int64_t(1) << 27)) return -1;
  Builder B(in);
  B.build(0, 0, in.n, 0);
  out.max_depth = B.max_depth.load();
  if (out.max_depth >= kBvhMaxDepth) return -1;
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

}  // namespace bgpu
