// BVH traversal on the device: closest hit and any hit.
//
// Replaces the reference's kd-tree walk `traverse`/`traverse'` with the leaf
// fold `nearest'` (Primitive/KdTree.hs:210-246, Primitive.hs:29-43).  The
// answer is the reference's: the primitive with the smallest hit distance in
// [tmin, tmax] computed with the reference's own intersection arithmetic, and
// among equal distances the one with the larger primitive ID (a later
// primitive with an equal t replaces the earlier one in the fold, because the
// intersection tests reject only t > tmax, TriangleMesh.hs:146,166).
//
// Box tests are conservative: the slab distances carry a relative error of a
// few ulp, and every box interval is widened by a relative 2^-16 so that a
// primitive whose reference-arithmetic t lies on a box face is never pruned
// (the quantised wide layout also widens each child box by one quantum).
#pragma once
#include <type_traits>

#include "bvh.h"
#include "dmath.cuh"
#include "dshape.cuh"
#include "internal.h"

namespace bgpu {

constexpr int kTraversalStack = 64;  // binary layout: depth < kBvhMaxDepth
constexpr int kMaxTraceBlock = 128;  // threads per block of every traversal launch
constexpr float kBoxSlack = 1.0f / 65536.0f;

// triangleIntersect / triangleIntersects (TriangleMesh.hs:140-181) on a
// pre-gathered slot (p1, e1, e2)
__device__ __forceinline__ bool triTest(const float4 s0, const float4 s1, const float4 s2,
                                        const Ray& r, float tmax, float& t, float& b1o,
                                        float& b2o) {
  V3 p1{s0.x, s0.y, s0.z}, e1{s0.w, s1.x, s1.y}, e2{s1.z, s1.w, s2.x};
  V3 s1v = cross(r.d, e2);
  float divisor = dot(s1v, e1);
  if (divisor == 0) return false;
  float invDiv = 1.0f / divisor;
  V3 d = r.o - p1;
  float b1 = dot(d, s1v) * invDiv;
  if (b1 < 0 || b1 > 1) return false;
  V3 s2v = cross(d, e1);
  float b2 = dot(r.d, s2v) * invDiv;
  if (b2 < 0 || b1 + b2 > 1) return false;
  float tt = dot(e2, s2v) * invDiv;
  if (tt < r.tmin || tt > tmax) return false;
  t = tt;
  b1o = b1;
  b2o = b2;
  return true;
}

// min/max that return NaN when either operand is NaN (PTX min.NaN/max.NaN)
__device__ __forceinline__ float fminNaN(float a, float b) {
  float r;
  asm("min.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}
__device__ __forceinline__ float fmaxNaN(float a, float b) {
  float r;
  asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
  return r;
}

// Widens a box's entry/exit distances by kBoxSlack (relative).  An infinite
// bound stays infinite: n - |n| * s alone would turn +inf into inf - inf =
// NaN and let a missed box pass.
__device__ __forceinline__ float widenNear(float n) { return fminf(n, fmaf(-fabsf(n), kBoxSlack, n)); }
__device__ __forceinline__ float widenFar(float f) { return fmaxf(f, fmaf(fabsf(f), kBoxSlack, f)); }

// three-operand forms (sm_100 and later): one instruction for a box's entry
// or exit over its three slabs
__device__ __forceinline__ float fmax3NaN(float a, float b, float c) {
  float r;
  asm("max.NaN.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}
__device__ __forceinline__ float fmin3NaN(float a, float b, float c) {
  float r;
  asm("min.NaN.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
  return r;
}

// Slab interval of a box.  A ray with a zero direction component (inv = +-inf)
// is inside that slab for all t when the origin lies strictly between its
// planes (-inf, +inf), outside for all t when it lies beyond them (+-inf on
// both planes).  An origin exactly on a plane gives 0 * inf = NaN: the
// NaN-propagating min/max carry it into the box's interval, and the hit test
// below (fmaxf/fminf drop NaN) then counts the box as hit, which keeps the
// traversal conservative for rays that run along a box face.
__device__ __forceinline__ void boxInterval(float lox, float hix, float loy, float hiy, float loz,
                                            float hiz, const V3& o, const V3& inv, float& tn,
                                            float& tf) {
  float x0 = (lox - o.x) * inv.x, x1 = (hix - o.x) * inv.x;
  float y0 = (loy - o.y) * inv.y, y1 = (hiy - o.y) * inv.y;
  float z0 = (loz - o.z) * inv.z, z1 = (hiz - o.z) * inv.z;
  float n = fmax3NaN(fminNaN(x0, x1), fminNaN(y0, y1), fminNaN(z0, z1));
  float f = fmin3NaN(fmaxNaN(x0, x1), fmaxNaN(y0, y1), fmaxNaN(z0, z1));
  tn = widenNear(n);
  tf = widenFar(f);
}

// work counters of a traversal (the instrumented variant only; the
// reference's dbgTraverse counts the same things, Primitive/KdTree.hs:252-281)
struct TraversalCounts {
  unsigned nodes;  // inner nodes visited (64-byte binary or 80-byte wide node reads)
  unsigned slots;  // leaf slots tested (48-byte primitive reads)
};

struct RayQueryResult {
  bool hit;
  float t, b1, b2;
  int prim;
};

// A ray with a NaN component makes every slab test pass (fminf/fmaxf drop
// NaN), so its walk would visit the whole tree; the reference's kd-tree walk
// does the same (`tp > tmax || tp <= 0` and `tp < tmin` are all False for NaN,
// KdTree.hs:212-215) and its NaN-distance "hit" ends in a sample that addSample
// drops (Image.hs:253-256).  Such rays are answered without traversal:
// occluded for any-hit queries (triangleIntersects is True for NaN), and the
// degenerate primitive ID kDegenerateRay for closest-hit queries.
constexpr int kDegenerateRay = -2;

__device__ __forceinline__ bool degenerateRay(const Ray& r) {
  return isnan(r.o.x) || isnan(r.o.y) || isnan(r.o.z) || isnan(r.d.x) || isnan(r.d.y) ||
         isnan(r.d.z) || isnan(r.tmin) || isnan(r.tmax);
}

// 32 bytes of read-only global memory, 32-byte aligned, in one 256-bit load
// (ld.global.nc.v8, sm_100 and later): half the load instructions of four
// 16-byte loads for a 64-byte node
__device__ __forceinline__ void ldg256(const float4* p, float4& a, float4& b) {
  asm("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
      : "=f"(a.x), "=f"(a.y), "=f"(a.z), "=f"(a.w), "=f"(b.x), "=f"(b.y), "=f"(b.z), "=f"(b.w)
      : "l"(p));
}

// u8 -> float without a conversion instruction: 0x4B0000bb is 2^23 + bb
__device__ __forceinline__ float qbyte(uint32_t word, uint32_t sel) {
  return __uint_as_float(__byte_perm(word, 0x4B000000u, sel)) - 8388608.0f;
}

// ---------------------------------------------------------------------------
// Warp-synchronous persistent traversal.
//  * every warp loops over rays it fetches itself: lanes whose ray finished
//    take the next rays from a global counter (one atomicAdd per warp,
//    __ballot_sync/__popc to rank the lanes), so lanes never idle while rays
//    remain;
//  * each round runs a node phase and a leaf phase for the whole warp (the
//    "while-while" order): in the node phase a lane that meets a leaf
//    postpones it and keeps walking inner nodes until every lane holds a leaf
//    or has finished, then the warp tests leaves together.
// WIDE selects the 8-wide quantised layout (bvh.h): each visit tests eight
// child boxes and pushes the hit ones in the octant order of the ray, so the
// nearest is taken next.  All votes use the full warp mask: every lane runs
// every iteration of the uniform loops and does work only when it has some.
// With an `accel_of` functor (ray index -> const DevAccel*) every lane walks
// the scene of its own ray (batches of jobs over several scenes, which must
// share the node layout); otherwise all rays walk A.
// MIXED (any-hit walks only): `load(q, by_intersect, rank_prim)` also says,
// per ray, which predicate answers an analytic shape: Shape.intersects
// (false, the occlusion test) or Shape.intersect (true: whether a closest-hit
// query would find a hit).  The two differ, e.g. a box does not `intersect` a
// ray that starts inside it, while it `intersects` it.  Triangles answer both
// alike.  With rank_prim >= 0 a hit counts only if a closest-hit query would
// rank it before a hit of primitive rank_prim at tmax: at t < tmax, or at
// tmax with a larger primitive ID (the tie rule of the closest-hit walk).
constexpr int kSentinel = INT32_MIN;

template <bool ANY, int LAYOUT, bool COUNT, bool MIXED = false, class LoadRay, class Emit,
          class AccelOf = std::nullptr_t>
__device__ __forceinline__ void traceWarpPersistent(const DevAccel& A, int64_t n,
                                                    unsigned long long* __restrict__ next_ray,
                                                    LoadRay load, Emit emit,
                                                    TraversalCounts* cnt = nullptr,
                                                    AccelOf accel_of = nullptr) {
  constexpr bool PER_LANE = !std::is_same<AccelOf, std::nullptr_t>::value;
  constexpr bool WIDE = LAYOUT == LAYOUT_WIDE;
  constexpr bool COMPACT = LAYOUT == LAYOUT_COMPACT;
  const float4* l_nodes = nullptr;
  const float4* l_nodesC = nullptr;
  const uint4* l_nodes8 = nullptr;
  const float4* l_slots = nullptr;
  const DShape* l_shapes = nullptr;
#define TW_ACC(field) (PER_LANE ? l_##field : A.field)
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned lt_mask = (1u << lane) - 1u;
  constexpr int kStack = WIDE ? kWideStack : kTraversalStack;
  int64_t rid = -1;
  bool exhausted = false;
  bool by_intersect = false;  // MIXED: this ray's shapes answer by Shape.intersect
  int rank_prim = -1;         // MIXED: hits must rank before this primitive's at tmax
  Ray r;
  V3 inv;
  int oct = 0;
  int zmask = 0;  // axes whose direction component is zero (inv = +-inf)
  float best_t = 0, bb1 = 0, bb2 = 0;
  int best_prim = -1;
  // The top kSharedStack entries of each lane's stack live in shared memory
  // (one column per thread, so the lanes of a warp hit distinct banks);
  // deeper entries go to a local array.  Pushes and pops then skip the L1
  // tag stage that local memory goes through (16M closest-hit rays on the
  // 1M soup: 14.2 -> 12.7 ms).  Blocks have at most kMaxTraceBlock threads
  // (every launch of this walk: 128, or 64/128 for batches).
  constexpr int kSharedStack = 24;
  __shared__ int s_stack[kSharedStack * kMaxTraceBlock];
  int* my_stack = s_stack + threadIdx.x;
  int stack[kStack - kSharedStack];
  int sp = 0;
  auto push = [&](int ref) {
    if (sp < kSharedStack)
      my_stack[sp * kMaxTraceBlock] = ref;
    else
      stack[sp - kSharedStack] = ref;
    sp++;
  };
  auto pop = [&]() -> int {
    if (sp == 0) return kSentinel;
    sp--;
    return sp < kSharedStack ? my_stack[sp * kMaxTraceBlock] : stack[sp - kSharedStack];
  };
  int cur = kSentinel;
  int leaf = kSentinel;  // postponed leaf
  for (;;) {
    // ---- refill lanes that have no ray
    bool need = rid < 0 && !exhausted;
    unsigned m = __ballot_sync(FULL, need);
    if (m) {
      int leader = __ffs(m) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(next_ray, (unsigned long long)__popc(m));
      base = __shfl_sync(FULL, base, leader);
      if (need) {
        unsigned long long my = base + (unsigned long long)__popc(m & lt_mask);
        if ((int64_t)my < n) {
          rid = (int64_t)my;
          if constexpr (MIXED)
            r = load(rid, by_intersect, rank_prim);
          else
            r = load(rid);
          if (degenerateRay(r)) {
            emit(rid, RayQueryResult{true, NAN, 0.0f, 0.0f, kDegenerateRay});
            rid = -1;  // take another ray next round
          } else {
            inv = V3{1.0f / r.d.x, 1.0f / r.d.y, 1.0f / r.d.z};
            oct = (signbit(inv.x) ? 1 : 0) | (signbit(inv.y) ? 2 : 0) | (signbit(inv.z) ? 4 : 0);
            zmask = (isinf(inv.x) ? 1 : 0) | (isinf(inv.y) ? 2 : 0) | (isinf(inv.z) ? 4 : 0);
            best_t = r.tmax;
            best_prim = -1;
            bb1 = bb2 = 0.0f;
            sp = 0;
            if constexpr (PER_LANE) {
              const DevAccel* la = accel_of(rid);
              l_nodes = la->nodes;
              l_nodesC = la->nodesC;
              l_nodes8 = la->nodes8;
              l_slots = la->slots;
              l_shapes = la->shapes;
              cur = WIDE ? la->root8 : (COMPACT ? la->rootC : la->root_ref);
            } else {
              cur = WIDE ? A.root8 : (COMPACT ? A.rootC : A.root_ref);
            }
            leaf = kSentinel;
          }
        } else {
          exhausted = true;
        }
      }
    }
    if (!__any_sync(FULL, rid >= 0 || !exhausted)) return;
    // ---- node phase
    // the vote at the end of a step implies this one for the next step
    bool go = __any_sync(FULL, rid >= 0 && cur >= 0);
    while (go) {
      // COUNT walks in plain depth-first order: a lane stops at its first
      // leaf, which the leaf phase tests before any further node is visited
      bool work = rid >= 0 && cur >= 0 && (!COUNT || leaf == kSentinel);
      if (work) {
        if (COUNT) cnt->nodes++;
        if (WIDE) {
          const uint4* nd = TW_ACC(nodes8) + 5 * (size_t)cur;
          uint4 w0 = __ldg(nd), w1 = __ldg(nd + 1), w2 = __ldg(nd + 2), w3 = __ldg(nd + 3),
                w4 = __ldg(nd + 4);
          // child box slab distances: t = q * (scale / d) + (p - o) / d
          float sx = __uint_as_float((w0.w & 0xffu) << 23) * inv.x;
          float sy = __uint_as_float(((w0.w >> 8) & 0xffu) << 23) * inv.y;
          float sz = __uint_as_float(((w0.w >> 16) & 0xffu) << 23) * inv.z;
          float bx = (__uint_as_float(w0.x) - r.o.x) * inv.x;
          float by = (__uint_as_float(w0.y) - r.o.y) * inv.y;
          float bz = (__uint_as_float(w0.z) - r.o.z) * inv.z;
          // near/far planes by the direction's sign
          uint32_t nx0 = (oct & 1) ? w3.z : w2.x, nx1 = (oct & 1) ? w3.w : w2.y;
          uint32_t fx0 = (oct & 1) ? w2.x : w3.z, fx1 = (oct & 1) ? w2.y : w3.w;
          uint32_t ny0 = (oct & 2) ? w4.x : w2.z, ny1 = (oct & 2) ? w4.y : w2.w;
          uint32_t fy0 = (oct & 2) ? w2.z : w4.x, fy1 = (oct & 2) ? w2.w : w4.y;
          uint32_t nz0 = (oct & 4) ? w4.z : w3.x, nz1 = (oct & 4) ? w4.w : w3.y;
          uint32_t fz0 = (oct & 4) ? w3.x : w4.z, fz1 = (oct & 4) ? w3.y : w4.w;
          uint32_t hits = 0;
#pragma unroll
          for (int i = 0; i < 8; i++) {
            const uint32_t sel = 0x7650u | (uint32_t)(i & 3);
            float tnx = fmaf(qbyte(i < 4 ? nx0 : nx1, sel), sx, bx);
            float tny = fmaf(qbyte(i < 4 ? ny0 : ny1, sel), sy, by);
            float tnz = fmaf(qbyte(i < 4 ? nz0 : nz1, sel), sz, bz);
            float tfx = fmaf(qbyte(i < 4 ? fx0 : fx1, sel), sx, bx);
            float tfy = fmaf(qbyte(i < 4 ? fy0 : fy1, sel), sy, by);
            float tfz = fmaf(qbyte(i < 4 ? fz0 : fz1, sel), sz, bz);
            // one plane per axis and side, so a NaN (0 * inf: a zero
            // direction component) is dropped across axes, which ignores
            // that axis: conservative
            float tn = widenNear(fmaxf(fmaxf(tnx, tny), tnz));
            float tf = widenFar(fminf(fminf(tfx, tfy), tfz));
            uint32_t meta = ((i < 4 ? w1.z : w1.w) >> (8 * (i & 3))) & 0xffu;
            bool h = meta != 0xffu && fmaxf(tn, r.tmin) <= fminf(tf, best_t);
            hits |= (h ? 1u : 0u) << i;
          }
          // push all hit children but the nearest, far ones first
          int first = kSentinel;
#pragma unroll
          for (int k = 7; k >= 0; k--) {
            int slot = k ^ oct;
            if (hits >> slot & 1u) {
              uint32_t meta = ((slot < 4 ? w1.z : w1.w) >> (8 * (slot & 3))) & 0xffu;
              int ref = (meta & 0x80u) ? (int)(w1.x + (meta & 0x7fu)) : ~(int)(w1.y + meta);
              if (first != kSentinel) push(first);
              first = ref;
            }
          }
          cur = first != kSentinel ? first : pop();
        } else if (COMPACT) {
          // 32-byte quantised node (bvh.h): child box slab distances
          // t = q * (scale / d) + (p - o) / d, as the 8-wide layout
          float4 a, b;
          ldg256(TW_ACC(nodesC) + 2 * (size_t)cur, a, b);
          const uint32_t w3 = __float_as_uint(a.w);
          const float sx = __uint_as_float((w3 & 0xffu) << 23) * inv.x;
          const float sy = __uint_as_float(((w3 >> 8) & 0xffu) << 23) * inv.y;
          const float sz = __uint_as_float(((w3 >> 16) & 0xffu) << 23) * inv.z;
          const float bx = (a.x - r.o.x) * inv.x;
          const float by = (a.y - r.o.y) * inv.y;
          const float bz = (a.z - r.o.z) * inv.z;
          // q bytes: c0 lo.xyz hi.xyz in b.x (4) and b.y (2), c1 in b.y (2) and b.z (4)
          const uint32_t q0 = __float_as_uint(b.x), q1 = __float_as_uint(b.y),
                         q2 = __float_as_uint(b.z);
          const float c0lx = qbyte(q0, 0x7650u), c0ly = qbyte(q0, 0x7651u),
                      c0lz = qbyte(q0, 0x7652u), c0hx = qbyte(q0, 0x7653u),
                      c0hy = qbyte(q1, 0x7650u), c0hz = qbyte(q1, 0x7651u),
                      c1lx = qbyte(q1, 0x7652u), c1ly = qbyte(q1, 0x7653u),
                      c1lz = qbyte(q2, 0x7650u), c1hx = qbyte(q2, 0x7651u),
                      c1hy = qbyte(q2, 0x7652u), c1hz = qbyte(q2, 0x7653u);
          const bool nxh = oct & 1, nyh = oct & 2, nzh = oct & 4;  // near plane is hi
          // per axis: near and far distance of child 0 and child 1
          float nx0 = fmaf(nxh ? c0hx : c0lx, sx, bx), fx0 = fmaf(nxh ? c0lx : c0hx, sx, bx);
          float ny0 = fmaf(nyh ? c0hy : c0ly, sy, by), fy0 = fmaf(nyh ? c0ly : c0hy, sy, by);
          float nz0 = fmaf(nzh ? c0hz : c0lz, sz, bz), fz0 = fmaf(nzh ? c0lz : c0hz, sz, bz);
          float nx1 = fmaf(nxh ? c1hx : c1lx, sx, bx), fx1 = fmaf(nxh ? c1lx : c1hx, sx, bx);
          float ny1 = fmaf(nyh ? c1hy : c1ly, sy, by), fy1 = fmaf(nyh ? c1ly : c1hy, sy, by);
          float nz1 = fmaf(nzh ? c1hz : c1lz, sz, bz), fz1 = fmaf(nzh ? c1lz : c1hz, sz, bz);
          if (zmask) {
            // a zero direction component (inv = +-inf) makes those distances
            // 0 * inf or inf - inf: decide that slab by the origin instead,
            // inside when it lies between the child's decoded planes (rounded
            // outward), for all t; outside for none
            auto slab = [&](float ql, float qh, float e_bits, float p, float o, float& n,
                            float& f) {
              bool in = __fmaf_rd(ql, e_bits, p) <= o && o <= __fmaf_ru(qh, e_bits, p);
              n = in ? -INFINITY : INFINITY;
              f = in ? INFINITY : -INFINITY;
            };
            if (zmask & 1) {
              const float e = __uint_as_float((w3 & 0xffu) << 23);
              slab(c0lx, c0hx, e, a.x, r.o.x, nx0, fx0);
              slab(c1lx, c1hx, e, a.x, r.o.x, nx1, fx1);
            }
            if (zmask & 2) {
              const float e = __uint_as_float(((w3 >> 8) & 0xffu) << 23);
              slab(c0ly, c0hy, e, a.y, r.o.y, ny0, fy0);
              slab(c1ly, c1hy, e, a.y, r.o.y, ny1, fy1);
            }
            if (zmask & 4) {
              const float e = __uint_as_float(((w3 >> 16) & 0xffu) << 23);
              slab(c0lz, c0hz, e, a.z, r.o.z, nz0, fz0);
              slab(c1lz, c1hz, e, a.z, r.o.z, nz1, fz1);
            }
          }
          float n0 = widenNear(fmaxf(fmaxf(nx0, ny0), nz0));
          float f0 = widenFar(fminf(fminf(fx0, fy0), fz0));
          float n1 = widenNear(fmaxf(fmaxf(nx1, ny1), nz1));
          float f1 = widenFar(fminf(fminf(fx1, fy1), fz1));
          bool h0 = fmaxf(n0, r.tmin) <= fminf(f0, best_t);
          bool h1 = fmaxf(n1, r.tmin) <= fminf(f1, best_t);
          const uint32_t meta = w3 >> 24, w7 = __float_as_uint(b.w);
          const bool l0 = meta & 1u, l1 = meta & 2u;
          int r0 = l0 ? ~(int)w7 : cur + 1;
          int r1 = l1 ? ~(int)(w7 + (meta >> 2)) : (l0 ? cur + 1 : (int)w7);
          if (h0 && h1) {
            bool swap = n1 < n0;
            cur = swap ? r1 : r0;
            push(swap ? r0 : r1);
          } else if (h0 || h1) {
            cur = h0 ? r0 : r1;
          } else {
            cur = pop();
          }
        } else {
          const float4* nd = TW_ACC(nodes) + 4 * (size_t)cur;  // 64-byte aligned
          float4 a, b, c, refs;
          ldg256(nd, a, b);
          ldg256(nd + 2, c, refs);
          float n0, f0, n1, f1;
          boxInterval(a.x, a.y, a.z, a.w, c.x, c.y, r.o, inv, n0, f0);
          boxInterval(b.x, b.y, b.z, b.w, c.z, c.w, r.o, inv, n1, f1);
          bool h0 = fmaxf(n0, r.tmin) <= fminf(f0, best_t);
          bool h1 = fmaxf(n1, r.tmin) <= fminf(f1, best_t);
          int r0 = __float_as_int(refs.x), r1 = __float_as_int(refs.y);
          if (h0 && h1) {
            bool swap = n1 < n0;
            cur = swap ? r1 : r0;
            push(swap ? r0 : r1);
          } else if (h0 || h1) {
            cur = h0 ? r0 : r1;
          } else {
            cur = pop();
          }
        }
        // postpone the first leaf met; keep walking inner nodes
        if (cur < 0 && cur != kSentinel && leaf == kSentinel) {
          leaf = cur;
          cur = pop();
        }
      }
      // leave the node phase once no lane both lacks a leaf and has nodes to visit
      go = __any_sync(FULL, rid >= 0 && leaf == kSentinel && cur >= 0);
    }
    // ---- leaf phase
    for (;;) {
      bool work = rid >= 0 && (leaf != kSentinel || (cur < 0 && cur != kSentinel));
      if (!__any_sync(FULL, work)) break;
      if (work) {
        if (leaf == kSentinel) {
          leaf = cur;
          cur = pop();
        }
        int slot = ~leaf;
        leaf = kSentinel;
        for (;;) {
          if (COUNT) cnt->slots++;
          const float4* sl = TW_ACC(slots) + 3 * (size_t)slot;
          float4 s0 = __ldg(sl), s1 = __ldg(sl + 1), s2 = __ldg(sl + 2);
          int flags = __float_as_int(s2.z);
          int prim = __float_as_int(s2.y);
          bool hit;
          float t = 0, b1 = 0, b2 = 0;
          if (!(flags & SLOT_SHAPE)) {
            hit = triTest(s0, s1, s2, r, best_t, t, b1, b2);
          } else {
            const DShape& sh = TW_ACC(shapes)[__float_as_int(s0.x)];
            Ray ro = transRay(sh.w2o, Ray{r.o, r.d, r.tmin, ANY ? r.tmax : best_t});
            if (ANY && !(MIXED && by_intersect)) {
              hit = shapeIntersects(sh, ro);
            } else {
              float e;
              hit = shapeIntersect<false>(sh, ro, t, e, nullptr);
            }
          }
          if (MIXED && rank_prim >= 0)  // ranked against a hit of rank_prim at tmax
            hit = hit && (t < r.tmax || prim > rank_prim);
          if (hit) {
            if (ANY) {
              best_prim = prim;
              cur = kSentinel;  // done: any hit suffices
              break;
            }
            if (t < best_t || prim > best_prim) {
              best_t = t;
              best_prim = prim;
              bb1 = b1;
              bb2 = b2;
            }
          }
          if (flags & SLOT_LAST) break;
          slot++;
        }
      }
    }
    // ---- finished rays
    if (rid >= 0 && cur == kSentinel && leaf == kSentinel) {
      emit(rid, RayQueryResult{best_prim >= 0, best_t, bb1, bb2, best_prim});
      rid = -1;
    }
  }
#undef TW_ACC
}

}  // namespace bgpu
