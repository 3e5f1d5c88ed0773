// Oracle (test infrastructure only): closest-hit ray queries for the CPU
// oracle, standing in for Embree's rtcIntersect1 as the reference calls it
// (core/src/Scene.cpp:281-303: tnear 1e-6, tfar +inf, u/v = weights of the
// triangle's 2nd/3rd vertex, Ng = (v1-v0)x(v2-v0) unnormalised).
//
// Embree 3 is absent (vcpkg "embree3", version not pinned by the reference),
// so the triangle test restates the published Moeller-Trumbore formulation in
// Embree's sign conventions, and the acceleration structure is a binary BVH
// (binned SAH, 32 bins, leaves of at most 4 triangles). Ties at equal t go to
// the smaller primitive index so that the answer does not depend on the
// traversal order. A double-precision brute-force query serves as a
// second, independent check.
#pragma once
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <limits>
#include <vector>

namespace hor {

struct BvhHit {
  int32_t prim = -1;      // index into the triangle list, -1 for a miss
  float t = 0.f, u = 0.f, v = 0.f;
  float ng[3] = {0, 0, 0};
};

struct BvhStats { uint64_t nodes = 0, tris = 0; };

// One ray/triangle test; returns true and fills t,u,v,Ng when the hit lies in
// (tnear, tfar]. Same arithmetic order as the CUDA intersector.
inline bool tri_intersect(const float o[3], const float d[3], const float* v0, const float* v1,
                          const float* v2, float tnear, float tfar, float& t, float& u, float& v,
                          float ng[3]) {
  float e1[3] = {v0[0] - v1[0], v0[1] - v1[1], v0[2] - v1[2]};
  float e2[3] = {v2[0] - v0[0], v2[1] - v0[1], v2[2] - v0[2]};
  float n[3] = {e2[1] * e1[2] - e2[2] * e1[1], e2[2] * e1[0] - e2[0] * e1[2], e2[0] * e1[1] - e2[1] * e1[0]};
  float c[3] = {v0[0] - o[0], v0[1] - o[1], v0[2] - o[2]};
  float r[3] = {c[1] * d[2] - c[2] * d[1], c[2] * d[0] - c[0] * d[2], c[0] * d[1] - c[1] * d[0]};
  float den = n[0] * d[0] + n[1] * d[1] + n[2] * d[2];
  float absden = std::fabs(den);
  float sgn = den < 0.f ? -1.f : 1.f;
  float U = (r[0] * e2[0] + r[1] * e2[1] + r[2] * e2[2]) * sgn;
  float V = (r[0] * e1[0] + r[1] * e1[1] + r[2] * e1[2]) * sgn;
  if (!(den != 0.f && U >= 0.f && V >= 0.f && U + V <= absden)) return false;
  float T = (n[0] * c[0] + n[1] * c[1] + n[2] * c[2]) * sgn;
  if (!(absden * tnear < T)) return false;
  // the far limit is applied to the divided distance, so that the closest
  // hit over a set of triangles does not depend on the order they are tested
  t = T / absden;
  if (!(t <= tfar)) return false;
  u = U / absden; v = V / absden;
  ng[0] = n[0]; ng[1] = n[1]; ng[2] = n[2];
  return true;
}

struct Bvh2 {
  struct Node { float bmin[3], bmax[3]; int32_t left_or_first; int32_t count; };
  std::vector<Node> nodes;
  std::vector<int32_t> order;       // leaf-ordered triangle indices
  const float* tv = nullptr;        // 9 floats per triangle (v0,v1,v2)
  size_t ntri = 0;

  void build(const float* tri_verts, size_t n) {
    tv = tri_verts; ntri = n;
    nodes.clear(); order.resize(n);
    for (size_t i = 0; i < n; ++i) order[i] = int32_t(i);
    if (n == 0) return;
    std::vector<float> cen(3 * n), bb(6 * n);
    for (size_t i = 0; i < n; ++i) {
      const float* p = tv + 9 * i;
      for (int a = 0; a < 3; ++a) {
        float lo = std::min(p[a], std::min(p[3 + a], p[6 + a]));
        float hi = std::max(p[a], std::max(p[3 + a], p[6 + a]));
        bb[6 * i + a] = lo; bb[6 * i + 3 + a] = hi;
        cen[3 * i + a] = 0.5f * (lo + hi);
      }
    }
    nodes.reserve(2 * n);
    nodes.push_back(Node());
    struct Task { int node, first, count; };
    std::vector<Task> stack{{0, 0, int(n)}};
    while (!stack.empty()) {
      Task tk = stack.back(); stack.pop_back();
      Node& nd = nodes[tk.node];
      float cmin[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, cmax[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
      for (int a = 0; a < 3; ++a) { nd.bmin[a] = FLT_MAX; nd.bmax[a] = -FLT_MAX; }
      for (int k = tk.first; k < tk.first + tk.count; ++k) {
        int i = order[k];
        for (int a = 0; a < 3; ++a) {
          nd.bmin[a] = std::min(nd.bmin[a], bb[6 * i + a]);
          nd.bmax[a] = std::max(nd.bmax[a], bb[6 * i + 3 + a]);
          cmin[a] = std::min(cmin[a], cen[3 * i + a]);
          cmax[a] = std::max(cmax[a], cen[3 * i + a]);
        }
      }
      auto area = [](const float* lo, const float* hi) {
        float dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
        return (dx < 0.f) ? 0.f : 2.f * (dx * dy + dy * dz + dz * dx);
      };
      int best_axis = -1, best_bin = -1;
      float best_cost = FLT_MAX;
      constexpr int B = 32;
      if (tk.count > 1) {
        for (int a = 0; a < 3; ++a) {
          float ext = cmax[a] - cmin[a];
          if (!(ext > 0.f)) continue;
          float lo[B][3], hi[B][3]; int cnt[B] = {0};
          for (int b = 0; b < B; ++b) for (int c = 0; c < 3; ++c) { lo[b][c] = FLT_MAX; hi[b][c] = -FLT_MAX; }
          float scale = float(B) / ext;
          for (int k = tk.first; k < tk.first + tk.count; ++k) {
            int i = order[k];
            int b = std::min(B - 1, int((cen[3 * i + a] - cmin[a]) * scale));
            cnt[b]++;
            for (int c = 0; c < 3; ++c) { lo[b][c] = std::min(lo[b][c], bb[6 * i + c]); hi[b][c] = std::max(hi[b][c], bb[6 * i + 3 + c]); }
          }
          float ra[B], rlo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, rhi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
          int rc[B], rcount = 0;
          for (int b = B - 1; b > 0; --b) {
            for (int c = 0; c < 3; ++c) { rlo[c] = std::min(rlo[c], lo[b][c]); rhi[c] = std::max(rhi[c], hi[b][c]); }
            rcount += cnt[b]; rc[b] = rcount; ra[b] = area(rlo, rhi);
          }
          float llo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, lhi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
          int lcount = 0;
          for (int b = 0; b < B - 1; ++b) {
            for (int c = 0; c < 3; ++c) { llo[c] = std::min(llo[c], lo[b][c]); lhi[c] = std::max(lhi[c], hi[b][c]); }
            lcount += cnt[b];
            if (lcount == 0 || rc[b + 1] == 0) continue;
            float cost = area(llo, lhi) * lcount + ra[b + 1] * rc[b + 1];
            if (cost < best_cost) { best_cost = cost; best_axis = a; best_bin = b; }
          }
        }
      }
      float leaf_cost = area(nd.bmin, nd.bmax) * tk.count;
      bool make_leaf = tk.count <= 1 || (tk.count <= 4 && (best_axis < 0 || leaf_cost <= best_cost));
      if (make_leaf) { nd.left_or_first = tk.first; nd.count = tk.count; continue; }
      int mid;
      if (best_axis >= 0) {
        float ext = cmax[best_axis] - cmin[best_axis];
        float scale = float(B) / ext;
        auto it = std::partition(order.begin() + tk.first, order.begin() + tk.first + tk.count, [&](int i) {
          return std::min(B - 1, int((cen[3 * i + best_axis] - cmin[best_axis]) * scale)) <= best_bin;
        });
        mid = int(it - order.begin());
      } else {
        mid = tk.first + tk.count / 2;
      }
      int l = int(nodes.size());
      nodes.push_back(Node()); nodes.push_back(Node());
      Node& nd2 = nodes[tk.node];
      nd2.left_or_first = l; nd2.count = 0;
      stack.push_back({l, tk.first, mid - tk.first});
      stack.push_back({l + 1, mid, tk.first + tk.count - mid});
    }
  }

  // Slab test with each distance rounded once and the interval widened by
  // 1 +/- 2*gamma(3), so that rounding never culls a box the ray touches.
  static bool ray_box(const float o[3], const float inv[3], const float* lo, const float* hi, float tmax, float& tent) {
    float t0 = 0.f, t1 = INFINITY;
    for (int a = 0; a < 3; ++a) {
      float ta = (lo[a] - o[a]) * inv[a], tb = (hi[a] - o[a]) * inv[a];
      if (ta > tb) std::swap(ta, tb);
      if (!(ta <= tb)) { ta = -INFINITY; tb = INFINITY; }  // 0*inf on a slab edge
      t0 = std::max(t0, ta); t1 = std::min(t1, tb);
    }
    t0 *= 0.9999992f;
    t1 = std::min(t1 * 1.0000008f, tmax * 1.0000008f);
    tent = t0;
    return t0 <= t1;
  }

  BvhHit intersect(const float o[3], const float d[3], float tnear, float tfar, BvhStats* st = nullptr) const {
    BvhHit h;
    if (nodes.empty()) return h;
    float inv[3];
    for (int a = 0; a < 3; ++a) inv[a] = 1.0f / d[a];
    float best = tfar;
    int stack[128]; int sp = 0; stack[sp++] = 0;
    while (sp) {
      const Node& nd = nodes[stack[--sp]];
      if (st) st->nodes++;
      float te;
      if (!ray_box(o, inv, nd.bmin, nd.bmax, best, te)) continue;
      if (nd.count > 0) {
        for (int k = nd.left_or_first; k < nd.left_or_first + nd.count; ++k) {
          int i = order[k];
          if (st) st->tris++;
          const float* p = tv + 9 * size_t(i);
          float t, u, v, ng[3];
          if (tri_intersect(o, d, p, p + 3, p + 6, tnear, best, t, u, v, ng)) {
            if (t < best || (t == best && (h.prim < 0 || i < h.prim))) {
              best = t; h.prim = i; h.t = t; h.u = u; h.v = v;
              h.ng[0] = ng[0]; h.ng[1] = ng[1]; h.ng[2] = ng[2];
            }
          }
        }
      } else {
        const Node& a = nodes[nd.left_or_first];
        const Node& b = nodes[nd.left_or_first + 1];
        float ta, tb;
        bool ha = ray_box(o, inv, a.bmin, a.bmax, best, ta);
        bool hb = ray_box(o, inv, b.bmin, b.bmax, best, tb);
        if (ha && hb) {
          if (ta <= tb) { stack[sp++] = nd.left_or_first + 1; stack[sp++] = nd.left_or_first; }
          else { stack[sp++] = nd.left_or_first; stack[sp++] = nd.left_or_first + 1; }
        } else if (ha) stack[sp++] = nd.left_or_first;
        else if (hb) stack[sp++] = nd.left_or_first + 1;
        if (sp > 124) sp = 124;  // depth guard; binned SAH trees stay far below
      }
    }
    return h;
  }

  // Every triangle with the same FP32 test: the exact closest hit for this
  // triangle test, independent of any tree.
  BvhHit intersect_brute(const float o[3], const float d[3], float tnear, float tfar) const {
    BvhHit h; float best = tfar;
    for (size_t i = 0; i < ntri; ++i) {
      const float* p = tv + 9 * i;
      float t, u, v, ng[3];
      if (tri_intersect(o, d, p, p + 3, p + 6, tnear, best, t, u, v, ng) &&
          (t < best || (t == best && (h.prim < 0 || int(i) < h.prim)))) {
        best = t; h.prim = int(i); h.t = t; h.u = u; h.v = v;
        h.ng[0] = ng[0]; h.ng[1] = ng[1]; h.ng[2] = ng[2];
      }
    }
    return h;
  }

  // Double-precision brute force over every triangle.
  BvhHit intersect_fp64(const float o[3], const float d[3], float tnear, float tfar) const {
    BvhHit h; double best = tfar;
    for (size_t i = 0; i < ntri; ++i) {
      const float* p = tv + 9 * i;
      double e1[3], e2[3], n[3], c[3], r[3], dd[3] = {d[0], d[1], d[2]};
      for (int a = 0; a < 3; ++a) { e1[a] = double(p[a]) - p[3 + a]; e2[a] = double(p[6 + a]) - p[a]; c[a] = double(p[a]) - o[a]; }
      n[0] = e2[1] * e1[2] - e2[2] * e1[1]; n[1] = e2[2] * e1[0] - e2[0] * e1[2]; n[2] = e2[0] * e1[1] - e2[1] * e1[0];
      r[0] = c[1] * dd[2] - c[2] * dd[1]; r[1] = c[2] * dd[0] - c[0] * dd[2]; r[2] = c[0] * dd[1] - c[1] * dd[0];
      double den = n[0] * dd[0] + n[1] * dd[1] + n[2] * dd[2];
      double ad = std::fabs(den), sg = den < 0 ? -1.0 : 1.0;
      double U = (r[0] * e2[0] + r[1] * e2[1] + r[2] * e2[2]) * sg;
      double V = (r[0] * e1[0] + r[1] * e1[1] + r[2] * e1[2]) * sg;
      if (!(den != 0 && U >= 0 && V >= 0 && U + V <= ad)) continue;
      double T = (n[0] * c[0] + n[1] * c[1] + n[2] * c[2]) * sg;
      if (!(ad * tnear < T && T <= ad * best)) continue;
      double t = T / ad;
      if (t < best || (t == best && (h.prim < 0 || int(i) < h.prim))) {
        best = t; h.prim = int(i); h.t = float(t); h.u = float(U / ad); h.v = float(V / ad);
        h.ng[0] = float(n[0]); h.ng[1] = float(n[1]); h.ng[2] = float(n[2]);
      }
    }
    return h;
  }
};

}  // namespace hor
