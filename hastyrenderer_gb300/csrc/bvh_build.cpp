// Binned-SAH binary BVH builder (host, multi-threaded). See bvh_build.h.
#include "bvh_build.h"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>

namespace hasty {
namespace {

struct Box {
  float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  void grow(const Box& b) { for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], b.lo[a]); hi[a] = std::max(hi[a], b.hi[a]); } }
  void grow(const float* p) { for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], p[a]); hi[a] = std::max(hi[a], p[a]); } }
  float area() const {
    float d[3] = {hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2]};
    if (d[0] < 0.f) return 0.f;
    return 2.f * (d[0] * d[1] + d[1] * d[2] + d[2] * d[0]);
  }
};

struct BNode { Box box; int32_t child = -1; int32_t first = 0, count = 0; };

struct Builder {
  const float* pos; size_t n; int max_leaf;
  std::vector<Box> tbox;
  std::vector<float> cen;
  std::vector<int32_t> idx;
  std::vector<BNode> nodes;
  std::atomic<int32_t> next_node{1};
  std::atomic<int32_t> max_depth{0};

  struct Task { int32_t node, first, count, depth; };
  std::mutex mu; std::condition_variable cv;
  std::deque<Task> queue; int active = 0;

  void push(const Task& t) { { std::lock_guard<std::mutex> g(mu); queue.push_back(t); } cv.notify_one(); }

  void run_task(Task t) {
    // large tasks split here and hand one child to the pool; small ones recurse locally
    std::vector<Task> local{t};
    while (!local.empty()) {
      Task k = local.back(); local.pop_back();
      int32_t d = k.depth;
      int32_t md = max_depth.load();
      while (d > md && !max_depth.compare_exchange_weak(md, d)) {}
      BNode& nd = nodes[size_t(k.node)];
      Box cb;
      nd.box = Box();
      for (int32_t i = k.first; i < k.first + k.count; ++i) { nd.box.grow(tbox[size_t(idx[size_t(i)])]); cb.grow(&cen[3 * size_t(idx[size_t(i)])]); }
      int axis = -1, split_bin = -1; float best = FLT_MAX;
      constexpr int B = 32;
      if (k.count > 1) {
        for (int a = 0; a < 3; ++a) {
          float ext = cb.hi[a] - cb.lo[a];
          if (!(ext > 0.f)) continue;
          Box bb[B]; int bc[B] = {0};
          float sc = float(B) / ext;
          for (int32_t i = k.first; i < k.first + k.count; ++i) {
            int32_t t2 = idx[size_t(i)];
            int b = std::max(0, std::min(B - 1, int((cen[3 * size_t(t2) + a] - cb.lo[a]) * sc)));
            bc[b]++; bb[b].grow(tbox[size_t(t2)]);
          }
          float rarea[B]; int rcnt[B];
          Box acc; int c = 0;
          for (int b = B - 1; b > 0; --b) { acc.grow(bb[b]); c += bc[b]; rarea[b] = acc.area(); rcnt[b] = c; }
          Box lacc; int lc = 0;
          for (int b = 0; b < B - 1; ++b) {
            lacc.grow(bb[b]); lc += bc[b];
            if (lc == 0 || rcnt[b + 1] == 0) continue;
            float cost = lacc.area() * float(lc) + rarea[b + 1] * float(rcnt[b + 1]);
            if (cost < best) { best = cost; axis = a; split_bin = b; }
          }
        }
      }
      float leaf_cost = nd.box.area() * float(k.count);
      bool leaf = k.count <= 1 || (k.count <= max_leaf && (axis < 0 || leaf_cost <= best));
      if (leaf) { nd.first = k.first; nd.count = k.count; nd.child = -1; continue; }
      int32_t mid;
      if (axis >= 0) {
        float sc = float(B) / (cb.hi[axis] - cb.lo[axis]);
        float lo = cb.lo[axis];
        auto it = std::partition(idx.begin() + k.first, idx.begin() + k.first + k.count, [&](int32_t t2) {
          return std::max(0, std::min(B - 1, int((cen[3 * size_t(t2) + axis] - lo) * sc))) <= split_bin;
        });
        mid = int32_t(it - idx.begin());
      } else {
        mid = k.first + k.count / 2;   // all centroids coincide: split by index
      }
      int32_t c0 = next_node.fetch_add(2);
      nd.child = c0; nd.count = 0;
      Task a{c0, k.first, mid - k.first, d + 1}, b{c0 + 1, mid, k.first + k.count - mid, d + 1};
      if (b.count > 65536) push(b); else local.push_back(b);
      if (a.count > 65536) push(a); else local.push_back(a);
    }
  }

  void worker() {
    for (;;) {
      Task t;
      {
        std::unique_lock<std::mutex> g(mu);
        cv.wait(g, [&] { return !queue.empty() || active == 0; });
        if (queue.empty()) return;
        t = queue.front(); queue.pop_front(); ++active;
      }
      run_task(t);
      { std::lock_guard<std::mutex> g(mu); --active; }
      cv.notify_all();
    }
  }
};

void run_builder(Builder& b, const float* tri_pos, size_t n, int max_leaf) {
  b.pos = tri_pos; b.n = n; b.max_leaf = max_leaf;
  b.tbox.resize(n); b.cen.resize(3 * n); b.idx.resize(n);
  for (size_t i = 0; i < n; ++i) {
    Box bx;
    for (int k = 0; k < 3; ++k) bx.grow(tri_pos + 9 * i + 3 * k);
    b.tbox[i] = bx;
    for (int a = 0; a < 3; ++a) b.cen[3 * i + size_t(a)] = 0.5f * (bx.lo[a] + bx.hi[a]);
    b.idx[i] = int32_t(i);
  }
  b.nodes.resize(std::max<size_t>(2 * n + 1, 3));
  b.push({0, 0, int32_t(n), 0});
  unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  if (n < 200000) nt = 1;
  std::vector<std::thread> th;
  for (unsigned i = 0; i < nt; ++i) th.emplace_back([&] { b.worker(); });
  for (auto& t : th) t.join();
}

void leaf_ordered_tris(const float* tri_pos, const std::vector<int32_t>& order, std::vector<float>& tris) {
  size_t n = order.size();
  tris.resize(12 * n);
  for (size_t i = 0; i < n; ++i) {
    int32_t t = order[i];
    const float* p = tri_pos + 9 * size_t(t);
    float* o = &tris[12 * i];
    o[0] = p[0]; o[1] = p[1]; o[2] = p[2]; std::memcpy(&o[3], &t, 4);
    o[4] = p[0] - p[3]; o[5] = p[1] - p[4]; o[6] = p[2] - p[5]; o[7] = 0.f;
    o[8] = p[6] - p[0]; o[9] = p[7] - p[1]; o[10] = p[8] - p[2]; o[11] = 0.f;
  }
}

}  // namespace

namespace {

Box box_of(const TreeNode& t) {
  Box b;
  for (int a = 0; a < 3; ++a) { b.lo[a] = t.lo[a]; b.hi[a] = t.hi[a]; }
  return b;
}

// The host builder's tree as a BinaryTree (nodes [0, used)).
void to_tree(const Builder& b, BinaryTree& t) {
  size_t used = size_t(b.next_node.load());
  t.nodes.resize(used);
  for (size_t i = 0; i < used; ++i) {
    const BNode& s = b.nodes[i];
    TreeNode& d = t.nodes[i];
    for (int a = 0; a < 3; ++a) { d.lo[a] = s.box.lo[a]; d.hi[a] = s.box.hi[a]; }
    d.child = s.child; d.first = s.first; d.count = s.count; d.pad = 0;
  }
  t.idx = b.idx;
  t.depth = b.max_depth.load() + 1;
}

}  // namespace

void emit_bvh_binary(const BinaryTree& t, const float* tri_pos, BvhHost& out) {
  // Emit the GPU layout breadth-first (keeps the top levels contiguous).
  // The root must be an inner node: a single leaf becomes child 0 of a root
  // whose child 1 is an empty leaf.
  const std::vector<TreeNode>& nd = t.nodes;
  struct Pending { TreeNode a, b; };
  TreeNode empty;
  for (int a = 0; a < 3; ++a) { empty.lo[a] = FLT_MAX; empty.hi[a] = -FLT_MAX; }
  empty.child = -1; empty.first = 0; empty.count = 0; empty.pad = 0;
  std::deque<Pending> q;
  if (nd[0].child < 0) q.push_back({nd[0], empty});
  else q.push_back({nd[size_t(nd[0].child)], nd[size_t(nd[0].child) + 1]});
  std::vector<size_t> fixups;   // float offsets of inner-child links, in push order
  out.nodes.clear();
  auto child_fields = [](const TreeNode& c, float* box6, int32_t& link, int32_t& cnt) {
    box6[0] = c.lo[0]; box6[1] = c.hi[0]; box6[2] = c.lo[1];
    box6[3] = c.hi[1]; box6[4] = c.lo[2]; box6[5] = c.hi[2];
    if (c.child < 0) { link = ~((c.first << 3) | c.count); cnt = c.count; } else { link = 0; cnt = 0; }
  };
  while (!q.empty()) {
    Pending p = q.front(); q.pop_front();
    size_t base = out.nodes.size();
    out.nodes.resize(base + 16);
    float* f = &out.nodes[base];
    float ba[6], bb[6]; int32_t la, lb, ca, cbn;
    child_fields(p.a, ba, la, ca); child_fields(p.b, bb, lb, cbn);
    f[0] = ba[0]; f[1] = ba[1]; f[2] = ba[2]; f[3] = ba[3];
    f[4] = bb[0]; f[5] = bb[1]; f[6] = bb[2]; f[7] = bb[3];
    f[8] = ba[4]; f[9] = ba[5]; f[10] = bb[4]; f[11] = bb[5];
    std::memcpy(&f[12], &la, 4); std::memcpy(&f[13], &lb, 4); std::memcpy(&f[14], &ca, 4); std::memcpy(&f[15], &cbn, 4);
    if (p.a.child >= 0) { fixups.push_back(base + 12); q.push_back({nd[size_t(p.a.child)], nd[size_t(p.a.child) + 1]}); }
    if (p.b.child >= 0) { fixups.push_back(base + 13); q.push_back({nd[size_t(p.b.child)], nd[size_t(p.b.child) + 1]}); }
  }
  // the k-th node pushed after the root is emitted as gpu node k+1
  for (size_t k = 0; k < fixups.size(); ++k) { int32_t v = int32_t(k + 1); std::memcpy(&out.nodes[fixups[k]], &v, 4); }
  out.order = t.idx;
  leaf_ordered_tris(tri_pos, out.order, out.tris);
  out.depth = t.depth;
}

void build_bvh_binary(const float* tri_pos, size_t n, int max_leaf, BvhHost& out) {
  auto t0 = std::chrono::steady_clock::now();
  Builder b;
  run_builder(b, tri_pos, n, max_leaf);
  BinaryTree t;
  to_tree(b, t);
  out.tree_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  emit_bvh_binary(t, tri_pos, out);
  out.build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

void build_bvh_binary_gpu(const float* tri_pos, size_t n, int max_leaf, BvhHost& out) {
  auto t0 = std::chrono::steady_clock::now();
  BinaryTree t;
  build_tree_gpu(tri_pos, n, max_leaf, t);
  out.tree_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  emit_bvh_binary(t, tri_pos, out);
  out.build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// ------------------------------------------------------------------------
// Compressed 8-wide BVH (the node format of Ylitie, Karras and Laine 2017):
// binary nodes are collapsed greedily (the child with the largest surface
// area is opened until 8 children), children are assigned to slots so that
// visiting slot (k ^ octant) for k = 7..0 is roughly front to back for a ray
// of that direction octant, and child boxes are quantised to 8 bits on a
// per-node power-of-two grid, conservatively (decoded in float, widened by
// one step when rounding would cut into the box).
namespace {

struct WideOut {
  std::vector<uint8_t> nodes;     // 80 bytes per node
  std::vector<int32_t> order;     // wide triangle position -> global id
  int depth = 0;
};

float pow2f(int e) { return std::ldexp(1.0f, e); }

// Smallest e with 255 * 2^e >= extent (exact comparisons; the log2 estimate
// only picks the start), clamped to [-100, 127]. The device writer in
// bvh_gpu.cu computes the same value.
int grid_exponent(float extent) {
  if (!(extent > 0.f)) return -100;
  int e = int(std::ceil(std::log2(double(extent) / 255.0)));
  e = std::max(-110, std::min(140, e));
  while (255.0 * std::ldexp(1.0, e) < double(extent)) ++e;
  while (255.0 * std::ldexp(1.0, e - 1) >= double(extent)) --e;
  return std::max(-100, std::min(127, e));
}

void emit_wide(const BinaryTree& b, WideOut& out) {
  const std::vector<TreeNode>& nd = b.nodes;
  auto area = [&](int32_t k) { return box_of(nd[size_t(k)]).area(); };
  struct Job { int32_t bnode; uint32_t wide; int depth; };
  std::deque<Job> q;
  out.nodes.assign(80, 0);
  q.push_back({0, 0, 1});
  uint32_t next_node = 1;
  out.order.clear();
  while (!q.empty()) {
    Job jb = q.front(); q.pop_front();
    out.depth = std::max(out.depth, jb.depth);
    // gather up to 8 children
    std::vector<int32_t> kids;
    const TreeNode& root = nd[size_t(jb.bnode)];
    if (root.child < 0) kids.push_back(jb.bnode);
    else { kids.push_back(root.child); kids.push_back(root.child + 1); }
    while (kids.size() < 8) {
      int best = -1; float best_area = -1.f;
      for (size_t i = 0; i < kids.size(); ++i) {
        const TreeNode& c = nd[size_t(kids[i])];
        if (c.child >= 0 && area(kids[i]) > best_area) { best_area = area(kids[i]); best = int(i); }
      }
      if (best < 0) break;
      int32_t c = kids[size_t(best)];
      kids[size_t(best)] = nd[size_t(c)].child;
      kids.push_back(nd[size_t(c)].child + 1);
    }
    // node box
    Box nb;
    for (int32_t k : kids) nb.grow(box_of(nd[size_t(k)]));
    float ctr[3] = {0.5f * (nb.lo[0] + nb.hi[0]), 0.5f * (nb.lo[1] + nb.hi[1]), 0.5f * (nb.lo[2] + nb.hi[2])};
    // slot assignment: slot s is entered first by rays whose direction signs
    // are ((s&4)?+:-, (s&2)?+:-, (s&1)?+:-); it takes the child that lies
    // furthest back along that direction.
    struct Cand { float cost; int kid, slot; };
    std::vector<Cand> cands;
    for (size_t i = 0; i < kids.size(); ++i) {
      const Box cb = box_of(nd[size_t(kids[i])]);
      float c[3] = {0.5f * (cb.lo[0] + cb.hi[0]) - ctr[0], 0.5f * (cb.lo[1] + cb.hi[1]) - ctr[1], 0.5f * (cb.lo[2] + cb.hi[2]) - ctr[2]};
      for (int s = 0; s < 8; ++s) {
        float d[3] = {(s & 4) ? 1.f : -1.f, (s & 2) ? 1.f : -1.f, (s & 1) ? 1.f : -1.f};
        cands.push_back({c[0] * d[0] + c[1] * d[1] + c[2] * d[2], int(i), s});
      }
    }
    std::stable_sort(cands.begin(), cands.end(), [](const Cand& a, const Cand& c) { return a.cost < c.cost; });
    int slot_of[8]; int kid_in[8];
    for (int i = 0; i < 8; ++i) { slot_of[i] = -1; kid_in[i] = -1; }
    for (const Cand& c : cands)
      if (slot_of[c.kid] < 0 && kid_in[c.slot] < 0) { slot_of[c.kid] = c.slot; kid_in[c.slot] = c.kid; }
    // quantisation grid
    int ex[3];
    for (int a = 0; a < 3; ++a) ex[a] = grid_exponent(nb.hi[a] - nb.lo[a]);
    uint8_t* node = &out.nodes[size_t(jb.wide) * 80];
    std::memcpy(node + 0, &nb.lo[0], 4); std::memcpy(node + 4, &nb.lo[1], 4); std::memcpy(node + 8, &nb.lo[2], 4);
    node[12] = uint8_t(int8_t(ex[0])); node[13] = uint8_t(int8_t(ex[1])); node[14] = uint8_t(int8_t(ex[2]));
    uint8_t imask = 0;
    uint32_t child_base = next_node;
    uint32_t tri_base = uint32_t(out.order.size());
    uint32_t tri_off = 0;
    // internal children get consecutive node indices in slot order
    for (int s = 0; s < 8; ++s) {
      uint8_t* meta = node + 24 + s;
      uint8_t* qlo[3] = {node + 32 + s, node + 40 + s, node + 48 + s};
      uint8_t* qhi[3] = {node + 56 + s, node + 64 + s, node + 72 + s};
      if (kid_in[s] < 0) { *meta = 0; for (int a = 0; a < 3; ++a) { *qlo[a] = 255; *qhi[a] = 0; } continue; }
      const TreeNode& c = nd[size_t(kids[size_t(kid_in[s])])];
      for (int a = 0; a < 3; ++a) {
        float sc = pow2f(ex[a]);
        float lo = nb.lo[a];
        double ql = std::floor((double(c.lo[a]) - double(lo)) / double(sc));
        double qh = std::ceil((double(c.hi[a]) - double(lo)) / double(sc));
        int il = int(std::max(0.0, std::min(255.0, ql)));
        int ih = int(std::max(0.0, std::min(255.0, qh)));
        // the device decodes fma(q, 2^e, p) rounded once; widen until conservative
        while (il > 0 && std::fma(float(il), sc, lo) > c.lo[a]) --il;
        while (ih < 255 && std::fma(float(ih), sc, lo) < c.hi[a]) ++ih;
        *qlo[a] = uint8_t(il); *qhi[a] = uint8_t(ih);
      }
      if (c.child >= 0) {
        imask |= uint8_t(1u << s);
        *meta = uint8_t((1u << 5) | uint32_t(24 + s));
      } else {
        int cnt = c.count;          // 0..3
        uint8_t unary = cnt == 0 ? 0 : (cnt == 1 ? 1 : (cnt == 2 ? 3 : 7));
        *meta = cnt == 0 ? 0 : uint8_t((unary << 5) | tri_off);
        for (int k = 0; k < cnt; ++k) out.order.push_back(b.idx[size_t(c.first + k)]);
        tri_off += uint32_t(cnt);
      }
    }
    for (int s = 0; s < 8; ++s) {
      if (kid_in[s] < 0) continue;
      int32_t k = kids[size_t(kid_in[s])];
      if (nd[size_t(k)].child >= 0) q.push_back({k, next_node++, jb.depth + 1});
    }
    node[15] = imask;
    std::memcpy(node + 16, &child_base, 4);
    std::memcpy(node + 20, &tri_base, 4);
    if (out.nodes.size() < size_t(next_node) * 80) out.nodes.resize(size_t(next_node) * 80, 0);
  }
}

}  // namespace

void emit_bvh_wide(const BinaryTree& t, const float* tri_pos, BvhHost& out) {
  WideOut w;
  emit_wide(t, w);
  out.nodes.resize(w.nodes.size() / 4);
  std::memcpy(out.nodes.data(), w.nodes.data(), w.nodes.size());
  out.order = w.order;
  leaf_ordered_tris(tri_pos, out.order, out.tris);
  out.depth = w.depth;
}

void build_bvh_wide(const float* tri_pos, size_t n, BvhHost& out) {
  auto t0 = std::chrono::steady_clock::now();
  Builder b;
  run_builder(b, tri_pos, n, 3);
  BinaryTree t;
  to_tree(b, t);
  out.tree_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  emit_bvh_wide(t, tri_pos, out);
  out.build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

void build_bvh_wide_gpu(const float* tri_pos, size_t n, BvhHost& out) {
  auto t0 = std::chrono::steady_clock::now();
  build_wide_gpu(tri_pos, n, out);       // tree and layout on the device
  out.build_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

namespace {
template <class T>
bool same_bytes(const std::vector<T>& a, const std::vector<T>& b) {
  return a.size() == b.size() && (a.empty() || std::memcmp(a.data(), b.data(), a.size() * sizeof(T)) == 0);
}
}  // namespace

bool check_wide_emit_gpu(const float* tri_pos, size_t n, int64_t* info) {
  BvhHost dev, dev2;
  build_wide_gpu(tri_pos, n, dev);
  build_wide_gpu(tri_pos, n, dev2);
  BinaryTree t;
  build_tree_gpu(tri_pos, n, 3, t);       // the same device tree, laid out on the host
  BvhHost host;
  emit_bvh_wide(t, tri_pos, host);
  int64_t first = -1;
  size_t m = std::min(dev.nodes.size(), host.nodes.size());
  for (size_t i = 0; i < m; ++i)
    if (std::memcmp(&dev.nodes[i], &host.nodes[i], 4) != 0) { first = int64_t(i); break; }
  bool nodes_eq = same_bytes(dev.nodes, host.nodes), tris_eq = same_bytes(dev.tris, host.tris);
  bool order_eq = same_bytes(dev.order, host.order);
  if (info) {
    info[0] = int64_t(dev.nodes.size() / 20); info[1] = int64_t(host.nodes.size() / 20); info[2] = first;
    info[3] = dev.depth; info[4] = host.depth; info[5] = tris_eq; info[6] = order_eq;
    info[7] = same_bytes(dev.nodes, dev2.nodes) && same_bytes(dev.order, dev2.order);
  }
  return nodes_eq && tris_eq && order_eq && dev.depth == host.depth;
}

}  // namespace hasty
