// Bounding-volume hierarchy over the scene's triangles, built with binned SAH
// (on the GPU by default, bvh_gpu.cu; on the host here) as a binary tree and
// written in the GPU traversal layouts:
//  * binary: 4 x float4 per node, (c0 x-range, c0 y-range), (c1 x, c1 y),
//    (c0 z-range, c1 z-range), (child0, child1, count0, count1) where a
//    negative child c is a leaf: ~c = first << 3 | count (count <= 7);
//  * triangles in leaf order as 3 x float4: v0 (w = global triangle id as
//    int bits), v0 - v1, v2 - v0 (the edge vectors of the intersection test).
// It stands in for Embree's scene build (core/src/Scene.cpp:122-191).
#pragma once
#include <cstdint>
#include <vector>

namespace hasty {

struct BvhHost {
  std::vector<float> nodes;       // 16 floats per node
  std::vector<float> tris;        // 12 floats per leaf-ordered triangle
  std::vector<int32_t> order;     // leaf position -> global triangle id
  int32_t depth = 0;
  double build_ms = 0;
  double tree_ms = 0;             // of which: the binary tree (device or host)
};

// Binary build tree: node 0 is the root; an inner node's children are the
// consecutive pair (child, child + 1); a leaf (child < 0) holds triangles
// idx[first .. first + count). Boxes are the exact float bounds of the
// triangles below.
struct TreeNode {
  float lo[3], hi[3];
  int32_t child, first, count;
  int32_t pad;
};
struct BinaryTree {
  std::vector<TreeNode> nodes;
  std::vector<int32_t> idx;
  int32_t depth = 0;
};

// Layout writers for a built tree (leaves of <= 7 triangles for the binary
// layout, <= 3 for the wide one).
void emit_bvh_binary(const BinaryTree& t, const float* tri_pos, BvhHost& out);
void emit_bvh_wide(const BinaryTree& t, const float* tri_pos, BvhHost& out);

// Device binned-SAH builder (bvh_gpu.cu): the same split rule as the host
// builder (32 bins per axis, leaf when no split beats the leaf cost), on the
// current CUDA device. Triangles are uploaded from tri_pos (host).
void build_tree_gpu(const float* tri_pos, size_t n, int max_leaf, BinaryTree& out);
// Tree and compressed 8-wide layout both on the device; byte-identical to
// build_tree_gpu + emit_bvh_wide (tree_ms set to the tree part).
void build_wide_gpu(const float* tri_pos, size_t n, BvhHost& out);
// True when the device layout equals the host layout of the same device
// tree, compared as bytes. info (8 values, may be null): device and host
// node counts, first differing node word (-1: none), device and host depth,
// triangles equal, order equal, two device builds equal.
bool check_wide_emit_gpu(const float* tri_pos, size_t n, int64_t* info);

// tri_pos: 9 floats per triangle (v0, v1, v2). max_leaf: triangles per leaf.
// Host builds; the _gpu variants build the tree on the device and write the
// layout on the host.
void build_bvh_binary(const float* tri_pos, size_t n, int max_leaf, BvhHost& out);
void build_bvh_binary_gpu(const float* tri_pos, size_t n, int max_leaf, BvhHost& out);

// Compressed 8-wide layout, 80 bytes per node (5 x float4):
//   p.xyz (float grid origin), e.xyz (int8 exponents of the power-of-two grid
//   step), inner-child mask (u8), first inner child (u32), first triangle
//   (u32), meta (8 x u8: 0 empty; 001|24+slot inner; unary count|offset leaf),
//   quantised child boxes qlo.x[8] qlo.y[8] qlo.z[8] qhi.x[8] qhi.y[8] qhi.z[8].
// Leaves hold up to 3 triangles; triangles are stored in slot order.
void build_bvh_wide(const float* tri_pos, size_t n, BvhHost& out);
void build_bvh_wide_gpu(const float* tri_pos, size_t n, BvhHost& out);

}  // namespace hasty
