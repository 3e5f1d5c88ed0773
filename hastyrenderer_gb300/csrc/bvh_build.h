// Bounding-volume hierarchy over the scene's triangles, built on the host
// with binned SAH and written in the GPU traversal layouts:
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
};

// tri_pos: 9 floats per triangle (v0, v1, v2). max_leaf: triangles per leaf.
void build_bvh_binary(const float* tri_pos, size_t n, int max_leaf, BvhHost& out);

}  // namespace hasty
