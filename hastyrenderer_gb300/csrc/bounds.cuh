// Bounds-checked build (HASTY_DEBUG_BOUNDS, a library variant built by
// `python -m hastyrenderer_gb300.build --debug-bounds`). Device code checks
// the indices it reads through — queue entries, ray ids, BVH nodes and
// leaf triangles, triangle ids of hits, materials, textures and texels,
// light triangles, medium-stack entries — and on a bad one records the kind
// in a status word and skips the access (a ray stops, a path ends, a lookup
// returns zero) instead of reading out of bounds; it never traps. The host
// reads and clears the word with hasty_debug_bounds_status. Without the
// flag the checks compile to nothing.
//
// Every translation unit that checks has its own status word (device
// variables are per module); each provides a reader (bounds_status_*). The
// bits are HASTY_BOUNDS_* of hasty_gpu.h.
#pragma once
#include <cstdint>

namespace hasty {

enum BoundsBit : uint32_t {
  BB_QUEUE = 1u << 0,       // path or ray queue entry outside the path pool
  BB_NODE = 1u << 1,        // BVH node index
  BB_LEAF_TRI = 1u << 2,    // leaf-ordered triangle index
  BB_TRI = 1u << 3,         // triangle id of a hit or light sample
  BB_MATERIAL = 1u << 4,
  BB_TEXTURE = 1u << 5,     // texture index or texel offset
  BB_LIGHT = 1u << 6,       // light-triangle or CDF index
  BB_MEDIA = 1u << 7,       // medium-stack entry or overflow block
  BB_SAMPLE = 1u << 8,      // per-sample output index
};

}  // namespace hasty

#if defined(HASTY_DEBUG_BOUNDS) && defined(__CUDACC__)
namespace hasty {
namespace {
__device__ unsigned int g_bounds_status;
}
}  // namespace hasty
#endif
#if defined(HASTY_DEBUG_BOUNDS) && defined(__CUDA_ARCH__)
// True when `cond` holds; otherwise records `bit` and is false.
#define HASTY_IN_BOUNDS(cond, bit) ((cond) ? true : (atomicOr(&::hasty::g_bounds_status, unsigned(bit)), false))
#else
#define HASTY_IN_BOUNDS(cond, bit) true
#endif

// Host side of one translation unit's status word: reads it and clears it
// (0 when the flag is off). Put once in each checking .cu file.
#if defined(HASTY_DEBUG_BOUNDS)
#define HASTY_BOUNDS_READER(name)                                                   \
  namespace hasty {                                                                 \
  uint32_t name() {                                                                 \
    unsigned int v = 0, z = 0;                                                      \
    if (cudaMemcpyFromSymbol(&v, g_bounds_status, sizeof(v)) != cudaSuccess) return ~0u; \
    cudaMemcpyToSymbol(g_bounds_status, &z, sizeof(z));                             \
    return v;                                                                       \
  }                                                                                 \
  }
#else
#define HASTY_BOUNDS_READER(name) \
  namespace hasty {               \
  uint32_t name() { return 0; }   \
  }
#endif
