// Stand-in for robin_hood.h (martinus/robin-hood-hashing, absent from the
// reference tree), providing only what core/include/Hasty/HashCells.h uses:
// hash_bytes and unordered_flat_map. The photon hash cells only look cells
// up (never iterate the map), so any hash and any map with the same lookup
// semantics gives the reference's results.
#pragma once
#include <cstddef>
#include <cstdint>
#include <unordered_map>

namespace robin_hood {

inline size_t hash_bytes(const void* p, size_t n) {   // FNV-1a, 64-bit
  const unsigned char* b = static_cast<const unsigned char*>(p);
  uint64_t h = 1469598103934665603ull;
  for (size_t i = 0; i < n; ++i) { h ^= b[i]; h *= 1099511628211ull; }
  return size_t(h);
}

template <class K, class V, class H, class E>
using unordered_flat_map = std::unordered_map<K, V, H, E>;

}  // namespace robin_hood
