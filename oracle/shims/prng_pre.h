// Oracle stand-in (test infrastructure only). Force-included before the
// reference's Random.h, which takes sizeof(prng_state) inside a template
// (core/include/Hasty/Random.h:62-70) and so needs the complete type first.
// The state holds the project's PCG32 stream or a position in a replayed list.
#pragma once
#include <stdint.h>
#include <stddef.h>
struct prng_state {
  uint64_t state, inc;     // PCG32
  uint64_t replay_pos;     // next index into the replayed list
  int replay;              // 1: serve values from the replayed list
};
