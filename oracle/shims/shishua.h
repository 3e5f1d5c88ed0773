// Oracle stand-in for shishua (upstream pinned at
// ed0d60a8b35fb6aba711dcbc24aaeda78c623b45 by the reference's
// cmake/AddShishua.cmake; not present here). Same two entry points the
// reference calls (core/src/Random.cpp:5-47); the values come from the
// project's PCG32 stream keyed by seed[0], or from a replayed list.
#pragma once
#include "prng_pre.h"
void prng_init(struct prng_state* s, uint64_t seed[4]);
void prng_gen(struct prng_state* s, uint8_t* buf, size_t size);
