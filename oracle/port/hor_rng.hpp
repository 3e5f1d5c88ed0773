// Oracle (test infrastructure only): the project's PCG-family random stream and
// the libstdc++ discrete-distribution draw, restated for the CPU oracle.
//
// The reference's RNG is shishua (core/src/Random.cpp:5-47, pinned commit
// ed0d60a8b35fb6aba711dcbc24aaeda78c623b45 in cmake/AddShishua.cmake:3), read
// through RNG::uniform01f (core/include/Hasty/Random.h:131-137) as
// (u32 & 0x7FFFFF) * 2^-23. shishua is not vendored, so parity of the raw
// stream with upstream is unpinned; the oracle, the reference build under
// oracle/_ref (through its shishua.h stand-in) and the CUDA path all draw from
// the PCG32 stream defined here, keyed per (job seed, pixel, pass).
#pragma once
#include <cstdint>
#include <cstddef>
#include <vector>
#include <algorithm>
#include <cmath>

namespace hor {

inline uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Stream key of one camera path: job seed, pixel index y*W+x, pass index.
inline uint64_t path_key(uint64_t seed, uint32_t pixel, uint32_t pass) {
  return splitmix64(splitmix64(seed) ^ ((uint64_t(pass) << 32) | uint64_t(pixel)));
}

// Photon mapper streams: photon i of iteration t, and the initial radius
// footprint of pixel p (pass value no render reaches).
constexpr uint64_t kPhotonKeyMix = 0x50484F544F4E5321ull;
constexpr uint32_t kFootprintPass = 0xFFFFFFFFu;
inline uint64_t photon_key(uint64_t seed, uint32_t photon, uint32_t iteration) {
  return path_key(seed ^ kPhotonKeyMix, photon, iteration);
}

constexpr uint64_t kPcgMult = 6364136223846793005ull;

// PCG32 (XSH-RR output, 64-bit LCG state), O'Neill 2014.
struct Pcg32 {
  uint64_t state = 0, inc = 1;
  void seed_key(uint64_t key) {
    inc = (splitmix64(key ^ 0xA5A5A5A5A5A5A5A5ull) << 1) | 1ull;
    state = 0;
    state = state * kPcgMult + inc;
    state += splitmix64(key);
    state = state * kPcgMult + inc;
  }
  uint32_t next() {
    uint64_t old = state;
    state = old * kPcgMult + inc;
    uint32_t xs = uint32_t(((old >> 18) ^ old) >> 27);
    uint32_t rot = uint32_t(old >> 59);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
  }
};

// A u32 source that is either a keyed PCG stream or a replayed list of
// values (known-answer tests feed the same list to the reference build).
struct Rng {
  Pcg32 pcg;
  const uint32_t* replay = nullptr;
  size_t replay_n = 0, replay_pos = 0;
  uint64_t draws = 0;
  explicit Rng(uint64_t key = 0) { pcg.seed_key(key); }
  static Rng from_replay(const uint32_t* v, size_t n) {
    Rng r(0); r.replay = v; r.replay_n = n; return r;
  }
  uint32_t next_u32() {
    ++draws;
    if (replay) { uint32_t v = replay[replay_pos % replay_n]; ++replay_pos; return v; }
    return pcg.next();
  }
  // RNG::uniform01f, core/include/Hasty/Random.h:139-145
  float uniform01f() { return float(next_u32() & 0x007FFFFFu) * 1.1920928955078125e-07f; }
  float uniformm11f() { return 2.0f * uniform01f() - 1.0f; }
};

// std::generate_canonical<double,53>(URBG with 32-bit range), as libstdc++
// (GCC 13, bits/random.tcc) evaluates it: two draws, low word first.
inline double canonical53(Rng& r) {
  double sum = 0.0, tmp = 1.0;
  for (int k = 0; k < 2; ++k) { sum += double(r.next_u32()) * tmp; tmp *= 4294967296.0; }
  double ret = sum / tmp;
  if (ret >= 1.0) ret = std::nextafter(1.0, 0.0);
  return ret;
}

// std::discrete_distribution<uint32_t> as libstdc++ builds and samples it:
// weights -> double, normalised by their sequential sum, partial sums with the
// last forced to 1.0, lower_bound of one canonical draw. Fewer than two
// weights: no draw, index 0.
struct DiscreteDist {
  std::vector<double> cdf;
  void build(const float* w, size_t n) {
    cdf.clear();
    if (n < 2) return;
    std::vector<double> p(w, w + n);
    double s = 0.0;
    for (double v : p) s += v;
    for (double& v : p) v = v / s;
    cdf.resize(n);
    double acc = 0.0;
    for (size_t i = 0; i < n; ++i) { acc = (i == 0) ? p[0] : acc + p[i]; cdf[i] = acc; }
    cdf[n - 1] = 1.0;
  }
  uint32_t sample(Rng& r) const {
    if (cdf.empty()) return 0;
    double u = canonical53(r);
    return uint32_t(std::lower_bound(cdf.begin(), cdf.end(), u) - cdf.begin());
  }
};

// HaltonSequence (core/include/Hasty/Random.h:14-47): the k-th value (k from 0)
// is float(n)/float(d) with d = b^digits(k+1) and n the digit reversal of k+1.
inline float halton(uint32_t base, uint32_t k) {
  uint32_t i = k + 1, n = 0, d = 1;
  while (i > 0) { n = n * base + (i % base); i /= base; d *= base; }
  return float(n) / float(d);
}

}  // namespace hor
