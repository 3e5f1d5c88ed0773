// Wavefront path state and kernel launch interface (host + device).
//
// One path slot per camera sample of a batch: slot = k * (W*H) + pixel for
// pass pass_base + k. State lives in structure-of-arrays buffers in HBM;
// each bounce runs `trace` (closest hit of every queued ray) and `shade`
// (resolve the previous vertex's NEE and BSDF samples, shade the new vertex,
// emit its rays). Queues are compacted with warp ballots.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>
#include "hasty_types.h"

namespace hasty {

// flags word (stored as the w lane of PathsDev::rad)
enum : uint32_t {
  PF_DEPTH_MASK = 0xFFu,          // depth of the vertex the pending BRDF ray leaves from
  PF_WL_SHIFT = 8,                // wavelength + 1 (0: not chosen yet)
  PF_WL_MASK = 0x3u << 8,
  PF_NMED_SHIFT = 10,             // media on the stack (0..4)
  PF_NMED_MASK = 0x7u << 10,
  PF_PEND_B = 1u << 14,           // BSDF-sampled ray queued in ray slot 2s
  PF_PEND_L = 1u << 15,           // light-sampled ray queued in ray slot 2s+1
  PF_CAMERA = 1u << 16,           // pending ray is the camera ray
};
constexpr int kMaxMedia = 4;

struct PathsDev {
  uint64_t* rng;        // PCG32 state
  float4* thr;          // xyz: path throughput up to the pending BSDF sample, w: its pdf
  float4* rad;          // xyz: radiance gathered so far, w: flags
  float4* pend_b;       // xyz: BSDF-sample weight (f|cos|/pdf * RR/Beer of its vertex), w: vertex triangle
  float4* nee_c;        // xyz: throughput * f * |cos| of the light sample, w: BSDF pdf of its direction
  float4* nee_t;        // xyz: medium transmittance along the light ray, w: sampled light triangle (-1: env)
  float4* med;          // 4 per path: medium transmittance xyz, IOR
  int32_t* med_geom;    // 4 per path: OBJ shape id of the medium
  float4* ray_o;        // 2 per path
  float4* ray_d;        // 2 per path
  float4* hit;          // 2 per path: t, u, v, triangle (-1 miss)
  int32_t* pq[2];       // path queues
  int32_t* rq[2];       // ray queues (ray ids 2s, 2s+1)
  uint32_t* counts;     // [pq0, pq1, rq0, rq1]
  float4* out_color;    // per slot: final radiance of the sample
  float4* out_normal;
  float4* out_albedo;
  unsigned long long* stats;   // see StatIndex
  int32_t capacity;
};

enum StatIndex { ST_RAYS = 0, ST_SHADED, ST_PATHS, ST_NAN, ST_MEDIA_OVERFLOW, ST_TRIAL_CAP, ST_COUNT };

struct BatchDesc {
  uint64_t seed;
  uint32_t pass_base;
  int32_t n_passes;
  int32_t n_paths;      // n_passes * W * H
};

// Kernel launchers (integrator.cu / trace.cu). All launches go to `stream`.
void launch_raygen(const SceneDev& sc, const PathsDev& p, const BatchDesc& b, cudaStream_t stream);
void launch_trace(const SceneDev& sc, const PathsDev& p, int q, int max_rays, cudaStream_t stream);
void launch_shade(const SceneDev& sc, const PathsDev& p, const BatchDesc& b, int q, int max_paths, cudaStream_t stream);
void launch_accumulate(const SceneDev& sc, const PathsDev& p, const BatchDesc& b, double* acc_color, double* acc_normal,
                       double* acc_albedo, cudaStream_t stream);
void launch_estimate(const double* acc, int n, float den, float scale, float* out, cudaStream_t stream);

// Closest-hit queries of arbitrary rays (n x 6 floats, device memory).
void launch_trace_rays(const SceneDev& sc, const float* rays, int n, float4* hits, cudaStream_t stream);

}  // namespace hasty
