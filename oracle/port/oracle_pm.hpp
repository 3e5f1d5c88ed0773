// Oracle (test infrastructure only): CPU restatement of the reference's
// stochastic progressive photon mapper (core/src/PhotonMapping.cpp,
// core/include/Hasty/PhotonMapping.h, core/include/Hasty/HashCells.h) as one
// render thread runs it: a caustics photon map (L S+ D paths, stored at
// diffuse surfaces after the first bounce) rebuilt every iteration into hash
// cells, a gather that path-traces from the camera with both MIS strategies
// and adds photon estimates at diffuse vertices, and the per-pixel radius /
// flux statistics of PMRenderJob. Random streams are keyed like the path
// tracer's: photon i of iteration t draws from photon_key(seed, i, t), the
// camera sample of pixel p in iteration t from path_key(seed, p, t), and the
// initial radius footprint of pixel p from path_key(seed, p, kFootprintPass).
#pragma once
#include <array>
#include <map>
#include <vector>

#include "oracle_core.hpp"

namespace hor {

// Photon (PhotonMapping.cpp:11-23) plus its emission index and depth, the
// order in which the reference appends it.
struct Photon { V3 wi; float ngwi; V3 x; V3 flux; uint32_t emitted; uint32_t depth; };

// PhotonMap with PointHashCells (PhotonMapping.cpp:73-186, HashCells.h:40-104).
struct PhotonMap {
  std::vector<Photon> photons;
  size_t emitted = 0;
  float cell = 1.0f;
  std::map<std::array<int32_t, 3>, std::vector<uint32_t>> cells;
  std::array<int32_t, 3> index(const V3& p) const {
    return {floor_int32(p.x / cell), floor_int32(p.y / cell), floor_int32(p.z / cell)};
  }
  void clear(float cell_size) { photons.clear(); cells.clear(); emitted = 0; cell = cell_size; }
  void build();
  // indices of the photons within `radius` of c, cells in (x, y, z)
  // lexicographic order and photons in insertion order within a cell
  void radius_search(const V3& c, float radius, std::vector<uint32_t>& out) const;
};

// tracePhoton with causticsMap = true (PhotonMapping.cpp:191-270).
void trace_photon(const Scene& sc, Rng& r, PhotonMap& pm, V3 o, V3 d, const V3& flux0, uint32_t emit_index);

// PathTraceWithCausticsMapResult (PhotonMapping.cpp:392-402).
struct PmResult { V3 photonFlux, LLight, LRest, LSpecular, LCaustic; int M = 0; };

// pathTraceWithCausticsMap (PhotonMapping.cpp:404-503).
PmResult path_trace_caustics(const Scene& sc, Rng& r, const PhotonMap& pm, LightRayInfo& lr, const V3& ro, const V3& rd,
                             const Hit* pre, V3& normal, V3& albedo, float& radius, int depth,
                             std::vector<uint32_t>& scratch);

// computeCellSize (PhotonMapping.cpp:522-576); radii[x + y * W].
float cell_size_for(const std::vector<float>& radii, uint32_t W, uint32_t H);
// computeRadiusPixelFootPrint (PhotonMapping.cpp:578-651), ignoreCosineTerm.
float footprint_radius(const Scene& sc, Rng& r, float default_r, int i, int j, int W, int H);
// getCloseNonNegative (PhotonMapping.cpp:653-678).
float close_non_negative(const std::vector<float>& img, int W, int H, int i, int j);

// PMRenderJobPixel (PhotonMapping.h:13-32).
struct PmPixel { float radius = -1.0f, N = 0.0f, Ne = 0.0f; V3 flux, LSum; int Nd = 0; };

struct PmState {
  uint32_t W = 0, H = 0;
  bool initialised = false;
  uint32_t iteration = 0;
  std::vector<float> radii;              // Image1f radii of renderPhotonThread, x + y * W
  std::vector<PmPixel> px;
  std::vector<float> color, normal, albedo;   // the thread's image buffers (3 per pixel)
  // last iteration: photons emitted, photons stored, cell size
  uint64_t emitted = 0, stored = 0;
  float cell = 0.0f;
};

// Initial radii of renderPhotonThread (PhotonMapping.cpp:830-833):
// computeInitialRadii(footprint scale 10) with a surface light, else 1.
void pm_init(const Scene& sc, PmState& st);
// One iteration of renderPhotonThread's loop (PhotonMapping.cpp:848-931).
void pm_iteration(const Scene& sc, PmState& st);

}  // namespace hor
