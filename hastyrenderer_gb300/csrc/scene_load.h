// Host-side loading of a render job into flat arrays ready for upload.
// Mirrors the reference's job surface: RenderJob::loadJSON
// (core/src/RenderJob.cpp:10-28), Scene::Scene (core/src/Scene.cpp:12-194),
// Camera from_json (core/src/Camera.cpp:9-38), EnvironmentTexture::load
// (core/include/Hasty/Environment.h:102-115), Texture loaders
// (core/src/Texture.cpp:21-49).
#pragma once
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "hasty_types.h"

namespace hasty {

// Loader failure; the C-ABI maps it to HASTY_ERR_LOAD (the reference's CLI
// exits with code 2 on a load exception, apps/PathTracingViewer.cpp:34-43).
struct LoadError : std::runtime_error { using std::runtime_error::runtime_error; };

struct RenderSettingsH {          // RenderSettings, core/include/Hasty/RenderJob.h:15-30
  int roulette_start = 1;
  float roulette_q = 0.3f;
  uint32_t width = 720, height = 720, num_threads = 4;
  int max_depth = 30, num_samples = 32;
  bool use_mis = true;
  uint64_t seed = 0;              // extension key "gb300": {"seed": N}
};

struct HostTexture { TextureDev desc; };

struct HostScene {
  RenderSettingsH settings;
  CameraDev cam{};
  // environment
  bool env_texture = false;
  float bg[3] = {0, 0, 0};
  int env_w = 0, env_h = 0;
  std::vector<float> env_texels, env_weights;
  std::vector<double> env_cdf;
  float env_value_sum = 0.f;
  // geometry
  std::vector<float> vertices, normals, texcoords;
  std::vector<float> tri_pos;     // 9 per triangle
  std::vector<TriAttr> tri_attr;
  uint32_t n_shapes = 0;
  // materials / textures
  std::vector<MaterialDev> mats;
  std::vector<TextureDev> textures;
  std::vector<float> tex_pool;      // float texels and the 8-bit textures' tables
  std::vector<uint8_t> tex_pool8;   // 8-bit texels
  // lights
  std::vector<int32_t> light_tris;
  std::vector<double> light_cdf;
  float total_light_area = 0.f;
  bool vary_glass_ior = false;
  // world "dispersion": {"model": "cauchy", "b": um^2, "wavelengths": [3 x um]}
  // (extension; default: the reference's fixed band ratios)
  bool cauchy = false;
  float cauchy_b = 0.0042f;
  float band_um[3] = {0.65f, 0.55f, 0.45f};

  size_t n_tris() const { return tri_attr.size(); }
  bool has_light() const {
    bool bg_zero = !env_texture && bg[0] == 0.f && bg[1] == 0.f && bg[2] == 0.f;
    return !light_tris.empty() || !bg_zero;
  }
};

// Loads renderJob.json and everything it references. Throws LoadError.
void load_render_job(const std::string& job_path, HostScene& out);
// The parts of load_render_job: the job file's settings and scene path; the
// scene file (camera, world, mesh, materials, lights; `out.settings` is left
// as it is); the checks that depend on both.
void load_job_settings(const std::string& job_path, RenderSettingsH& st, std::string& scene_path);
void load_scene_file(const std::string& scene_path, HostScene& out);
void check_job_settings(const RenderSettingsH& st, const HostScene& sc);

// libstdc++'s std::discrete_distribution table: weights normalised by their
// sequential double sum, running sums, last entry forced to 1. Fewer than
// two weights: empty (the distribution then returns 0 without drawing).
std::vector<double> build_discrete_cdf(const float* w, size_t n);

// Bucket starts for an exact lower_bound over `cdf`: with K = 2^log2k
// buckets, entry k is the first index whose value is >= k/K (K+1 entries).
// Empty for tables with fewer than two entries.
std::vector<uint32_t> build_cdf_guide(const std::vector<double>& cdf, uint32_t& log2k);

// Halton offsets of pass k (core/include/Hasty/Random.h:14-63).
float halton_value(uint32_t base, uint32_t k);
// Parses an OBJ file (and its MTL libraries) with `chunks` parse chunks (0:
// as many as the loader would use): a digest of the triangles' corner
// indices, materials, smoothing groups and shape boundaries, for checking
// that the result does not depend on the chunking.
uint64_t obj_digest(const std::string& path, size_t chunks, int64_t* n_tris, int64_t* n_shapes);

}  // namespace hasty
