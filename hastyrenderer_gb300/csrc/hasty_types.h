// Device-resident scene and wavefront layouts shared by the host loader, the
// BVH builder and the CUDA kernels. All arrays live in HBM; the integrator
// reads them through the pointers of SceneDev.
#pragma once
#include <stdint.h>
#include <vector_types.h>   // float4 (CUDA header, usable from host C++)

#ifdef __CUDACC__
#define HD __host__ __device__ __forceinline__
#else
#define HD inline
#endif

namespace hasty {

// Principled material (core/include/Hasty/BRDF.h:161-171 plus MTL emission);
// a texture index of -1 means the constant value is used.
struct MaterialDev {
  float albedo[3]; int32_t albedo_tex;
  float roughness; int32_t roughness_tex;
  float metallic; int32_t metallic_tex;
  float specular, ior, anisotropy, transmission;
  int32_t normal_tex; int32_t vary_ior;
  float emission[3]; int32_t is_light;
  // IOR of the three dispersion bands (used when vary_ior): the reference's
  // ratios ior * {1.43, 1.45, 1.47} / 1.45 (core/src/BRDF.cpp:589-603), or
  // Cauchy's ior + b / lambda^2 when the world asks for it (extension).
  float ior_band[3]; int32_t pad_band;
};

// Nearest-neighbour texture, row 0 = top of the picture
// (core/include/Hasty/Texture.h:119-139). fmt 0: `ch` floats per texel at
// `offset` in the float pool; fmt 1: bytes at `offset` in the 8-bit pool (4
// per texel for ch 3, 1 for ch 1), each mapped through the 256 floats at
// `lut` in the float pool.
struct TextureDev { int32_t w, h, ch; int32_t clamp_u, clamp_v; int32_t fmt; int64_t offset; int64_t lut; };

// Per-triangle shading record, indexed by the global triangle id (shapes in
// file order, faces in shape order): vertex, normal and texcoord indices,
// material, OBJ shape (Embree geomID) and face index (primID).
struct TriAttr {
  int32_t vi[3], ni[3], ti[3];
  int32_t mat; uint32_t geom, prim; uint32_t smooth; int32_t pad;
};

struct CameraDev {
  float pos[3], fwd[3], right[3], up[3];
  float q;             // tan(fov/2), evaluated on the host as Camera.cpp:53
  float aperture, focal, exposure, blade_rot;
  int32_t blades;
  float ngon_per, ngon_nx, ngon_ny;   // sector angle and half-plane normal (Sample.cpp:18-20)
};

struct EnvDev {
  int32_t is_texture; float color[3];
  int32_t w, h;
  const float* texels;        // w*h*3, row 0 = zenith
  const float* weights;       // w*h, |rgb| * sin(theta)
  const double* cdf;          // w*h cumulative probabilities (last = 1)
  const uint32_t* guide;      // 2^guide_log2 + 1 bucket starts into cdf (exact lower_bound search ranges)
  uint32_t guide_log2;
  float value_sum;
};

// Wide BVH node: 8 children with 8-bit quantised boxes relative to the
// node's box (origin p, per-axis scale 2^e). 80 bytes = 5 x float4.
struct WideNodeDev {
  float px, py, pz;
  uint32_t exyz_imask;        // ex | ey<<8 | ez<<16 | inner-mask<<24
  uint32_t child_base;        // first inner child node index
  uint32_t tri_base;          // first triangle (leaf-ordered) index
  uint32_t meta_lo, meta_hi;  // 8 x meta byte
  uint32_t qlo_x_lo, qlo_x_hi, qlo_y_lo, qlo_y_hi, qlo_z_lo, qlo_z_hi;
  uint32_t qhi_x_lo, qhi_x_hi, qhi_y_lo, qhi_y_hi, qhi_z_lo, qhi_z_hi;
};

struct SceneDev {
  // geometry
  int32_t n_tris;
  const float* tri_pos;       // 9 floats per triangle (v0,v1,v2), global order
  const TriAttr* tri_attr;
  const float* normals;       // 3 per normal
  const float* texcoords;     // 2 per texcoord
  int64_t n_texcoords;        // number of floats in texcoords
  // acceleration structure (binary: 4 x float4 per node; wide: 5 x float4)
  int32_t bvh_kind;           // 0: binary, 1: wide
  const float4* nodes;
  const float4* isect_tris;   // 3 x float4 per leaf-ordered triangle: v0 (w = global id), v0-v1, v2-v0
  int32_t n_nodes;            // nodes of `nodes` (for the bounds-checked build)
  // materials and textures
  const MaterialDev* mats;
  const TextureDev* textures;
  int32_t n_mats, n_textures;
  const float* tex_pool;
  const uint8_t* tex_pool8;
  // lights
  int32_t n_light_tris;
  const int32_t* light_tris;
  const double* light_cdf;    // empty (nullptr) when fewer than 2 lights
  const uint32_t* light_guide;
  uint32_t light_guide_log2;
  float light_pdf_area;       // 1 / total light area (Scene.cpp:512)
  EnvDev env;
  CameraDev cam;
  // settings
  int32_t width, height, max_depth, rr_start;
  float rr_q;
  int32_t two_strategies;     // hasLight() && use_mis (MIS.cpp:60-72)
  int32_t env_is_sampled;     // world has an environment texture
  float p_surface;            // probability of surface-light sampling (Scene.cpp:545)
};

}  // namespace hasty
